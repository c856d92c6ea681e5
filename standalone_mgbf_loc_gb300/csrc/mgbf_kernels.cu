// sm_103a kernels for the HBM-bound stages of the MGBF pipeline:
//   vertical line beta filter (forward / adjoint) on whole-sample mirrored
//   columns, restriction (fold o P^T), prolongation-and-add (P o fill),
//   the direct-sum radial beta filter used when no moment kernel matches,
//   and small helpers (x-halo mirror, copy, halo zeroing, dot product).
//
// Layout: the level index k is fastest (the reference's VALL order), so
// consecutive lanes take consecutive k and every warp access is one
// contiguous 128-byte (FP32) segment.  MPI halo exchange of the reference
// becomes index reflection at the global edges.
#include <cuda.h>

#include "mgbf_common.cuh"
#include "mgbf_kernels.cuh"

#include <algorithm>
#include <cstdint>

namespace mgbf {

// ------------------------------------------------------------- z filter
// out(k) = sum_d band[L][d+mz] * in(c0+L+d) for z columns (k < nzk), where
// band is the FP64-built matrix of sup_vrbeta1_* / sup_vrbeta1T_*
// (mg_filtering.f90:2042-2262) including the whole-sample mirror and, for
// the adjoint, the edge fold; entries k >= nzk (2D variables) are copied.
// One lane per level k (coalesced), ZI consecutive columns i per thread; the
// band row of the lane's level sits in registers (MZ = compile-time half
// width; taps outside the column get weight 0 and a clamped address).
template <typename T, int MZ, int ZI>
__global__ void __launch_bounds__(128) k_zfilter(ZArgs a) {
    using A = typename AccOf<T>::type;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.nk) return;
    const int i0 = blockIdx.y * ZI;
    const int j = blockIdx.z;
    const T* in = static_cast<const T*>(a.in.p) + a.in.sj * j;
    T* out = static_cast<T*>(a.out.p) + a.out.sj * j + k;
    const bool zc = k < a.nzk;
    A w[2 * MZ + 1];
    int off[2 * MZ + 1];
    if (zc) {
        const int L = k % a.lm;
        const int c0 = k - L;
        const A* b = static_cast<const A*>(a.band) + (size_t)L * (2 * a.mz + 1) + a.mz;
#pragma unroll
        for (int d = -MZ; d <= MZ; ++d) {
            const bool ok = d >= -a.mz && d <= a.mz && L + d >= 0 && L + d < a.lm;
            w[d + MZ] = ok ? b[d] : A(0);
            off[d + MZ] = ok ? c0 + L + d : k;
        }
    }
#pragma unroll
    for (int q = 0; q < ZI; ++q) {
        const int i = i0 + q;
        if (i >= a.I) break;
        const T* row = in + a.in.si * i;
        A v;
        if (zc) {
            v = A(0);
#pragma unroll
            for (int d = 0; d < 2 * MZ + 1; ++d) v = fma(w[d], ldv(row + off[d]), v);
        } else {
            v = ldv(row + k);
        }
        stv(out + a.out.si * i, v);
        if (a.mirror_hx) {
            if (i < a.mirror_hx) stv(out + a.out.si * (-1 - i), v);
            if (i >= a.I - a.mirror_hx) stv(out + a.out.si * (2 * a.I - 1 - i), v);
        }
    }
}

// Vectorised z filter: each thread owns levels k..k+3 (k % 4 == 0) and a
// strip of ncol columns, taken ZI at a time; the band rows of its four
// levels sit in registers for the whole strip (levels past nzk get the
// identity row, so 2D variables are copied by the same code); the window
// k-4NB .. k+4NB+3 comes in 2NB+1 vector loads.  Needs nk % 4 == 0 and
// 16-byte aligned views.
template <typename T, int MZ, int ZI>
__global__ void __launch_bounds__(128) k_zfilter4(ZArgs a, int ncol) {
    using A = typename AccOf<T>::type;
    constexpr int NB = (MZ + 3) / 4;
    constexpr int NWIN = 4 * (2 * NB + 1);
    const int k = (blockIdx.x * blockDim.x + threadIdx.x) * 4;
    if (k >= a.nk) return;
    const int i0 = blockIdx.y * ncol;
    const int j = blockIdx.z;
    A w[4][2 * MZ + 1];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int kq = k + q;
        const bool zc = kq < a.nzk;
        const int L = zc ? kq % a.lm : 0;
        const A* b = static_cast<const A*>(a.band) + (size_t)L * (2 * a.mz + 1) + a.mz;
#pragma unroll
        for (int d = -MZ; d <= MZ; ++d) {
            const bool ok = zc && d >= -a.mz && d <= a.mz && L + d >= 0 && L + d < a.lm;
            w[q][d + MZ] = ok ? b[d] : ((!zc && d == 0) ? A(1) : A(0));
        }
    }
    int voff[2 * NB + 1];
#pragma unroll
    for (int v = 0; v < 2 * NB + 1; ++v) voff[v] = min(max(k + 4 * (v - NB), 0), a.nk - 4);
    const T* in = static_cast<const T*>(a.in.p) + a.in.sj * j;
    T* out = static_cast<T*>(a.out.p) + a.out.sj * j + k;
    const int i1 = min(i0 + ncol, a.I);
    for (int ic = i0; ic < i1; ic += ZI)
#pragma unroll
    for (int c = 0; c < ZI; ++c) {
        const int i = ic + c;
        if (i >= i1) break;
        const T* row = in + a.in.si * i;
        A x[NWIN];
#pragma unroll
        for (int v = 0; v < 2 * NB + 1; ++v) {
            A t[4];
            V4<T>::ld(row + voff[v], t);
#pragma unroll
            for (int e = 0; e < 4; ++e) x[4 * v + e] = t[e];
        }
        A y[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            A acc = A(0);
#pragma unroll
            for (int d = -MZ; d <= MZ; ++d) acc = fma(w[q][d + MZ], x[4 * NB + q + d], acc);
            y[q] = acc;
        }
        V4<T>::st(out + a.out.si * i, y);
        if (a.mirror_hx) {
            if (i < a.mirror_hx) V4<T>::st(out + a.out.si * (-1 - i), y);
            if (i >= a.I - a.mirror_hx) V4<T>::st(out + a.out.si * (2 * a.I - 1 - i), y);
        }
    }
}

// --------------------------------------------------------- restriction
// coarse(c,d) = sum_b wy[d][b] sum_a wx[c][a] fine(2c-3+a, 2d-3+b): the
// separable transpose of (P o fill2) (adjoint + bocoT_2d(...,2,2),
// mg_generations.f90:1117-1187, mg_bocos.f90:929-1061) with the mirror
// images already merged into the 8-wide weight rows.  Each thread makes a
// RC x RC block of coarse points from its (2RC+6)^2 fine footprint, loaded
// once: every fine row is first reduced along x, then added into the coarse
// rows it feeds.
constexpr int RC = 4;
template <typename T>
__global__ void __launch_bounds__(128) k_restrict(RestrictArgs a) {
    using A = typename AccOf<T>::type;
    constexpr int NF = 2 * RC + 6;
    const int Ic = a.If / 2, Jc = a.Jf / 2;
    int k = blockIdx.x * 32 + threadIdx.x;
    const bool kv = k < a.nk;
    if (!kv) k = a.nk - 1;
    const int c0 = (blockIdx.y * blockDim.y + threadIdx.y) * RC;
    if (c0 >= Ic) return;
    const int d0 = blockIdx.z * RC;
    A wx[RC][8], wy[RC][8];
#pragma unroll
    for (int c = 0; c < RC; ++c) {
        const int cc = min(c0 + c, Ic - 1);
        const int dd = min(d0 + c, Jc - 1);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            wx[c][q] = static_cast<const A*>(a.wx)[cc * 8 + q];
            wy[c][q] = static_cast<const A*>(a.wy)[dd * 8 + q];
        }
    }
    int fcol[NF];
#pragma unroll
    for (int s = 0; s < NF; ++s) fcol[s] = min(max(2 * c0 - 3 + s, 0), a.If - 1);
    const T* fine = static_cast<const T*>(a.fine.p) + k;
    A acc[RC][RC];
#pragma unroll
    for (int r = 0; r < RC; ++r)
#pragma unroll
        for (int c = 0; c < RC; ++c) acc[r][c] = A(0);
#pragma unroll
    for (int rr = 0; rr < NF; ++rr) {
        const int fj = min(max(2 * d0 - 3 + rr, 0), a.Jf - 1);
        const T* row = fine + a.fine.sj * fj;
        A seg[NF];
#pragma unroll
        for (int s = 0; s < NF; ++s) seg[s] = ldv(row + a.fine.si * fcol[s]);
        A xr[RC];
#pragma unroll
        for (int c = 0; c < RC; ++c) {
            A v = A(0);
#pragma unroll
            for (int q = 0; q < 8; ++q) v = fma(wx[c][q], seg[2 * c + q], v);
            xr[c] = v;
        }
#pragma unroll
        for (int r = 0; r < RC; ++r) {
            const int b = rr - 2 * r;  // fine row 2(d0+r)-3+b
            if (b >= 0 && b < 8) {
#pragma unroll
                for (int c = 0; c < RC; ++c) acc[r][c] = fma(wy[r][b], xr[c], acc[r][c]);
            }
        }
    }
    if (!kv) return;
#pragma unroll
    for (int r = 0; r < RC; ++r) {
        const int d = d0 + r;
        if (d >= Jc) break;
        T* out = static_cast<T*>(a.coarse.p) + a.coarse.sj * d + k;
#pragma unroll
        for (int c = 0; c < RC; ++c) {
            const int cc = c0 + c;
            if (cc >= Ic) break;
            const A v = acc[r][c];
            stv(out + a.coarse.si * cc, v);
            if (cc < a.mirror_hx) stv(out + a.coarse.si * (-1 - cc), v);
            if (cc >= Ic - a.mirror_hx) stv(out + a.coarse.si * (2 * Ic - 1 - cc), v);
        }
    }
}

// Pipelined restriction.  A block takes 128 levels x 4*CX coarse columns x
// a segment of coarse rows and walks down the rows.  Fine rows are staged
// in shared memory by cp.async, S rows in flight (two rows per step), and
// each warp restricts its CX coarse columns from there: lane = 4 levels, the
// x pass (8 taps) once per fine row, then the row goes into a ring of the
// four coarse rows it touches (fine rows 2d+3 and 2d+4 feed coarse rows
// d..d+3 with taps 6-2s and 7-2s), and coarse row d is final once both are
// in.  Every fine value is read from HBM once per block (plus 6 shared
// columns and 6 rows of ring fill), and the x pass is not repeated across
// coarse rows.
constexpr int kRsWarps = 4;
constexpr int kRsLevels = 128;
template <typename T, int CX>
__host__ __device__ constexpr int rs_cols() { return 2 * kRsWarps * CX + 6; }
template <typename T, int CX, int S>
constexpr size_t rs_smem() { return (size_t)S * rs_cols<T, CX>() * kRsLevels * sizeof(T); }

template <typename T, int CX, int S>
__global__ void __launch_bounds__(kRsWarps * 32) k_restrict_p(RestrictArgs a, int seg_rows) {
    using A = typename AccOf<T>::type;
    static_assert(S % 2 == 0 && S >= 4, "stages come in pairs of fine rows");
    constexpr int NF = rs_cols<T, CX>();
    constexpr int EPC = 16 / (int)sizeof(T);          // elements per 16-byte chunk
    constexpr int CH = kRsLevels / EPC;               // chunks per staged column
    constexpr int P2 = S / 2;                         // steps in flight
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T* stg = reinterpret_cast<T*>(smem_raw);          // [S][NF][kRsLevels]
    const unsigned sbase = (unsigned)__cvta_generic_to_shared(smem_raw);
    const int Ic = a.If / 2, Jc = a.Jf / 2;
    const int kb = blockIdx.x * kRsLevels;
    const int chunks = (min(kRsLevels, a.nk - kb)) / EPC;
    const int cs = blockIdx.y * (kRsWarps * CX);
    const int d0 = blockIdx.z * seg_rows;
    const int d1 = min(d0 + seg_rows, Jc);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c0 = cs + warp * CX;
    const T* fine = static_cast<const T*>(a.fine.p) + kb;

    auto issue = [&](int fr, int stage) {
        const int fj = min(max(fr, 0), a.Jf - 1);
        const T* row = fine + a.fine.sj * fj;
        for (int t = threadIdx.x; t < NF * CH; t += kRsWarps * 32) {
            const int col = t / CH, ch = t - col * CH;
            if (ch < chunks) {
                const int fc = min(max(2 * cs - 3 + col, 0), a.If - 1);
                cp_async16(sbase + (unsigned)(((stage * NF + col) * kRsLevels + ch * EPC) * (int)sizeof(T)),
                           row + a.fine.si * fc + ch * EPC, 16);
            }
        }
    };

    const A* wyp = static_cast<const A*>(a.wy);
    A wx[CX][8];
#pragma unroll
    for (int c = 0; c < CX; ++c) {
        const int cc = min(c0 + c, Ic - 1);
#pragma unroll
        for (int q = 0; q < 8; ++q) wx[c][q] = static_cast<const A*>(a.wx)[cc * 8 + q];
    }
    A acc[4][CX][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < CX; ++c)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[r][c][e] = A(0);

    const int niter = d1 - d0 + 3;  // ring base d = d0-3+it
#pragma unroll
    for (int q = 0; q < P2; ++q) {
        if (q < niter) {
            issue(2 * d0 - 3 + 2 * q, 2 * q);
            issue(2 * d0 - 2 + 2 * q, 2 * q + 1);
        }
        cp_async_commit();
    }
    const bool kv = 4 * lane < chunks * EPC;
    for (int it = 0; it < niter; ++it) {
        const int d = d0 - 3 + it;
        const int sp = it % P2;
        cp_async_wait<P2 - 1>();
        __syncthreads();
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const T* srow = stg + (size_t)(2 * sp + h) * NF * kRsLevels + 4 * lane + 2 * warp * CX * kRsLevels;
            A wy[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int dd = min(max(d + r, 0), Jc - 1);
                wy[r] = __ldg(wyp + dd * 8 + 6 + h - 2 * r);
            }
#pragma unroll
            for (int c = 0; c < CX; ++c) {
                A xr[4] = {A(0), A(0), A(0), A(0)};
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    A v[4];
                    V4<T>::ldc(srow + (2 * c + q) * kRsLevels, v);
#pragma unroll
                    for (int e = 0; e < 4; ++e) xr[e] = fma(wx[c][q], v[e], xr[e]);
                }
#pragma unroll
                for (int r = 0; r < 4; ++r)
#pragma unroll
                    for (int e = 0; e < 4; ++e) acc[r][c][e] = fma(wy[r], xr[e], acc[r][c][e]);
            }
        }
        __syncthreads();  // every warp is done with stage pair sp
        if (it + P2 < niter) {
            issue(2 * d0 - 3 + 2 * (it + P2), 2 * sp);
            issue(2 * d0 - 2 + 2 * (it + P2), 2 * sp + 1);
        }
        cp_async_commit();
        if (d >= d0 && kv) {
            T* out = static_cast<T*>(a.coarse.p) + a.coarse.sj * d + kb + 4 * lane;
#pragma unroll
            for (int c = 0; c < CX; ++c) {
                const int cc = c0 + c;
                if (cc < Ic) {
                    V4<T>::st(out + a.coarse.si * cc, acc[0][c]);
                    if (cc < a.mirror_hx) V4<T>::st(out + a.coarse.si * (-1 - cc), acc[0][c]);
                    if (cc >= Ic - a.mirror_hx) V4<T>::st(out + a.coarse.si * (2 * Ic - 1 - cc), acc[0][c]);
                }
            }
        }
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < CX; ++c)
#pragma unroll
                for (int e = 0; e < 4; ++e) acc[r][c][e] = acc[r + 1][c][e];
#pragma unroll
        for (int c = 0; c < CX; ++c)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[3][c][e] = A(0);
    }
    cp_async_wait<0>();
}

// Generation 1's vertical adjoint filter fused into its restriction, fed by
// TMA.  A block takes LV levels (whole z columns: lm divides LV) x 4*CX
// coarse columns x a segment of coarse rows and walks down the rows in pairs
// of fine rows.  One elected thread loads each fine row with
// cp.async.bulk.tensor (box: LV + 2*PAD levels x NF columns x 1 row of the
// caller's field; levels, columns and rows outside the field arrive as zeros,
// and the restriction gives them zero weight) into a ring of kZrPairs pairs,
// one mbarrier per pair.  Phase `it` z-filters pair it+1 in place and
// restricts pair it, then one block barrier frees pair it's slot for the
// load of pair it+kZrPairs.  The z filter (Bz^T: the band matrix with the
// whole-sample mirror and fold of sup_vrbeta1T, mg_filtering.f90:2094-2262)
// runs per staged column: lane = 4 levels, a window of 12 levels (vertical
// reach MZ = 4) or 20 (MZ = 8) from the padded column (the band gives levels
// outside the lane's z column zero weight), band rows in registers; the columns the block owns go to generation 1
// (zout, with the mirrored x halo).  The restriction is k_restrict_p's: the
// x pass once per fine row, then the ring of the four coarse rows it feeds.
// x is read from HBM once.
constexpr int kZrPairs = 3;
// Levels staged below and above each column: the z window of a lane reaches
// 4*ceil(MZ/4) levels past its own four, and a TMA row starts on 16 bytes.
template <typename T, int MZ>
__host__ __device__ constexpr int zr_pad() {
    return 4 * ((MZ + 3) / 4) > 16 / (int)sizeof(T) ? 4 * ((MZ + 3) / 4) : 16 / (int)sizeof(T);
}
template <typename T, int CX, int LV, int MZ>
__host__ __device__ constexpr size_t zr_row_bytes() {
    return ((size_t)rs_cols<T, CX>() * (LV + 2 * zr_pad<T, MZ>()) * sizeof(T) + 127) / 128 * 128;
}
template <typename T, int CX, int LV, int MZ>
constexpr size_t zr_smem() { return 2 * kZrPairs * zr_row_bytes<T, CX, LV, MZ>(); }

// RONLY: restriction only (no z columns, generation 1 not written); the
// two-pass chain's form compiles without that branch
template <typename T, int CX, int LV, int MZ, bool RONLY = false>
__global__ void __launch_bounds__(kRsWarps * 32, 3)
    k_zrestrict_tma(ZRestrictArgs z, const __grid_constant__ CUtensorMap xmap, int seg_rows) {
    static_assert(sizeof(T) <= 4, "FP32 accumulation: float or bfloat16 storage");
    static_assert(MZ <= 8 && LV % 4 == 0 && LV + 2 * zr_pad<T, MZ>() <= 256, "z window, 4 levels per lane, TMA box");
    constexpr int PAD = zr_pad<T, MZ>();
    constexpr int NB = (MZ + 3) / 4;                  // window: NB vectors of 4 levels on each side
    constexpr int COL = LV + 2 * PAD;                 // staged levels per column
    constexpr int NF = rs_cols<T, CX>();              // staged fine columns: 2*4*CX owned + 6 shared
    constexpr unsigned ROWB = (unsigned)zr_row_bytes<T, CX, LV, MZ>();
    constexpr unsigned BOXB = (unsigned)(NF * COL * sizeof(T));
    const RestrictArgs& a = z.r;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) unsigned long long bars[kZrPairs];
    const unsigned sbase = (unsigned)__cvta_generic_to_shared(smem_raw);
    const unsigned bbase = (unsigned)__cvta_generic_to_shared(bars);
    const int Ic = a.If / 2, Jc = a.Jf / 2;
    const int kb = blockIdx.x * LV;
    const int cs = blockIdx.y * (kRsWarps * CX);
    const int d0 = blockIdx.z * seg_rows;
    const int d1 = min(d0 + seg_rows, Jc);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int c0 = cs + warp * CX;
    const int niter = d1 - d0 + 3;  // coarse rows d0-3 .. d1-1; pair it = fine rows 2d0-3+2it, 2d0-2+2it
    if (tid == 0) {
#pragma unroll
        for (int s = 0; s < kZrPairs; ++s) mbar_init(bbase + 8 * s, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    auto issue = [&](int it) {  // thread 0: pair it into slot it % kZrPairs
        const int sl = it % kZrPairs;
        const int fr = 2 * d0 - 3 + 2 * it;
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        mbar_expect_tx(bbase + 8 * sl, 2 * BOXB);
        tma_load_3d(sbase + 2 * sl * ROWB, &xmap, kb - PAD, 2 * cs - 3, fr, bbase + 8 * sl);
        tma_load_3d(sbase + (2 * sl + 1) * ROWB, &xmap, kb - PAD, 2 * cs - 3, fr + 1, bbase + 8 * sl);
    };
    if (tid == 0)
        for (int it = 0; it < kZrPairs && it < niter; ++it) issue(it);

    // lanes past LV (LV = 96) take no part: their window would reach into
    // the next staged column
    constexpr unsigned kLanes = LV / 4 >= 32 ? 0xffffffffu : (1u << (LV / 4)) - 1u;
    const bool lin = lane < LV / 4;
    // band rows of this lane's four levels (identity past the z columns)
    const bool lv = lin && kb + 4 * lane < a.nk;  // nk % 4 == 0: all four levels exist
    float wz[4][2 * MZ + 1];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int kq = kb + 4 * lane + q;
        const bool zc = lv && kq < z.nzk;
        const int L = zc ? kq % z.lm : 0;
        const float* b = static_cast<const float*>(z.band) + (size_t)L * (2 * z.mz + 1) + z.mz;
#pragma unroll
        for (int d = -MZ; d <= MZ; ++d) {
            const bool ok = zc && d >= -z.mz && d <= z.mz && L + d >= 0 && L + d < z.lm;
            wz[q][d + MZ] = ok ? b[d] : ((!zc && d == 0) ? 1.f : 0.f);
        }
    }
    const float* wyp = static_cast<const float*>(a.wy);
    float wx[CX][8];
#pragma unroll
    for (int c = 0; c < CX; ++c) {
        const int cc = min(c0 + c, Ic - 1);
#pragma unroll
        for (int q = 0; q < 8; ++q) wx[c][q] = static_cast<const float*>(a.wx)[cc * 8 + q];
    }
    float acc[4][CX][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < CX; ++c)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[r][c][e] = 0.f;

    T* const stg = reinterpret_cast<T*>(smem_raw);
    // Bz^T in place on staged row sr (fine row fr); owned columns to zout
    auto zfilter_row = [&](int sr, int fr) {
        T* srow = stg + (size_t)sr * (ROWB / sizeof(T)) + PAD + 4 * lane;
        const bool own_row = lv && fr >= 2 * d0 && fr < 2 * d1;
        T* zrow = static_cast<T*>(z.zout.p) + z.zout.sj * (long long)fr + kb + 4 * lane;
#pragma unroll
        for (int t = 0; t < (NF + kRsWarps - 1) / kRsWarps; ++t) {
            const int col = warp + kRsWarps * t;
            if (col < NF && lin) {  // col is warp-uniform
                T* cp = srow + col * COL;
                float x[2 * NB + 1][4];  // levels 4*lane-4*NB .. 4*lane+3+4*NB
#pragma unroll
                for (int v = 0; v <= 2 * NB; ++v) V4<T>::ldc(cp + 4 * (v - NB), x[v]);
                __syncwarp(kLanes);  // every lane has its window before any lane overwrites
                float y[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    float s2 = 0.f;
#pragma unroll
                    for (int dd = -MZ; dd <= MZ; ++dd)
                        s2 = fmaf(wz[q][dd + MZ], x[(4 * NB + q + dd) / 4][(4 * NB + q + dd) % 4], s2);
                    y[q] = s2;
                }
                V4<T>::st(cp, y);
                const int gc = 2 * cs - 3 + col;
                if (own_row && col >= 3 && col < 3 + 2 * kRsWarps * CX && gc < a.If) {
                    V4<T>::st(zrow + z.zout.si * gc, y);
                    if (gc < z.mirror_z) V4<T>::st(zrow + z.zout.si * (-1 - gc), y);
                    if (gc >= a.If - z.mirror_z) V4<T>::st(zrow + z.zout.si * (2 * a.If - 1 - gc), y);
                }
            }
        }
    };
    // R on the filtered pair in slot sl: its rows feed coarse rows d..d+3
    auto restrict_pair = [&](int sl, int d) {
        if (!lin) return;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const T* srow = stg + (size_t)(2 * sl + h) * (ROWB / sizeof(T)) + PAD + 4 * lane + 2 * warp * CX * COL;
            float wy[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int dd = min(max(d + r, 0), Jc - 1);
                wy[r] = __ldg(wyp + dd * 8 + 6 + h - 2 * r);
            }
            // x pass: the warp's 2*CX+6 staged columns are each read once
            // and feed every coarse column whose 8 taps cover them
            float xr[CX][4];
#pragma unroll
            for (int c = 0; c < CX; ++c)
#pragma unroll
                for (int e = 0; e < 4; ++e) xr[c][e] = 0.f;
#pragma unroll
            for (int j = 0; j < 2 * CX + 6; ++j) {
                float v[4];
                V4<T>::ldc(srow + j * COL, v);
#pragma unroll
                for (int c = 0; c < CX; ++c) {
                    const int q = j - 2 * c;
                    if (q >= 0 && q < 8) {
#pragma unroll
                        for (int e = 0; e < 4; ++e) xr[c][e] = fmaf(wx[c][q], v[e], xr[c][e]);
                    }
                }
            }
#pragma unroll
            for (int c = 0; c < CX; ++c)
#pragma unroll
                for (int r = 0; r < 4; ++r)
#pragma unroll
                    for (int e = 0; e < 4; ++e) acc[r][c][e] = fmaf(wy[r], xr[c][e], acc[r][c][e]);
        }
    };

    // pipeline fill: pair 0 filtered before the first restriction
    // (restriction only skips the z pass, which would copy the staged rows
    // onto themselves)
    constexpr bool zpass = !RONLY;
    int waited = 0;                          // pairs whose barrier every thread has passed
    int issued = min(niter, kZrPairs);       // pairs whose loads thread 0 has issued
    bool ok = __all_sync(0xffffffffu, mbar_wait_bounded(bbase, 0u, z.max_polls));
    if (ok && zpass) {
        zfilter_row(0, 2 * d0 - 3);
        zfilter_row(1, 2 * d0 - 2);
    }
    bool failed = __syncthreads_or(!ok);
    if (!failed) waited = 1;
    for (int it = 0; it < niter && !failed; ++it) {
        const int d = d0 - 3 + it;
        if (it + 1 < niter) {
            const int sl1 = (it + 1) % kZrPairs;
            ok = __all_sync(0xffffffffu, mbar_wait_bounded(bbase + 8 * sl1, (unsigned)(((it + 1) / kZrPairs) & 1), z.max_polls));
            if (ok && zpass) {
                zfilter_row(2 * sl1, 2 * d0 - 1 + 2 * it);
                zfilter_row(2 * sl1 + 1, 2 * d0 + 2 * it);
            }
        }
        restrict_pair(it % kZrPairs, d);
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        waited = min(niter, it + 2);
        if (tid == 0 && it + kZrPairs < niter) issue(it + kZrPairs);  // into the slot pair it has left
        issued = min(niter, it + 1 + kZrPairs);
        if (d >= d0 && lv) {
            T* out = static_cast<T*>(a.coarse.p) + a.coarse.sj * d + kb + 4 * lane;
#pragma unroll
            for (int c = 0; c < CX; ++c) {
                const int cc = c0 + c;
                if (cc < Ic) {
                    V4<T>::st(out + a.coarse.si * cc, acc[0][c]);
                    if (cc < a.mirror_hx) V4<T>::st(out + a.coarse.si * (-1 - cc), acc[0][c]);
                    if (cc >= Ic - a.mirror_hx) V4<T>::st(out + a.coarse.si * (2 * Ic - 1 - cc), acc[0][c]);
                }
            }
        }
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < CX; ++c)
#pragma unroll
                for (int e = 0; e < 4; ++e) acc[r][c][e] = acc[r + 1][c][e];
#pragma unroll
        for (int c = 0; c < CX; ++c)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[3][c][e] = 0.f;
    }
    if (failed) {
        // record, then drain this block's outstanding copies (bounded) before exit
        if (tid == 0) {
            atomicExch(z.status, 1);
            for (int p = waited; p < issued; ++p)
                mbar_wait_bounded(bbase + 8 * (p % kZrPairs), (unsigned)((p / kZrPairs) & 1), kDefaultWaitPolls);
        }
        __syncthreads();
    }
}

// -------------------------------------------------------- prolongation
// out(i,j) = base(i,j) + (P o fill2) coarse: downsend + boco_2d(...,2,2) +
// direct1 + add (mg_generations.f90:210-267, 1190-1250), or the quadratic
// direct2 with fill1 (1319-1374).  Fine points come in pairs that read the
// same NT coarse cells: with the 4-point offset stencil fine columns
// (2m-1, 2m) (0-based) use coarse m-2..m+1 with weights p and q
// (def_offset_coef, mg_interpolate.f90:76-79); with the quadratic stencil
// (2m, 2m+1) use m-1..m+1 with a and b.  Coarse indices are mirrored
// (half-sample) at the edges; the weights stay those of the fine parity, as
// in direct1 after boco_2d.  Each thread makes PX column pairs x one row
// pair; x pass inside, y pass outside, as direct1 orders them.
template <int NT> struct PCoef;
template <> struct PCoef<4> {
    static __device__ __forceinline__ double c0(int t) {  // p_coef
        return t == 0 ? -9.0 / 128.0 : t == 1 ? 111.0 / 128.0 : t == 2 ? 29.0 / 128.0 : -3.0 / 128.0;
    }
    static __device__ __forceinline__ double c1(int t) {  // q_coef
        return t == 0 ? -3.0 / 128.0 : t == 1 ? 29.0 / 128.0 : t == 2 ? 111.0 / 128.0 : -9.0 / 128.0;
    }
};
template <> struct PCoef<3> {
    static __device__ __forceinline__ double c0(int t) {  // a_coef
        return t == 0 ? 5.0 / 32.0 : t == 1 ? 30.0 / 32.0 : -3.0 / 32.0;
    }
    static __device__ __forceinline__ double c1(int t) {  // b_coef
        return t == 0 ? -3.0 / 32.0 : t == 1 ? 30.0 / 32.0 : 5.0 / 32.0;
    }
};

constexpr int PX = 4;
template <typename T, int NT>
__global__ void __launch_bounds__(128) k_prolong(ProlongArgs a) {
    using A = typename AccOf<T>::type;
    constexpr int O = NT == 4 ? 1 : 0;       // fine column of pair m is 2m - O
    constexpr int S = NT == 4 ? 2 : 1;       // first coarse tap of pair m is m - S
    constexpr int NC = PX + NT - 1;          // coarse columns per thread
    const int Ic = a.If / 2, Jc = a.Jf / 2;
    const int npx = Ic + O, npy = Jc + O;    // pairs per direction
    int k = blockIdx.x * 32 + threadIdx.x;
    const bool kv = k < a.nk;
    if (!kv) k = a.nk - 1;
    const int m0 = (blockIdx.y * blockDim.y + threadIdx.y) * PX;
    if (m0 >= npx) return;
    const int n = blockIdx.z;  // row pair
    int ccol[NC];
#pragma unroll
    for (int s = 0; s < NC; ++s) ccol[s] = reflect_half(m0 - S + s, Ic);
    const T* coarse = static_cast<const T*>(a.coarse.p) + k;
    A r0[2 * PX], r1[2 * PX];  // fine rows 2n-O and 2n+1-O
#pragma unroll
    for (int q = 0; q < 2 * PX; ++q) r0[q] = r1[q] = A(0);
#pragma unroll
    for (int t = 0; t < NT; ++t) {
        const int cr = reflect_half(n - S + t, Jc);
        const T* row = coarse + a.coarse.sj * cr;
        A v[NC];
#pragma unroll
        for (int s = 0; s < NC; ++s) v[s] = ldv(row + a.coarse.si * ccol[s]);
        const A wy0 = (A)PCoef<NT>::c0(t), wy1 = (A)PCoef<NT>::c1(t);
#pragma unroll
        for (int q = 0; q < PX; ++q) {
            A x0 = A(0), x1 = A(0);
#pragma unroll
            for (int u = 0; u < NT; ++u) {
                x0 = fma((A)PCoef<NT>::c0(u), v[q + u], x0);
                x1 = fma((A)PCoef<NT>::c1(u), v[q + u], x1);
            }
            r0[2 * q] = fma(wy0, x0, r0[2 * q]);
            r0[2 * q + 1] = fma(wy0, x1, r0[2 * q + 1]);
            r1[2 * q] = fma(wy1, x0, r1[2 * q]);
            r1[2 * q + 1] = fma(wy1, x1, r1[2 * q + 1]);
        }
    }
    if (!kv) return;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int fj = 2 * n - O + h;
        if (fj < 0 || fj >= a.Jf) continue;
        const T* base = static_cast<const T*>(a.base.p) + a.base.sj * fj + k;
        T* out = static_cast<T*>(a.out.p) + a.out.sj * fj + k;
#pragma unroll
        for (int q = 0; q < 2 * PX; ++q) {
            const int fi = 2 * m0 - O + q;
            if (fi < 0 || fi >= a.If) continue;
            A v = h ? r1[q] : r0[q];
            if (a.has_base) v = ldc(base + a.base.si * fi) + v;
            stv(out + a.out.si * fi, v);
        }
    }
}

// Vectorised prolongation: levels k..k+3 per thread, PV column pairs x one
// row pair; the base values are fetched first so their latency overlaps
// the coarse loads.
constexpr int PV = 2;
template <typename T, int NT>
__global__ void __launch_bounds__(128) k_prolong4(ProlongArgs a) {
    using A = typename AccOf<T>::type;
    constexpr int O = NT == 4 ? 1 : 0;
    constexpr int S = NT == 4 ? 2 : 1;
    constexpr int NC = PV + NT - 1;
    const int Ic = a.If / 2, Jc = a.Jf / 2;
    const int k = (blockIdx.x * blockDim.x + threadIdx.x) * 4;
    if (k >= a.nk) return;
    const int m0 = blockIdx.y * PV;
    const int n = blockIdx.z;
    A b0[2 * PV][4], b1[2 * PV][4];
    if (a.has_base) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int fj = min(max(2 * n - O + h, 0), a.Jf - 1);
            const T* base = static_cast<const T*>(a.base.p) + a.base.sj * fj + k;
#pragma unroll
            for (int q = 0; q < 2 * PV; ++q) {
                const int fi = min(max(2 * m0 - O + q, 0), a.If - 1);
                if (h) V4<T>::ldc(base + a.base.si * fi, b1[q]);
                else V4<T>::ldc(base + a.base.si * fi, b0[q]);
            }
        }
    } else {
#pragma unroll
        for (int q = 0; q < 2 * PV; ++q)
#pragma unroll
            for (int e = 0; e < 4; ++e) b0[q][e] = b1[q][e] = A(0);
    }
    int ccol[NC];
#pragma unroll
    for (int s = 0; s < NC; ++s) ccol[s] = reflect_half(m0 - S + s, Ic);
    const T* coarse = static_cast<const T*>(a.coarse.p) + k;
#pragma unroll
    for (int t = 0; t < NT; ++t) {
        const int cr = reflect_half(n - S + t, Jc);
        const T* row = coarse + a.coarse.sj * cr;
        A v[NC][4];
#pragma unroll
        for (int s = 0; s < NC; ++s) V4<T>::ld(row + a.coarse.si * ccol[s], v[s]);
        const A wy0 = (A)PCoef<NT>::c0(t), wy1 = (A)PCoef<NT>::c1(t);
#pragma unroll
        for (int q = 0; q < PV; ++q) {
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                A x0 = A(0), x1 = A(0);
#pragma unroll
                for (int u = 0; u < NT; ++u) {
                    x0 = fma((A)PCoef<NT>::c0(u), v[q + u][e], x0);
                    x1 = fma((A)PCoef<NT>::c1(u), v[q + u][e], x1);
                }
                b0[2 * q][e] = fma(wy0, x0, b0[2 * q][e]);
                b0[2 * q + 1][e] = fma(wy0, x1, b0[2 * q + 1][e]);
                b1[2 * q][e] = fma(wy1, x0, b1[2 * q][e]);
                b1[2 * q + 1][e] = fma(wy1, x1, b1[2 * q + 1][e]);
            }
        }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int fj = 2 * n - O + h;
        if (fj < 0 || fj >= a.Jf) continue;
        T* out = static_cast<T*>(a.out.p) + a.out.sj * fj + k;
#pragma unroll
        for (int q = 0; q < 2 * PV; ++q) {
            const int fi = 2 * m0 - O + q;
            if (fi < 0 || fi >= a.If) continue;
            V4<T>::st(out + a.out.si * fi, h ? b1[q] : b0[q]);
        }
    }
}

// Fused prolongation + vertical forward filter.  A block owns KT = c*lm
// consecutive levels (whole z columns, one lane per level) and a 2 x 2PZ
// block of fine points (PZ column pairs x one row pair): each lane first
// forms base + P(coarse) for its level at the 4PZ points into shared memory,
// then applies its band row across the column from shared memory and
// writes y.  Generation 1 is thereby never written back before the z filter.
constexpr int PZ = 2;
template <typename T, int NT, int MZ>
__global__ void __launch_bounds__(256) k_prolong_z(ProlongZArgs z) {
    using A = typename AccOf<T>::type;
    constexpr int O = NT == 4 ? 1 : 0;
    constexpr int S = NT == 4 ? 2 : 1;
    constexpr int NC = PZ + NT - 1;
    constexpr int NP = 4 * PZ;  // fine points per lane: rows h = 0,1 x columns q = 0..2PZ-1
    extern __shared__ unsigned char smem_raw[];
    A* buf = reinterpret_cast<A*>(smem_raw);  // [NP][KT]
    const ProlongArgs& a = z.p;
    const int KT = blockDim.x;
    const int tid = threadIdx.x;
    const int k = blockIdx.x * KT + tid;
    const bool kv = k < a.nk;
    const int kk = kv ? k : a.nk - 1;
    const int Ic = a.If / 2, Jc = a.Jf / 2;
    const int m0 = blockIdx.y * PZ;
    const int n = blockIdx.z;
    // prolongation (x pass inside, y pass outside, as direct1)
    int ccol[NC];
#pragma unroll
    for (int s2 = 0; s2 < NC; ++s2) ccol[s2] = reflect_half(m0 - S + s2, Ic);
    const T* coarse = static_cast<const T*>(a.coarse.p) + kk;
    A r0[2 * PZ], r1[2 * PZ];
#pragma unroll
    for (int q = 0; q < 2 * PZ; ++q) r0[q] = r1[q] = A(0);
#pragma unroll
    for (int t = 0; t < NT; ++t) {
        const T* row = coarse + a.coarse.sj * reflect_half(n - S + t, Jc);
        A v[NC];
#pragma unroll
        for (int s2 = 0; s2 < NC; ++s2) v[s2] = ldv(row + a.coarse.si * ccol[s2]);
        const A wy0 = (A)PCoef<NT>::c0(t), wy1 = (A)PCoef<NT>::c1(t);
#pragma unroll
        for (int q = 0; q < PZ; ++q) {
            A x0 = A(0), x1 = A(0);
#pragma unroll
            for (int u = 0; u < NT; ++u) {
                x0 = fma((A)PCoef<NT>::c0(u), v[q + u], x0);
                x1 = fma((A)PCoef<NT>::c1(u), v[q + u], x1);
            }
            r0[2 * q] = fma(wy0, x0, r0[2 * q]);
            r0[2 * q + 1] = fma(wy0, x1, r0[2 * q + 1]);
            r1[2 * q] = fma(wy1, x0, r1[2 * q]);
            r1[2 * q + 1] = fma(wy1, x1, r1[2 * q + 1]);
        }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int fj = min(max(2 * n - O + h, 0), a.Jf - 1);
        const T* base = static_cast<const T*>(a.base.p) + a.base.sj * fj + kk;
#pragma unroll
        for (int q = 0; q < 2 * PZ; ++q) {
            const int fi = min(max(2 * m0 - O + q, 0), a.If - 1);
            const A v = ldc(base + a.base.si * fi) + (h ? r1[q] : r0[q]);
            buf[(h * 2 * PZ + q) * KT + tid] = v;
        }
    }
    __syncthreads();
    if (!kv) return;
    // vertical forward filter from shared memory
    const bool zc = k < z.nzk;
    A w[2 * MZ + 1];
    int off[2 * MZ + 1];
    {
        const int L = zc ? k % z.lm : 0;
        const A* b = static_cast<const A*>(z.band) + (size_t)L * (2 * z.mz + 1) + z.mz;
#pragma unroll
        for (int d = -MZ; d <= MZ; ++d) {
            const bool ok = zc && d >= -z.mz && d <= z.mz && L + d >= 0 && L + d < z.lm;
            w[d + MZ] = ok ? b[d] : ((!zc && d == 0) ? A(1) : A(0));
            off[d + MZ] = ok ? tid + d : tid;
        }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int fj = 2 * n - O + h;
        if (fj < 0 || fj >= a.Jf) continue;
        T* out = static_cast<T*>(a.out.p) + a.out.sj * fj + k;
#pragma unroll
        for (int q = 0; q < 2 * PZ; ++q) {
            const int fi = 2 * m0 - O + q;
            if (fi < 0 || fi >= a.If) continue;
            const A* col = buf + (h * 2 * PZ + q) * KT;
            A acc = A(0);
#pragma unroll
            for (int d = 0; d < 2 * MZ + 1; ++d) acc = fma(w[d], col[off[d]], acc);
            stv(out + a.out.si * fi, acc);
        }
    }
}

// Last prolongation fused with the forward vertical filter, fed by TMA:
// y = Bz (base + P coarse) for generation 1 (downsending + direct1/direct2
// then sup_vrbeta1_ens, mg_generations.f90:1190-1374, mg_filtering.f90:2042-2092).
// A block takes LV levels (whole z columns: lm divides LV) x 4*PW column
// pairs x a run of row pairs and walks down the coarse rows.  One elected
// thread loads each coarse row (box: LV levels x 4*PW+NT-1 coarse columns x
// 1 row, the row index mirrored half-sample) into a ring of kPzStages
// stages, one mbarrier each.  Each warp owns PW column pairs: it
// x-interpolates every coarse row once as it arrives (the NT taps of each
// pair, column indices mirrored at the grid's edges within the staged
// window) into a register ring of the NT rows a row pair reads, combines
// them along y on top of the base values of its 2 x 2*PW fine points, stores
// those columns into its own padded staging columns in shared memory and
// applies the band rows of its lane's four levels (a window of 12 levels for
// vertical reach MZ = 4, 20 for MZ = 8) before writing y.  One block barrier per row pair frees the coarse row's stage.
constexpr int kPzStages = 6;
constexpr int kPzPairsPerWarp = 2;
// staged levels below and above each fine column (zero): the reach of a
// lane's z window, 4*ceil(MZ/4) levels past its own four
template <int MZ>
__host__ __device__ constexpr int pz_pad() { return 4 * ((MZ + 3) / 4); }
template <typename T, int NT>
__host__ __device__ constexpr int pz_cols() { return 4 * kPzPairsPerWarp + NT - 1; }  // staged coarse columns
template <typename T, int NT, int LV>
__host__ __device__ constexpr size_t pz_stage_bytes() { return ((size_t)pz_cols<T, NT>() * LV * sizeof(T) + 127) / 128 * 128; }
template <int LV, int MZ>
__host__ __device__ constexpr size_t pz_zst_bytes() {  // z staging: per warp 2 rows x 2*PW columns of LV + 2*pad floats
    return (size_t)4 * 4 * kPzPairsPerWarp * (LV + 2 * pz_pad<MZ>()) * sizeof(float);
}
template <typename T, int NT, int LV, int MZ>
constexpr size_t pz_smem() {
    // coarse ring + z staging + the base values of the next row pair (per
    // warp 2 rows x 2*PW columns of LV levels, in storage type)
    return kPzStages * pz_stage_bytes<T, NT, LV>() + pz_zst_bytes<LV, MZ>() +
           (size_t)4 * 4 * kPzPairsPerWarp * LV * sizeof(T);
}

template <typename T, int NT, int LV, int MZ>
__global__ void __launch_bounds__(128, MZ <= 4 ? 3 : 2)
    k_prolong_z_tma(ProlongZArgs z, const __grid_constant__ CUtensorMap cmap, int seg_steps) {
    static_assert(sizeof(T) <= 4 && MZ <= 8 && LV % 4 == 0 && LV <= 128, "FP32 arithmetic, z window, 4 levels per lane");
    constexpr int PAD = pz_pad<MZ>();
    constexpr int NB = PAD / 4;              // window: NB vectors of 4 levels on each side
    constexpr int O = NT == 4 ? 1 : 0;       // fine column of pair m is 2m - O
    constexpr int S = NT == 4 ? 2 : 1;       // first coarse tap of pair m is m - S
    constexpr int PW = kPzPairsPerWarp;
    constexpr int FC = 2 * PW;               // fine columns per warp
    constexpr int CW = pz_cols<T, NT>();
    constexpr unsigned STB = (unsigned)pz_stage_bytes<T, NT, LV>();
    constexpr unsigned BOXB = (unsigned)(CW * LV * sizeof(T));
    constexpr int ZC = LV + 2 * PAD;         // staged levels per fine column
    constexpr unsigned kLanes = LV / 4 >= 32 ? 0xffffffffu : (1u << (LV / 4)) - 1u;
    const ProlongArgs& a = z.p;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) unsigned long long bars[kPzStages];
    const unsigned sbase = (unsigned)__cvta_generic_to_shared(smem_raw);
    const unsigned bbase = (unsigned)__cvta_generic_to_shared(bars);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int Ic = a.If / 2, Jc = a.Jf / 2;
    const int npy = Jc + O;
    const int kb = blockIdx.x * LV;
    const int m0 = blockIdx.y * (4 * PW);     // first column pair of the block
    const int n0 = blockIdx.z * seg_steps;
    const int n1 = min(n0 + seg_steps, npy);
    const int nsteps = n1 - n0;
    const int nq = nsteps + NT - 1;           // coarse rows n0-S .. n1-1-S+NT-1
    if (tid == 0) {
#pragma unroll
        for (int st = 0; st < kPzStages; ++st) mbar_init(bbase + 8 * st, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    const bool lin = lane < LV / 4;
    const bool lv = lin && kb + 4 * lane < a.nk;
    // this warp's staging columns, zero pads
    float* zst = reinterpret_cast<float*>(smem_raw + kPzStages * STB) + (size_t)warp * 2 * FC * ZC;
    // this warp's base values of the next row pair ([h][f][LV]), fetched by
    // cp.async one row pair ahead; each lane reads back only what it copied
    const unsigned bst = sbase + kPzStages * STB + (unsigned)pz_zst_bytes<LV, MZ>() +
                         (unsigned)((warp * 2 * FC * LV + 4 * lane) * sizeof(T));
    for (int i = lane; i < 2 * FC * 2 * PAD; i += 32) {
        const int col = i / (2 * PAD), e = i % (2 * PAD);
        zst[col * ZC + (e < PAD ? e : LV + e)] = 0.f;
    }
    __syncthreads();
    auto issue = [&](int q) {  // thread 0: coarse row n0-S+q into stage q % kPzStages
        const int st = q % kPzStages;
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        mbar_expect_tx(bbase + 8 * st, BOXB);
        tma_load_3d(sbase + st * STB, &cmap, kb, m0 - S, reflect_half(n0 - S + q, Jc), bbase + 8 * st);
    };
    if (tid == 0)
        for (int q = 0; q < kPzStages && q < nq; ++q) issue(q);

    // staged-window column of tap u of this warp's pair p (mirrored at the
    // edges).  Pairs past the last one (npx - 1) write nothing; they read the
    // last pair's taps, which lie inside the window like every real pair's.
    const int npx = Ic + O;
    int tcol[PW][NT];
#pragma unroll
    for (int p = 0; p < PW; ++p)
#pragma unroll
        for (int u = 0; u < NT; ++u)
            tcol[p][u] = reflect_half(min(m0 + PW * warp + p, npx - 1) - S + u, Ic) - (m0 - S);
    // band rows of this lane's four levels (identity past the z columns)
    float wz[4][2 * MZ + 1];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int kq = kb + 4 * lane + q;
        const bool zc = lv && kq < z.nzk;
        const int L = zc ? kq % z.lm : 0;
        const float* b = static_cast<const float*>(z.band) + (size_t)L * (2 * z.mz + 1) + z.mz;
#pragma unroll
        for (int d = -MZ; d <= MZ; ++d) {
            const bool ok = zc && d >= -z.mz && d <= z.mz && L + d >= 0 && L + d < z.lm;
            wz[q][d + MZ] = ok ? b[d] : ((!zc && d == 0) ? 1.f : 0.f);
        }
    }
    const T* const ring = reinterpret_cast<const T*>(smem_raw) + 4 * lane;
    float xr[NT][FC][4];  // x-interpolated coarse rows, oldest first
#pragma unroll
    for (int t = 0; t < NT; ++t)
#pragma unroll
        for (int f = 0; f < FC; ++f)
#pragma unroll
            for (int e = 0; e < 4; ++e) xr[t][f][e] = 0.f;
    int waited = 0, issued = min(nq, kPzStages);
    bool failed = false;
    // x pass of coarse row q into xr[NT-1]; false if its wait ran out
    auto xpass = [&](int q) -> bool {
        const int st = q % kPzStages;
        const bool ok = mbar_wait_bounded(bbase + 8 * st, (unsigned)((q / kPzStages) & 1), z.max_polls);
        if (ok && lin) {
            const T* row = ring + (size_t)st * (STB / sizeof(T));
#pragma unroll
            for (int f = 0; f < FC; ++f)
#pragma unroll
                for (int e = 0; e < 4; ++e) xr[NT - 1][f][e] = 0.f;
#pragma unroll
            for (int p = 0; p < PW; ++p)
#pragma unroll
                for (int u = 0; u < NT; ++u) {
                    float v[4];
                    V4<T>::ldc(row + tcol[p][u] * LV, v);
                    const float c0 = (float)PCoef<NT>::c0(u), c1 = (float)PCoef<NT>::c1(u);
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        xr[NT - 1][2 * p][e] = fmaf(c0, v[e], xr[NT - 1][2 * p][e]);
                        xr[NT - 1][2 * p + 1][e] = fmaf(c1, v[e], xr[NT - 1][2 * p + 1][e]);
                    }
                }
        }
        // every warp is done with the stage: load the row kPzStages ahead into it
        if (__syncthreads_or(!ok)) return false;
        waited = q + 1;
        if (tid == 0 && q + kPzStages < nq) issue(q + kPzStages);
        issued = min(nq, q + 1 + kPzStages);
        return true;
    };
    // ring fill: coarse rows 0 .. NT-2
    for (int q = 0; q < NT - 1 && !failed; ++q) {
#pragma unroll
        for (int t = 0; t < NT - 1; ++t)
#pragma unroll
            for (int f = 0; f < FC; ++f)
#pragma unroll
                for (int e = 0; e < 4; ++e) xr[t][f][e] = xr[t + 1][f][e];
        failed = !xpass(q);
    }
    const T* base = static_cast<const T*>(a.base.p) + kb + 4 * lane;
    T* out = static_cast<T*>(a.out.p) + kb + 4 * lane;
    // base values of row pair s (fine rows 2n-O, 2n-O+1) into this lane's
    // slots of bst; points outside the field (or levels past nk) are zero
    auto prefetch = [&](int s) {
        if (!lin) return;
        const int n = n0 + s;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int fj = 2 * n - O + h;
#pragma unroll
            for (int f = 0; f < FC; ++f) {
                const int fi = 2 * (m0 + PW * warp + f / 2) - O + (f & 1);
                const bool in = lv && fj >= 0 && fj < a.Jf && fi >= 0 && fi < a.If;
                const T* src = in ? base + a.base.sj * (long long)fj + a.base.si * (long long)fi
                                  : static_cast<const T*>(a.base.p);
                const unsigned dst = bst + (unsigned)((h * FC + f) * LV * sizeof(T));
                if constexpr (sizeof(T) == 4) cp_async16(dst, src, in ? 16 : 0);
                else cp_async8(dst, src, in ? 8 : 0);
            }
        }
        cp_async_commit();
    };
    if (nsteps > 0 && !failed) prefetch(0);
    for (int s = 0; s < nsteps && !failed; ++s) {
        const int n = n0 + s;
#pragma unroll
        for (int t = 0; t < NT - 1; ++t)
#pragma unroll
            for (int f = 0; f < FC; ++f)
#pragma unroll
                for (int e = 0; e < 4; ++e) xr[t][f][e] = xr[t + 1][f][e];
        if (!xpass(s + NT - 1)) {
            failed = true;
            break;
        }
        if (!lin) continue;
        // base values of the row pair, fetched one row pair ahead
        float acc[2][FC][4];
        cp_async_wait<0>();
        const T* bsp = reinterpret_cast<const T*>(smem_raw + kPzStages * STB + pz_zst_bytes<LV, MZ>()) +
                       warp * 2 * FC * LV + 4 * lane;
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int f = 0; f < FC; ++f) V4<T>::ldc(bsp + (h * FC + f) * LV, acc[h][f]);
        // y pass on top of the base values
#pragma unroll
        for (int t = 0; t < NT; ++t) {
            const float w0 = (float)PCoef<NT>::c0(t), w1 = (float)PCoef<NT>::c1(t);
#pragma unroll
            for (int f = 0; f < FC; ++f)
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    acc[0][f][e] = fmaf(w0, xr[t][f][e], acc[0][f][e]);
                    acc[1][f][e] = fmaf(w1, xr[t][f][e], acc[1][f][e]);
                }
        }
        // the slots are read (the y pass used every value): fetch the next
        // row pair's base values behind this one's z filter and the next
        // coarse row's x pass
        if (s + 1 < nsteps) prefetch(s + 1);
        // the warp's columns into its staging area, then Bz per column
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int f = 0; f < FC; ++f) V4<float>::st(zst + (h * FC + f) * ZC + PAD + 4 * lane, acc[h][f]);
        __syncwarp(kLanes);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int fj = 2 * n - O + h;
#pragma unroll
            for (int f = 0; f < FC; ++f) {
                const float* cp = zst + (h * FC + f) * ZC + PAD + 4 * lane;
                float x[2 * NB + 1][4];  // levels 4*lane-PAD .. 4*lane+3+PAD
#pragma unroll
                for (int v = 0; v <= 2 * NB; ++v) V4<float>::ldc(cp + 4 * (v - NB), x[v]);
                float y[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    float s2 = 0.f;
#pragma unroll
                    for (int dd = -MZ; dd <= MZ; ++dd)
                        s2 = fmaf(wz[q][dd + MZ], x[(4 * NB + q + dd) / 4][(4 * NB + q + dd) % 4], s2);
                    y[q] = s2;
                }
                const int fi = 2 * (m0 + PW * warp + f / 2) - O + (f & 1);
                if (lv && fj >= 0 && fj < a.Jf && fi >= 0 && fi < a.If)
                    V4<T>::st(out + a.out.sj * (long long)fj + a.out.si * (long long)fi, y);
            }
        }
        __syncwarp(kLanes);  // the staging columns are rewritten by the next row pair
    }
    cp_async_wait<0>();  // a prefetch left behind by a failed wait lands before the block exits
    if (failed) {
        // record, then drain this block's outstanding copies (bounded) before exit
        if (tid == 0) {
            atomicExch(z.status, 1);
            for (int q = waited; q < issued; ++q)
                mbar_wait_bounded(bbase + 8 * (q % kPzStages), (unsigned)((q / kPzStages) & 1), kDefaultWaitPolls);
        }
        __syncthreads();
    }
}

// Vectorised fused prolongation + z forward: each lane owns 4 consecutive
// levels (one 16-byte access), the block a tile of KT = blockDim.x * 4
// levels (whole z columns).  Base values are fetched first, the prolonged
// field goes to shared memory as float4 rows, and each lane then applies the
// band rows of its four levels to a window of three vectors.
template <typename T, int NT, int MZ>
__global__ void __launch_bounds__(128) k_prolong_z4(ProlongZArgs z) {
    using A = typename AccOf<T>::type;
    constexpr int O = NT == 4 ? 1 : 0;
    constexpr int S = NT == 4 ? 2 : 1;
    constexpr int NC = PZ + NT - 1;
    constexpr int NP = 4 * PZ;
    constexpr int NB = (MZ + 3) / 4;
    extern __shared__ unsigned char smem_raw[];
    A* buf = reinterpret_cast<A*>(smem_raw);  // [NP][KT]
    const ProlongArgs& a = z.p;
    const int nv = blockDim.x;                // vectors per tile
    const int KT = nv * 4;
    const int tid = threadIdx.x;
    const int k = blockIdx.x * KT + 4 * tid;
    const bool kv = k < a.nk;
    const int kk = kv ? k : a.nk - 4;
    const int Ic = a.If / 2, Jc = a.Jf / 2;
    const int m0 = blockIdx.y * PZ;
    const int n = blockIdx.z;
    A vals[2][2 * PZ][4];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int fj = min(max(2 * n - O + h, 0), a.Jf - 1);
        const T* base = static_cast<const T*>(a.base.p) + a.base.sj * fj + kk;
#pragma unroll
        for (int q = 0; q < 2 * PZ; ++q) {
            const int fi = min(max(2 * m0 - O + q, 0), a.If - 1);
            V4<T>::ldc(base + a.base.si * fi, vals[h][q]);
        }
    }
    int ccol[NC];
#pragma unroll
    for (int s2 = 0; s2 < NC; ++s2) ccol[s2] = reflect_half(m0 - S + s2, Ic);
    const T* coarse = static_cast<const T*>(a.coarse.p) + kk;
#pragma unroll
    for (int t = 0; t < NT; ++t) {
        const T* row = coarse + a.coarse.sj * reflect_half(n - S + t, Jc);
        A v[NC][4];
#pragma unroll
        for (int s2 = 0; s2 < NC; ++s2) V4<T>::ld(row + a.coarse.si * ccol[s2], v[s2]);
        const A wy0 = (A)PCoef<NT>::c0(t), wy1 = (A)PCoef<NT>::c1(t);
#pragma unroll
        for (int q = 0; q < PZ; ++q)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                A x0 = A(0), x1 = A(0);
#pragma unroll
                for (int u = 0; u < NT; ++u) {
                    x0 = fma((A)PCoef<NT>::c0(u), v[q + u][e], x0);
                    x1 = fma((A)PCoef<NT>::c1(u), v[q + u][e], x1);
                }
                vals[0][2 * q][e] = fma(wy0, x0, vals[0][2 * q][e]);
                vals[0][2 * q + 1][e] = fma(wy0, x1, vals[0][2 * q + 1][e]);
                vals[1][2 * q][e] = fma(wy1, x0, vals[1][2 * q][e]);
                vals[1][2 * q + 1][e] = fma(wy1, x1, vals[1][2 * q + 1][e]);
            }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int q = 0; q < 2 * PZ; ++q)
#pragma unroll
            for (int e = 0; e < 4; ++e) buf[(h * 2 * PZ + q) * KT + 4 * tid + e] = vals[h][q][e];
    __syncthreads();
    if (!kv) return;
    A w[4][2 * MZ + 1];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const int ke = k + e;
        const bool zc = ke < z.nzk;
        const int L = zc ? ke % z.lm : 0;
        const A* b = static_cast<const A*>(z.band) + (size_t)L * (2 * z.mz + 1) + z.mz;
#pragma unroll
        for (int d = -MZ; d <= MZ; ++d) {
            const bool ok = zc && d >= -z.mz && d <= z.mz && L + d >= 0 && L + d < z.lm;
            w[e][d + MZ] = ok ? b[d] : ((!zc && d == 0) ? A(1) : A(0));
        }
    }
    int voff[2 * NB + 1];
#pragma unroll
    for (int v = 0; v < 2 * NB + 1; ++v) voff[v] = 4 * min(max(tid + v - NB, 0), nv - 1);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int fj = 2 * n - O + h;
        if (fj < 0 || fj >= a.Jf) continue;
        T* out = static_cast<T*>(a.out.p) + a.out.sj * fj + k;
#pragma unroll
        for (int q = 0; q < 2 * PZ; ++q) {
            const int fi = 2 * m0 - O + q;
            if (fi < 0 || fi >= a.If) continue;
            const A* col = buf + (h * 2 * PZ + q) * KT;
            A x[4 * (2 * NB + 1)];
#pragma unroll
            for (int v = 0; v < 2 * NB + 1; ++v)
#pragma unroll
                for (int e = 0; e < 4; ++e) x[4 * v + e] = col[voff[v] + e];
            A y[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                A acc = A(0);
#pragma unroll
                for (int d = -MZ; d <= MZ; ++d) acc = fma(w[e][d + MZ], x[4 * NB + e + d], acc);
                y[e] = acc;
            }
            V4<T>::st(out + a.out.si * fi, y);
        }
    }
}

// ------------------------------------------------- fast filters: line beta
// vrbeta1 along one horizontal axis (jp_pbfil.f90:856-885) as the fast
// filters apply it (mg_filtering.f90:825-997, 1316-1506): the mirror fill of
// bocox/bocoy is an index reflection, so the kernel reads the interior only.
// The stencil is symmetric and the mirror half-sample, so the same gather
// also gives the adjoint (rbetaT then bocoTx/bocoTy).  Each thread owns
// levels k..k+3 and TL consecutive outputs of one line; its window of
// TL+2MR inputs sits in registers (MR = compile-time reach bound, taps past
// the runtime reach carry weight 0).
// Flat thread index -> (level group, strip of TL outputs, line), level
// group fastest: warps stay full whatever nk is, and neighbouring warps take
// neighbouring strips (their windows overlap in L1).
template <typename A> __device__ __forceinline__ A line_w(const LineArgs& a, int d);
template <> __device__ __forceinline__ float line_w<float>(const LineArgs& a, int d) { return a.wf[d]; }
template <> __device__ __forceinline__ double line_w<double>(const LineArgs& a, int d) { return a.w[d]; }
template <typename A> __device__ __forceinline__ A line_scale(const LineArgs& a);
template <> __device__ __forceinline__ float line_scale<float>(const LineArgs& a) { return a.scalef; }
template <> __device__ __forceinline__ double line_scale<double>(const LineArgs& a) { return a.scale; }

struct LinePos {
    int q, t0, line;
    bool ok;
};
__device__ __forceinline__ LinePos line_pos(int nq, int n, int m, int TL) {
    const int nstrip = (n + TL - 1) / TL;
    LinePos r;
    if ((unsigned long long)gridDim.x * blockDim.x <= 0xffffffffull) {
        // 32-bit decode (every launch of realistic size): a 64-bit division
        // by a runtime value costs more than a thread's share of the filter
        const unsigned idx = blockIdx.x * blockDim.x + threadIdx.x;
        const unsigned rest = idx / (unsigned)nq;
        r.q = (int)(idx - rest * (unsigned)nq);
        const unsigned ln = rest / (unsigned)nstrip;
        r.t0 = (int)(rest - ln * (unsigned)nstrip) * TL;
        r.line = (int)ln;
    } else {
        const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
        r.q = (int)(idx % nq);
        const long long rest = idx / nq;
        r.t0 = (int)(rest % nstrip) * TL;
        r.line = (int)(rest / nstrip);
    }
    r.ok = r.line < m;
    return r;
}

template <typename T, int MR, int TL>
__global__ void __launch_bounds__(128) k_line_w(LineArgs a) {
    using A = typename AccOf<T>::type;
    const int n = a.dir ? a.J : a.I;
    const LinePos lp = line_pos(a.nk / 4, n, a.dir ? a.I : a.J, TL);
    if (!lp.ok) return;
    const int k = 4 * lp.q;
    const int t0 = lp.t0;
    const int line = lp.line;
    const long long ls_in = a.dir ? a.in.sj : a.in.si, os_in = a.dir ? a.in.si : a.in.sj;
    const long long ls_out = a.dir ? a.out.sj : a.out.si, os_out = a.dir ? a.out.si : a.out.sj;
    const T* in = static_cast<const T*>(a.in.p) + k + os_in * line;
    T* out = static_cast<T*>(a.out.p) + k + os_out * line;
    A w[MR + 1];
#pragma unroll
    for (int d = 0; d <= MR; ++d) w[d] = d <= a.R ? line_w<A>(a, d) : A(0);
    A x[TL + 2 * MR][4];
#pragma unroll
    for (int s2 = 0; s2 < TL + 2 * MR; ++s2) V4<T>::ld(in + ls_in * reflect_half(t0 - MR + s2, n), x[s2]);
    const A sc = line_scale<A>(a);
#pragma unroll
    for (int q = 0; q < TL; ++q) {
        if (t0 + q >= n) break;
        A y[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            A acc = w[0] * x[q + MR][e];
#pragma unroll
            for (int d = 1; d <= MR; ++d) acc = fma(w[d], x[q + MR + d][e] + x[q + MR - d][e], acc);
            y[e] = acc * sc;
        }
        V4<T>::st(out + ls_out * (t0 + q), y);
    }
}

// Any reach: taps read through L1, four outputs per thread.
template <typename T>
__global__ void __launch_bounds__(128) k_line_g(LineArgs a) {
    using A = typename AccOf<T>::type;
    constexpr int TL = 4;
    const int n = a.dir ? a.J : a.I;
    const LinePos lp = line_pos(a.nk / 4, n, a.dir ? a.I : a.J, TL);
    if (!lp.ok) return;
    const int k = 4 * lp.q;
    const int t0 = lp.t0;
    const int line = lp.line;
    const long long ls_in = a.dir ? a.in.sj : a.in.si, os_in = a.dir ? a.in.si : a.in.sj;
    const long long ls_out = a.dir ? a.out.sj : a.out.si, os_out = a.dir ? a.out.si : a.out.sj;
    const T* in = static_cast<const T*>(a.in.p) + k + os_in * line;
    T* out = static_cast<T*>(a.out.p) + k + os_out * line;
    const A sc = line_scale<A>(a);
#pragma unroll
    for (int q = 0; q < TL; ++q) {
        const int t = t0 + q;
        if (t >= n) break;
        A acc[4], v[4];
        V4<T>::ld(in + ls_in * t, v);
        const A w0 = line_w<A>(a, 0);
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[e] = w0 * v[e];
        for (int d = 1; d <= a.R; ++d) {
            A u[4];
            V4<T>::ld(in + ls_in * reflect_half(t + d, n), u);
            V4<T>::ld(in + ls_in * reflect_half(t - d, n), v);
            const A wd = line_w<A>(a, d);
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[e] = fma(wd, u[e] + v[e], acc[e]);
        }
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[e] *= sc;
        V4<T>::st(out + ls_out * t, acc);
    }
}

// ------------------------------------------- direct-sum radial beta filter
// General support table (any aspect, any integer p): the gather form of
// fill_h + vrbeta2 (jp_pbfil.f90:888-928).  Because the radial weights are
// even in gx and gy and the mirror is half-sample, the same gather also
// equals vrbeta2t + fold_h (jp_pbfil.f90:1011-1050); the tests check this
// against the oracle's literal scatter form.  Each lane owns one k and TX
// consecutive columns; the input carries an x halo >= R + TX - 1.

// Weights and row half-widths of the support table into shared memory.
template <typename A>
__device__ __forceinline__ void hdirect_stage(const HDirectArgs& a, A* w, int* mrow) {
    const int W = 2 * a.R + 1;
    const int nthreads = blockDim.x * blockDim.y;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    for (int t = tid; t < W * W; t += nthreads) w[t] = static_cast<const A*>(a.w)[t];
    for (int t = tid; t < W; t += nthreads) mrow[t] = a.mrow[t];
    __syncthreads();
}

// One thread's sum: level k, columns i0 .. i0+TX-1 of row j (kv false: a
// padding lane that computes on a valid level but stores nothing).
template <typename T, int TX>
__device__ __forceinline__ void hdirect_strip(const HDirectArgs& a, const typename AccOf<T>::type* w,
                                              const int* mrow, int k, bool kv, int i0, int j) {
    using A = typename AccOf<T>::type;
    const int W = 2 * a.R + 1;
    A acc[TX];
#pragma unroll
    for (int q = 0; q < TX; ++q) acc[q] = A(0);
    const T* inb = static_cast<const T*>(a.in.p) + k;
    for (int gy = -a.R; gy <= a.R; ++gy) {
        const int m = mrow[gy + a.R];
        if (m < 0) continue;
        const int jr = reflect_half(j + gy, a.J);
        const T* rp = inb + a.in.sj * jr + a.in.si * (long long)(i0 - m);
        const A* wr = w + (gy + a.R) * W + a.R;
        const int ns = 2 * m + TX;
        for (int s = 0; s < ns; ++s) {
            const A v = ldv(rp + a.in.si * (long long)s);
#pragma unroll
            for (int q = 0; q < TX; ++q) {
                const int gx = s - m - q;
                if (gx >= -m && gx <= m) acc[q] = fma(wr[gx], v, acc[q]);
            }
        }
    }
    if (!kv) return;
    const A scale = static_cast<A>(a.scale);
    T* out = static_cast<T*>(a.out.p) + a.out.sj * j + k;
#pragma unroll
    for (int q = 0; q < TX; ++q) {
        const int i = i0 + q;
        if (i >= a.I) break;
        const A v = acc[q] * scale;
        stv(out + a.out.si * i, v);
        if (i < a.mirror_hx) stv(out + a.out.si * (-1 - i), v);
        if (i >= a.I - a.mirror_hx) stv(out + a.out.si * (2 * a.I - 1 - i), v);
    }
}

template <typename T, int TX>
__global__ void __launch_bounds__(128) k_hdirect(HDirectArgs a) {
    using A = typename AccOf<T>::type;
    extern __shared__ unsigned char smem_raw[];
    A* w = reinterpret_cast<A*>(smem_raw);
    int* mrow = reinterpret_cast<int*>(w + (2 * a.R + 1) * (2 * a.R + 1));
    hdirect_stage(a, w, mrow);
    int k = blockIdx.x * 32 + threadIdx.x;
    const bool kv = k < a.nk;
    if (!kv) k = a.nk - 1;
    const int i0 = (blockIdx.y * blockDim.y + threadIdx.y) * TX;
    if (i0 >= a.I) return;
    hdirect_strip<T, TX>(a, w, mrow, k, kv, i0, blockIdx.z);
}

// Few levels (the 2D variables of filtering_rad3: often one): lanes of a
// warp cover (level, strip) pairs instead of 32 levels, so none idles.
template <typename T, int TX>
__global__ void __launch_bounds__(128) k_hdirect_flat(HDirectArgs a) {
    using A = typename AccOf<T>::type;
    extern __shared__ unsigned char smem_raw[];
    A* w = reinterpret_cast<A*>(smem_raw);
    int* mrow = reinterpret_cast<int*>(w + (2 * a.R + 1) * (2 * a.R + 1));
    hdirect_stage(a, w, mrow);
    const int nstrip = (a.I + TX - 1) / TX;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)a.nk * nstrip * a.J) return;
    const int k = (int)(idx % a.nk);
    const long long r = idx / a.nk;
    hdirect_strip<T, TX>(a, w, mrow, k, true, (int)(r % nstrip) * TX, (int)(r / nstrip));
}

// ---------------------------------------------------------------- helpers
template <typename T>
__global__ void __launch_bounds__(256) k_mirror_x(View v, int nk, int I, int hx) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nk * hx) return;
    const int q = (int)(t / nk);
    const int k = (int)(t - (long long)q * nk);
    T* row = static_cast<T*>(v.p) + v.sj * blockIdx.y + k;
    row[v.si * (-1 - q)] = row[v.si * q];
    row[v.si * (I + q)] = row[v.si * (I - 1 - q)];
}

template <typename T>
__global__ void __launch_bounds__(256) k_copy(View in, View out, int nk, int I, int mirror_hx) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nk * I) return;
    const int i = (int)(t / nk);
    const int k = (int)(t - (long long)i * nk);
    const int j = blockIdx.y;
    const T v = static_cast<const T*>(in.p)[in.sj * j + in.si * i + k];
    T* o = static_cast<T*>(out.p) + out.sj * j + k;
    o[out.si * i] = v;
    if (mirror_hx) {
        if (i < mirror_hx) o[out.si * (-1 - i)] = v;
        if (i >= I - mirror_hx) o[out.si * (2 * I - 1 - i)] = v;
    }
}

// Zero every halo cell of a (nk, -hx..I+hx-1, -hy..J+hy-1) field.
template <typename T>
__global__ void __launch_bounds__(256) k_zero_halo(View v, int nk, int I, int J, int hx, int hy) {
    const int ni = I + 2 * hx;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nk * ni) return;
    const int i = (int)(t / nk) - hx;
    const int k = (int)(t - (long long)(i + hx) * nk);
    const int j = (int)blockIdx.y - hy;
    const bool halo = i < 0 || i >= I || j < 0 || j >= J;
    if (halo) static_cast<T*>(v.p)[v.sj * j + v.si * i + k] = T(0);
}

// The fast filters leave the halo corners as they were (bocox/bocoy write
// the x halo of interior rows and the y halo of interior columns only) and
// zero the rest of the halo (vrbeta1's a = b on each line).
template <typename T>
__global__ void __launch_bounds__(256) k_zero_halo_edges(View v, int nk, int I, int J, int hx, int hy) {
    const int ni = I + 2 * hx;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nk * ni) return;
    const int i = (int)(t / nk) - hx;
    const int k = (int)(t - (long long)(i + hx) * nk);
    const int j = (int)blockIdx.y - hy;
    const bool iin = i >= 0 && i < I, jin = j >= 0 && j < J;
    if (iin != jin) static_cast<T*>(v.p)[v.sj * j + v.si * i + k] = T(0);
}

template <typename T>
__global__ void __launch_bounds__(256) k_dot(DotArgs a) {
    __shared__ double red[256 / 32];
    double s = 0.0;
    const long long n = (long long)a.nk * a.I;
    const int j = blockIdx.y;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t / a.nk);
        const int k = (int)(t - (long long)i * a.nk);
        const double x = (double)ldv(static_cast<const T*>(a.a.p) + a.a.sj * j + a.a.si * i + k);
        const double y = (double)ldv(static_cast<const T*>(a.b.p) + a.b.sj * j + a.b.si * i + k);
        s = fma(x, y, s);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) atomicAdd(a.out, s);
    }
}

// ---------------------------------------------------------------- launchers
#define MGBF_DISPATCH(t, F)                                          \
    switch (t) {                                                     \
        case DType::F64: { using T = double; F; } break;             \
        case DType::F32: { using T = float; F; } break;              \
        case DType::BF16: { using T = __nv_bfloat16; F; } break;     \
    }

static inline size_t acc_size(DType t) { return t == DType::F64 ? 8 : 4; }
static inline size_t elem_size(DType t) { return t == DType::F64 ? 8 : (t == DType::F32 ? 4 : 2); }

static inline int last_err() {
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : (int)e;
}

static bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

template <typename T, int MZ>
static void zlaunch(const ZArgs& a, cudaStream_t s) {
    constexpr int ZI = 4;
    if constexpr (MZ <= 8) {  // the vector form keeps 4*(2MZ+1) weights in registers
        const bool vec = a.nk % 4 == 0 && aligned16(a.in.p) && aligned16(a.out.p);
        if (vec) {
            // column strips long enough to amortise the band setup, short
            // enough for about 8 resident waves of blocks
            const int nt = a.nk / 4;
            const long long blocks_per_col = (long long)((nt + 127) / 128) * a.J;
            int ncol = 32;
            while (ncol > ZI && blocks_per_col * ((a.I + ncol - 1) / ncol) < (long long)device_sm_count() * 8 * 4) ncol /= 2;
            dim3 block(128), grid((nt + 127) / 128, (a.I + ncol - 1) / ncol, a.J);
            k_zfilter4<T, MZ, ZI><<<grid, block, 0, s>>>(a, ncol);
            return;
        }
    }
    dim3 block(128), grid((a.nk + 127) / 128, (a.I + ZI - 1) / ZI, a.J);
    k_zfilter<T, MZ, ZI><<<grid, block, 0, s>>>(a);
}

int launch_zfilter(DType t, const ZArgs& a, void* stream) {
    if (a.nk == 0 || a.I == 0 || a.J == 0) return 0;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int mz = a.mz;
    if (mz > kMaxZReach) return (int)cudaErrorInvalidValue;
    MGBF_DISPATCH(t, (mz <= 2 ? zlaunch<T, 2>(a, s)
                      : mz <= 4 ? zlaunch<T, 4>(a, s)
                      : mz <= 6 ? zlaunch<T, 6>(a, s)
                      : mz <= 8 ? zlaunch<T, 8>(a, s)
                      : zlaunch<T, kMaxZReach>(a, s)));
    return last_err();
}


// Rows per block of the restriction kernels: about 8 waves of blocks (2
// resident per SM), at least 8 coarse rows.
static int rs_rows(long long tiles, int Jc) {
    const long long nseg = (8LL * 2 * device_sm_count() + tiles - 1) / tiles;
    int rows = (int)((Jc + nseg - 1) / nseg);
    return std::max(rows, std::min(Jc, 8));
}

ZrBox zrestrict_box(DType t, int lm, int nzk, int mz) {
    ZrBox b;
    if (t == DType::F64 || lm < 1 || mz > 8) return b;
    const int lv = (nzk == 0 || 128 % lm == 0) ? 128 : (96 % lm == 0 ? 96 : 0);
    if (!lv) return b;
    b.lv = lv;
    const int pad = t == DType::BF16 ? (mz <= 4 ? zr_pad<__nv_bfloat16, 4>() : zr_pad<__nv_bfloat16, 8>())
                                     : (mz <= 4 ? zr_pad<float, 4>() : zr_pad<float, 8>());
    b.levels = lv + 2 * pad;
    b.cols = rs_cols<float, 2>();
    return b;
}

template <typename T, int LV, int MZ, bool RONLY = false>
static int zrlaunch(const ZRestrictArgs& z, cudaStream_t s) {
    constexpr int CX = 2;
    const RestrictArgs& a = z.r;
    const int Ic = a.If / 2, Jc = a.Jf / 2;
    dim3 block(kRsWarps * 32), grid((a.nk + LV - 1) / LV, (Ic + kRsWarps * CX - 1) / (kRsWarps * CX), 1);
    const int rows = rs_rows((long long)grid.x * grid.y, Jc);
    grid.z = (Jc + rows - 1) / rows;
    constexpr size_t sm = zr_smem<T, CX, LV, MZ>();
    static unsigned long long done = 0;  // per instantiation
    cudaError_t e = smem_optin(k_zrestrict_tma<T, CX, LV, MZ, RONLY>, sm, done);
    if (e != cudaSuccess) return (int)e;
    k_zrestrict_tma<T, CX, LV, MZ, RONLY><<<grid, block, sm, s>>>(z, *static_cast<const CUtensorMap*>(z.tmap), rows);
    return last_err();
}

// compiled z reaches: 4, 5, 6 and 8 (7 runs as 8); the band's own reach
// z.mz <= MZ, taps past it have zero weight
template <typename T, int LV>
static int zrdispatch(const ZRestrictArgs& z, cudaStream_t s) {
    if (!z.write_zout && z.nzk == 0) return zrlaunch<T, LV, 4, true>(z, s);
    if (z.mz <= 4) return zrlaunch<T, LV, 4>(z, s);
    if (z.mz == 5) return zrlaunch<T, LV, 5>(z, s);
    if (z.mz == 6) return zrlaunch<T, LV, 6>(z, s);
    return zrlaunch<T, LV, 8>(z, s);
}

int launch_zrestrict(DType t, const ZRestrictArgs& z, void* stream) {
    const RestrictArgs& a = z.r;
    const ZrBox b = zrestrict_box(t, z.lm, z.nzk, z.mz);
    const long long es = (long long)elem_size(t);
    // the tensor map covers the fine field; V4 stores need 16-byte (FP32) or
    // 8-byte (BF16) aligned columns in zout and coarse
    if (!b.lv || !z.tmap || !z.status || a.nk % 4 || z.mz > 8 || a.If < 2 || a.Jf < 2 || !aligned16(z.zout.p) ||
        !aligned16(a.coarse.p) || (z.zout.si * es) % 16 || (z.zout.sj * es) % 16 || (a.coarse.si * es) % 16 ||
        (a.coarse.sj * es) % 16)
        return -1;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (t == DType::F32) return b.lv == 128 ? zrdispatch<float, 128>(z, s) : zrdispatch<float, 96>(z, s);
    return b.lv == 128 ? zrdispatch<__nv_bfloat16, 128>(z, s) : zrdispatch<__nv_bfloat16, 96>(z, s);
}

int launch_restrict(DType t, const RestrictArgs& a, void* stream) {
    const int Ic = a.If / 2, Jc = a.Jf / 2;
    if (a.nk == 0 || Ic == 0 || Jc == 0) return 0;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // lanes work in groups of 4 levels: nk % 4 == 0 (the 16-byte condition
    // alone admits nk = 2 mod 4 in FP64, whose last group would spill into
    // the next column)
    if (a.nk % 4 == 0 && (a.nk * elem_size(t)) % 16 == 0 && aligned16(a.fine.p) && aligned16(a.coarse.p)) {
        // Row segments: about 8 waves of blocks (2 resident per SM), at least
        // 8 coarse rows (3 steps of ring fill per segment); small coarse
        // generations get short segments and enough blocks, the finest
        // generation long ones.
        const int cx = t == DType::F64 ? 2 : 4;
        dim3 block(kRsWarps * 32), grid((a.nk + kRsLevels - 1) / kRsLevels, (Ic + kRsWarps * cx - 1) / (kRsWarps * cx), 1);
        const long long tiles = (long long)grid.x * grid.y;
        const long long nseg = (8LL * 2 * device_sm_count() + tiles - 1) / tiles;
        int rows = (int)((Jc + nseg - 1) / nseg);
        rows = std::max(rows, std::min(Jc, 8));
        grid.z = (Jc + rows - 1) / rows;
        static unsigned long long done[3] = {0, 0, 0};
        cudaError_t e = cudaSuccess;
        if (t == DType::F64) {
            constexpr size_t sm = rs_smem<double, 2, 4>();
            e = smem_optin(k_restrict_p<double, 2, 4>, sm, done[0]);
            if (e == cudaSuccess) k_restrict_p<double, 2, 4><<<grid, block, sm, s>>>(a, rows);
        } else if (t == DType::F32) {
            constexpr size_t sm = rs_smem<float, 4, 4>();
            e = smem_optin(k_restrict_p<float, 4, 4>, sm, done[1]);
            if (e == cudaSuccess) k_restrict_p<float, 4, 4><<<grid, block, sm, s>>>(a, rows);
        } else {
            constexpr size_t sm = rs_smem<__nv_bfloat16, 4, 4>();
            e = smem_optin(k_restrict_p<__nv_bfloat16, 4, 4>, sm, done[2]);
            if (e == cudaSuccess) k_restrict_p<__nv_bfloat16, 4, 4><<<grid, block, sm, s>>>(a, rows);
        }
        if (e != cudaSuccess) return (int)e;
        return last_err();
    }
    constexpr int NW = 4;
    const int nstrip = (Ic + RC - 1) / RC;
    dim3 block(32, NW), grid((a.nk + 31) / 32, (nstrip + NW - 1) / NW, (Jc + RC - 1) / RC);
    MGBF_DISPATCH(t, (k_restrict<T><<<grid, block, 0, s>>>(a)));
    return last_err();
}

int launch_prolong(DType t, const ProlongArgs& a, void* stream) {
    if (a.nk == 0 || a.If == 0 || a.Jf == 0) return 0;
    const int O = a.ntap == 4 ? 1 : 0;
    const int npx = a.If / 2 + O, npy = a.Jf / 2 + O;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (a.nk % 4 == 0 && aligned16(a.coarse.p) && aligned16(a.out.p) && (!a.has_base || aligned16(a.base.p))) {
        const int nt = a.nk / 4;
        dim3 block(std::min(128, ((nt + 31) / 32) * 32)), grid((nt + block.x - 1) / block.x, (npx + PV - 1) / PV, npy);
        if (a.ntap == 4) {
            MGBF_DISPATCH(t, (k_prolong4<T, 4><<<grid, block, 0, s>>>(a)));
        } else {
            MGBF_DISPATCH(t, (k_prolong4<T, 3><<<grid, block, 0, s>>>(a)));
        }
        return last_err();
    }
    constexpr int NW = 4;
    const int nstrip = (npx + PX - 1) / PX;
    dim3 block(32, NW), grid((a.nk + 31) / 32, (nstrip + NW - 1) / NW, npy);
    if (a.ntap == 4) {
        MGBF_DISPATCH(t, (k_prolong<T, 4><<<grid, block, 0, s>>>(a)));
    } else {
        MGBF_DISPATCH(t, (k_prolong<T, 3><<<grid, block, 0, s>>>(a)));
    }
    return last_err();
}

template <typename T, int MZ>
static void pzlaunch(const ProlongZArgs& z, int KT, dim3 grid, cudaStream_t s) {
    const size_t sm = sizeof(typename AccOf<T>::type) * 4 * PZ * KT;
    if (z.p.ntap == 4) k_prolong_z<T, 4, MZ><<<grid, KT, sm, s>>>(z);
    else k_prolong_z<T, 3, MZ><<<grid, KT, sm, s>>>(z);
}

template <typename T, int MZ>
static void pzlaunch4(const ProlongZArgs& z, int KT, dim3 grid, cudaStream_t s) {
    const size_t sm = sizeof(typename AccOf<T>::type) * 4 * PZ * KT;
    if (z.p.ntap == 4) k_prolong_z4<T, 4, MZ><<<grid, KT / 4, sm, s>>>(z);
    else k_prolong_z4<T, 3, MZ><<<grid, KT / 4, sm, s>>>(z);
}

PzBox prolongz_box(DType t, int lm, int ntap) {
    PzBox b;
    if (t == DType::F64 || lm < 1 || (ntap != 3 && ntap != 4)) return b;
    b.lv = 128 % lm == 0 ? 128 : (96 % lm == 0 ? 96 : 0);
    b.cols = b.lv ? (ntap == 4 ? pz_cols<float, 4>() : pz_cols<float, 3>()) : 0;
    return b;
}

// MZ: the compiled z reach (the band's own reach z.mz <= MZ; taps past it
// have zero weight)
template <typename T, int NT, int LV, int MZ>
static int pzlaunch_tma(const ProlongZArgs& z, cudaStream_t s) {
    const ProlongArgs& a = z.p;
    constexpr int O = NT == 4 ? 1 : 0;
    constexpr int kResident = MZ <= 4 ? 3 : 2;  // blocks per SM (launch bounds)
    const int npx = a.If / 2 + O, npy = a.Jf / 2 + O;
    dim3 block(128), grid((a.nk + LV - 1) / LV, (npx + 4 * kPzPairsPerWarp - 1) / (4 * kPzPairsPerWarp), 1);
    // row runs: about 8 waves of blocks, at least 4*NT row pairs so that the
    // NT-1 rows of ring fill stay cheap
    const long long tiles = (long long)grid.x * grid.y;
    const long long nseg = (8LL * kResident * device_sm_count() + tiles - 1) / tiles;
    int seg = (int)((npy + nseg - 1) / nseg);
    seg = std::max(seg, std::min(npy, 4 * NT));
    grid.z = (npy + seg - 1) / seg;
    constexpr size_t sm = pz_smem<T, NT, LV, MZ>();
    static unsigned long long done = 0;  // per instantiation
    cudaError_t e = smem_optin(k_prolong_z_tma<T, NT, LV, MZ>, sm, done);
    if (e != cudaSuccess) return (int)e;
    k_prolong_z_tma<T, NT, LV, MZ><<<grid, block, sm, s>>>(z, *static_cast<const CUtensorMap*>(z.tmap), seg);
    return last_err();
}

template <typename T, int MZ>
static int pzdispatch_tma(const ProlongZArgs& z, int lv, cudaStream_t s) {
    if (z.p.ntap == 4) return lv == 128 ? pzlaunch_tma<T, 4, 128, MZ>(z, s) : pzlaunch_tma<T, 4, 96, MZ>(z, s);
    return lv == 128 ? pzlaunch_tma<T, 3, 128, MZ>(z, s) : pzlaunch_tma<T, 3, 96, MZ>(z, s);
}

int launch_prolong_z(DType t, const ProlongZArgs& z, void* stream) {
    const ProlongArgs& a = z.p;
    if (z.lm < 2 || z.lm > 256 || z.mz > 8 || !a.has_base) return -1;
    const int O = a.ntap == 4 ? 1 : 0;
    const int npx = a.If / 2 + O, npy = a.Jf / 2 + O;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // TMA-fed form: whole z columns in 128- or 96-level blocks, 16-byte
    // aligned columns, vertical reach <= 8, coarse grids of at least NT
    // points per direction (edge mirroring stays inside the staged window)
    const PzBox b = prolongz_box(t, z.lm, a.ntap);
    const long long es = (long long)elem_size(t);
    if (b.lv && z.tmap && z.status && a.nk % 4 == 0 && a.If / 2 >= a.ntap && a.Jf / 2 >= a.ntap &&
        aligned16(a.base.p) && aligned16(a.out.p) && (a.base.si * es) % 16 == 0 && (a.base.sj * es) % 16 == 0 &&
        (a.out.si * es) % 16 == 0 && (a.out.sj * es) % 16 == 0) {
        // compiled z reaches: 4, 5, 6 and 8 (7 runs as 8)
        const int mzc = z.mz <= 4 ? 4 : z.mz <= 6 ? z.mz : 8;
        if (t == DType::F32)
            return mzc == 4 ? pzdispatch_tma<float, 4>(z, b.lv, s) : mzc == 5 ? pzdispatch_tma<float, 5>(z, b.lv, s)
                 : mzc == 6 ? pzdispatch_tma<float, 6>(z, b.lv, s) : pzdispatch_tma<float, 8>(z, b.lv, s);
        return mzc == 4 ? pzdispatch_tma<__nv_bfloat16, 4>(z, b.lv, s)
             : mzc == 5 ? pzdispatch_tma<__nv_bfloat16, 5>(z, b.lv, s)
             : mzc == 6 ? pzdispatch_tma<__nv_bfloat16, 6>(z, b.lv, s) : pzdispatch_tma<__nv_bfloat16, 8>(z, b.lv, s);
    }
    // vector form: whole columns in tiles of a multiple of 4 levels (<= 512)
    if (a.nk % 4 == 0 && aligned16(a.coarse.p) && aligned16(a.base.p) && aligned16(a.out.p)) {
        int c = 512 / z.lm;
        while (c > 0 && (c * z.lm) % 4) --c;
        if (c > 0) {
            const int KT = c * z.lm;
            dim3 grid((a.nk + KT - 1) / KT, (npx + PZ - 1) / PZ, npy);
            MGBF_DISPATCH(t, (z.mz <= 2 ? pzlaunch4<T, 2>(z, KT, grid, s)
                              : z.mz <= 4 ? pzlaunch4<T, 4>(z, KT, grid, s)
                              : pzlaunch4<T, 8>(z, KT, grid, s)));
            return last_err();
        }
    }
    const int KT = (256 / z.lm) * z.lm;
    dim3 grid((a.nk + KT - 1) / KT, (npx + PZ - 1) / PZ, npy);
    MGBF_DISPATCH(t, (z.mz <= 2 ? pzlaunch<T, 2>(z, KT, grid, s)
                      : z.mz <= 4 ? pzlaunch<T, 4>(z, KT, grid, s)
                      : pzlaunch<T, 8>(z, KT, grid, s)));
    return last_err();
}

int hmom_dispatch_f32(int R, const HMomArgs& a, const HMomCoefs<double>& c, cudaStream_t s);
int hmom_dispatch_f64(int R, const HMomArgs& a, const HMomCoefs<double>& c, cudaStream_t s);
int hmom_dispatch_bf16(int R, const HMomArgs& a, const HMomCoefs<double>& c, cudaStream_t s);

bool hmom_available(DType, int R, int p) {
    if (p != 2) return false;
    switch (R) {
#define MGBF_CASE(r) case r:
        MGBF_HMOM_REACHES(MGBF_CASE)
#undef MGBF_CASE
        return true;
        default:
            return false;
    }
}

int launch_hmom(DType t, int R, int p, const HMomArgs& a, const HMomCoefs<double>& c, void* stream) {
    if (!hmom_available(t, R, p)) return -1;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (t) {
        case DType::F64: return hmom_dispatch_f64(R, a, c, s);
        case DType::F32: return hmom_dispatch_f32(R, a, c, s);
        case DType::BF16: return hmom_dispatch_bf16(R, a, c, s);
    }
    return -1;
}

int hmom_persist_dispatch_f32(int R, const HMomPersistArgs& pa, const HMomMaps& maps, const HMomCoefs<double>& c,
                              cudaStream_t s);
int hmom_persist_dispatch_bf16(int R, const HMomPersistArgs& pa, const HMomMaps& maps, const HMomCoefs<double>& c,
                               cudaStream_t s);

int launch_hmom_persist(DType t, int R, int p, const HMomPersistArgs& pa, const HMomMaps& maps,
                        const HMomCoefs<double>& c, void* stream) {
    if (t == DType::F64 || !hmom_available(t, R, p)) return -1;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    return t == DType::F32 ? hmom_persist_dispatch_f32(R, pa, maps, c, s) : hmom_persist_dispatch_bf16(R, pa, maps, c, s);
}

int launch_hdirect(DType t, const HDirectArgs& a, void* stream) {
    constexpr int TX = 4, NW = 4;
    const int W = 2 * a.R + 1;
    const size_t sm = acc_size(t) * W * W + sizeof(int) * W;
    const int nstrip = (a.I + TX - 1) / TX;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (a.nk < 16) {
        const long long n = (long long)a.nk * nstrip * a.J;
        if (n == 0) return 0;
        if (sm > 48 * 1024) {
            MGBF_DISPATCH(t, (cudaFuncSetAttribute(k_hdirect_flat<T, TX>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm)));
        }
        MGBF_DISPATCH(t, (k_hdirect_flat<T, TX><<<(unsigned)((n + 127) / 128), 128, sm, s>>>(a)));
        return last_err();
    }
    dim3 block(32, NW), grid((a.nk + 31) / 32, (nstrip + NW - 1) / NW, a.J);
    if (sm > 48 * 1024) {
        MGBF_DISPATCH(t, (cudaFuncSetAttribute(k_hdirect<T, TX>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm)));
    }
    MGBF_DISPATCH(t, (k_hdirect<T, TX><<<grid, block, sm, s>>>(a)));
    return last_err();
}

int launch_mirror_x(DType t, View v, int nk, int I, int J, int hx, void* stream) {
    const long long n = (long long)nk * hx;
    if (n == 0 || J == 0) return 0;
    dim3 block(256), grid((unsigned)((n + 255) / 256), J);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    MGBF_DISPATCH(t, (k_mirror_x<T><<<grid, block, 0, s>>>(v, nk, I, hx)));
    return last_err();
}

int launch_copy(DType t, View in, View out, int nk, int I, int J, int mirror_hx, void* stream) {
    const long long n = (long long)nk * I;
    if (n == 0 || J == 0) return 0;
    dim3 block(256), grid((unsigned)((n + 255) / 256), J);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    MGBF_DISPATCH(t, (k_copy<T><<<grid, block, 0, s>>>(in, out, nk, I, mirror_hx)));
    return last_err();
}

int launch_zero_halo(DType t, View v, int nk, int I, int J, int hx, int hy, void* stream) {
    const long long n = (long long)nk * (I + 2 * hx);
    if (n == 0 || (hx == 0 && hy == 0)) return 0;
    dim3 block(256), grid((unsigned)((n + 255) / 256), J + 2 * hy);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    MGBF_DISPATCH(t, (k_zero_halo<T><<<grid, block, 0, s>>>(v, nk, I, J, hx, hy)));
    return last_err();
}

int launch_zero_halo_edges(DType t, View v, int nk, int I, int J, int hx, int hy, void* stream) {
    const long long n = (long long)nk * (I + 2 * hx);
    if (n == 0 || (hx == 0 && hy == 0)) return 0;
    dim3 block(256), grid((unsigned)((n + 255) / 256), J + 2 * hy);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    MGBF_DISPATCH(t, (k_zero_halo_edges<T><<<grid, block, 0, s>>>(v, nk, I, J, hx, hy)));
    return last_err();
}

// One level per thread (any nk, any alignment), four outputs, any reach.
template <typename T>
__global__ void __launch_bounds__(128) k_line_s(LineArgs a) {
    using A = typename AccOf<T>::type;
    constexpr int TL = 4;
    const int n = a.dir ? a.J : a.I;
    const LinePos lp = line_pos(a.nk, n, a.dir ? a.I : a.J, TL);
    if (!lp.ok) return;
    const int k = lp.q;
    const int t0 = lp.t0;
    const int line = lp.line;
    const long long ls_in = a.dir ? a.in.sj : a.in.si, os_in = a.dir ? a.in.si : a.in.sj;
    const long long ls_out = a.dir ? a.out.sj : a.out.si, os_out = a.dir ? a.out.si : a.out.sj;
    const T* in = static_cast<const T*>(a.in.p) + k + os_in * line;
    T* out = static_cast<T*>(a.out.p) + k + os_out * line;
    const A sc = line_scale<A>(a);
#pragma unroll
    for (int q = 0; q < TL; ++q) {
        const int t = t0 + q;
        if (t >= n) break;
        A acc = line_w<A>(a, 0) * ldv(in + ls_in * t);
        for (int d = 1; d <= a.R; ++d)
            acc = fma(line_w<A>(a, d),
                      ldv(in + ls_in * reflect_half(t + d, n)) + ldv(in + ls_in * reflect_half(t - d, n)), acc);
        stv(out + ls_out * t, acc * sc);
    }
}

static dim3 line_grid(long long nq, int n, int m, int TL) {
    const long long threads = nq * ((n + TL - 1) / TL) * (long long)m;
    return dim3((unsigned)((threads + 127) / 128));
}

template <typename T, int MR, int TL>
static void line_launch(const LineArgs& a, int n, int m, cudaStream_t s) {
    k_line_w<T, MR, TL><<<line_grid(a.nk / 4, n, m, TL), 128, 0, s>>>(a);
}

int launch_line(DType t, const LineArgs& args, void* stream) {
    if (args.nk == 0 || args.I == 0 || args.J == 0) return 0;
    if (args.R < 0 || args.R > kMaxLineReach) return (int)cudaErrorInvalidValue;
    LineArgs a = args;
    for (int d = 0; d <= kMaxLineReach; ++d) a.wf[d] = d <= a.R ? (float)a.w[d] : 0.f;
    a.scalef = (float)a.scale;
    const int n = a.dir ? a.J : a.I, m = a.dir ? a.I : a.J;
    if (a.R > n) return (int)cudaErrorInvalidValue;  // one mirror image at most
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t es = elem_size(t);
    const bool vec = a.nk % 4 == 0 && aligned16(a.in.p) && aligned16(a.out.p) && (a.in.si * es) % 16 == 0 &&
                     (a.in.sj * es) % 16 == 0 && (a.out.si * es) % 16 == 0 && (a.out.sj * es) % 16 == 0;
    if (!vec || (t == DType::BF16 && (a.nk % 8 || !aligned16(a.in.p)))) {
        MGBF_DISPATCH(t, (k_line_s<T><<<line_grid(a.nk, n, m, 4), 128, 0, s>>>(a)));
        return last_err();
    }
    if (t == DType::F64) {
        if (a.R <= 4) line_launch<double, 4, 4>(a, n, m, s);
        else if (a.R <= 8) line_launch<double, 8, 4>(a, n, m, s);
        else k_line_g<double><<<line_grid(a.nk / 4, n, m, 4), 128, 0, s>>>(a);
        return last_err();
    }
    // reach buckets; the register window TL + 2MR stays at <= 32 inputs
    auto run = [&](auto tag) {
        using T = decltype(tag);
        if (a.R <= 2) {
            line_launch<T, 2, 16>(a, n, m, s);
        } else if (a.R <= 4) {
            line_launch<T, 4, 16>(a, n, m, s);
        } else if (a.R <= 6) {
            line_launch<T, 6, 16>(a, n, m, s);
        } else if (a.R <= 8) {
            line_launch<T, 8, 16>(a, n, m, s);
        } else if (a.R <= 12) {
            line_launch<T, 12, 8>(a, n, m, s);
        } else if (a.R <= 14) {
            line_launch<T, 14, 4>(a, n, m, s);
        } else if (a.R <= 16) {
            line_launch<T, 16, 4>(a, n, m, s);
        } else {
            k_line_g<T><<<line_grid(a.nk / 4, n, m, 4), 128, 0, s>>>(a);
        }
    };
    if (t == DType::F32) run(float());
    else run(__nv_bfloat16());
    return last_err();
}

int launch_dot(DType t, const DotArgs& a, void* stream) {
    const long long n = (long long)a.nk * a.I;
    if (n == 0 || a.J == 0) return 0;
    unsigned gx = (unsigned)((n + 255) / 256);
    if (gx > 64) gx = 64;
    dim3 block(256), grid(gx, a.J);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    MGBF_DISPATCH(t, (k_dot<T><<<grid, block, 0, s>>>(a)));
    return last_err();
}

}  // namespace mgbf
