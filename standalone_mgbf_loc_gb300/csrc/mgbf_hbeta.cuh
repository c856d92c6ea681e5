// Radial beta filter, moment form (sm_103a).
//
// The reference's normalised radial beta weight (vrbeta2, jp_pbfil.f90:888-928)
// is w(gx,gy) = s*(1 - e^2 gy^2 - e^2 gx^2)^p on a disk whose row half-widths
// are m(gy).  For a fixed row gy it is a polynomial of degree p in
// u = (e gx)^2:  w = s * sum_q C(p,q) (-1)^q A(gy)^(p-q) u^q,  A = 1 - (e gy)^2.
// So the row sum  sum_{|gx|<=m(gy)} w a(i+gx)  equals
//   sum_q c_q(gy) T_q^{m(gy)}(i),   T_q^m(i) = sum_{|gx|<=m} (e gx)^(2q) a(i+gx),
// and T_q^m grows from T_q^{m-1} by (e m)^(2q) (a(i+m)+a(i-m)).  With the
// binomial factors and signs folded into the increments (T'_q) and s moved
// to the store, the row sum is the Horner form ((T'_0 A + T'_1) A + ...) + T'_p.  One pass over
// m = 0..R per input row yields every row width the disk needs; each width is
// emitted (symmetrically for +gy and -gy) into a ring of output-row
// accumulators as the kernel streams down the rows.  This is the same linear
// operator as the reference's direct disk sum (exact in exact arithmetic);
// it costs about (p+2)R + (p+3)(R+1) operations per point and row instead of
// the disk's ~pi R^2 multiply-adds.
//
// The disk shape is compiled in: the kernel for reach R uses the row widths
// of radius R + 1/2 (m(gy)^2 <= R^2 + R - gy^2), which is the support of
// every aspect mg_ampl02 = (R+1/2)^2/(2p+4).  The host checks the runtime
// support against this table and otherwise runs the direct-sum kernel.
//
// Thread mapping: lane = level index k (coalesced 128-byte rows in the
// k-fastest layout); each lane owns TX consecutive columns and streams
// a block of output rows; the input carries a mirrored x halo >= R+TX-1 and
// rows are mirrored (half-sample) by index.
#pragma once
#include "mgbf_common.cuh"
#include "mgbf_kernels.cuh"

#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

namespace mgbf {

template <int R>
__host__ __device__ constexpr int mcanon(int gy) {
    const int lim = R * R + R - gy * gy;
    int m = 0;
    while ((m + 1) * (m + 1) <= lim) ++m;
    return m;
}

template <int R, int P, int TX, int U, typename T>
__global__ void __launch_bounds__(128) k_hmom(HMomArgs a,
                                              const __grid_constant__ HMomCoefs<typename AccOf<T>::type> c) {
    static_assert(U == 2, "the row pipeline alternates two register buffers");
    using A = typename AccOf<T>::type;
    constexpr int NS = TX + 2 * R;  // input columns per row
    constexpr int NR = 2 * R + U;   // ring of output rows
    constexpr int PQ = P + 1;
    int k = blockIdx.x * 32 + threadIdx.x;
    const bool kv = k < a.nk;
    if (!kv) k = a.nk - 1;
    const int i0 = (blockIdx.y * blockDim.y + threadIdx.y) * TX;
    if (i0 >= a.I) return;
    const int jb = blockIdx.z * a.rows;
    const int je = min(jb + a.rows, a.J);
    const T* inb = static_cast<const T*>(a.in.p) + k + a.in.si * (long long)(i0 - R);
    T* outb = static_cast<T*>(a.out.p) + k;
    const A scale = static_cast<A>(a.scale);

    A acc[NR][TX];
#pragma unroll
    for (int r = 0; r < NR; ++r)
#pragma unroll
        for (int q = 0; q < TX; ++q) acc[r][q] = A(0);

    auto load_row = [&](int jin, A (&seg)[NS]) {
        const T* rp = inb + a.in.sj * (long long)reflect_half(jin, a.J);
#pragma unroll
        for (int s = 0; s < NS; ++s) seg[s] = ldv(rp + a.in.si * (long long)s);
    };
    // moments of one input row, emitted into the ring rows u-gy+R and u+gy+R
    auto row = [&](const A (&seg)[NS], const int u) {
#pragma unroll
        for (int q = 0; q < TX; ++q) {
            A t[PQ];
            t[0] = seg[R + q];
#pragma unroll
            for (int e = 1; e < PQ; ++e) t[e] = A(0);
#pragma unroll
            for (int m = 0; m <= R; ++m) {
                if (m > 0) {
                    const A pr = seg[R + q + m] + seg[R + q - m];
                    t[0] += pr;
#pragma unroll
                    for (int e = 1; e < PQ; ++e) t[e] = fma(c.upow[m * PQ + e], pr, t[e]);
                }
#pragma unroll
                for (int gy = 0; gy <= R; ++gy) {
                    if (mcanon<R>(gy) == m) {
                        const A Ay = c.coef[gy * PQ];  // A(gy) = 1 - (e gy)^2
                        A v = t[0];
#pragma unroll
                        for (int e = 1; e < PQ; ++e) v = fma(v, Ay, t[e]);
                        acc[R + u - gy][q] += v;
                        if (gy) acc[R + u + gy][q] += v;
                    }
                }
            }
        }
    };

    A segA[NS], segB[NS];
    load_row(jb - R, segA);
    for (int jin0 = jb - R; jin0 < je + R; jin0 += U) {
        load_row(jin0 + 1, segB);  // in flight while row jin0 is processed
        row(segA, 0);
        load_row(jin0 + 2, segA);
        row(segB, 1);
        // rows jin0-R .. jin0-R+U-1 have received every contribution
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int jo = jin0 - R + u;
            if (kv && jo >= jb && jo < je) {
                T* orow = outb + a.out.sj * (long long)jo;
#pragma unroll
                for (int q = 0; q < TX; ++q) {
                    const int i = i0 + q;
                    if (i < a.I) {
                        const A v = acc[u][q] * scale;
                        stv(orow + a.out.si * (long long)i, v);
                        if (i < a.mirror_hx) stv(orow + a.out.si * (long long)(-1 - i), v);
                        if (i >= a.I - a.mirror_hx) stv(orow + a.out.si * (long long)(2 * a.I - 1 - i), v);
                    }
                }
            }
        }
#pragma unroll
        for (int r = 0; r < NR - U; ++r)
#pragma unroll
            for (int q = 0; q < TX; ++q) acc[r][q] = acc[r + U][q];
#pragma unroll
        for (int r = NR - U; r < NR; ++r)
#pragma unroll
            for (int q = 0; q < TX; ++q) acc[r][q] = A(0);
    }
}

// Shared-memory staged variant: the block's rows (32 levels x the block's
// column range + 2R halo) are copied into a DS-deep ring of tiles by
// cp.async (16-byte chunks, zero-filled outside the field), DS-1 rows ahead
// of the row being filtered; lanes then read their row segment from shared
// memory.  Needs nk * sizeof(T) to be a multiple of 16 (16-byte aligned
// columns; chunks never straddle a column end).
constexpr int kStages = 4;
constexpr int kStageWarps = 4;


template <int R, int TX, typename T>
constexpr size_t hmom_stage_bytes() {
    return (size_t)kStages * (kStageWarps * TX + 2 * R) * 32 * sizeof(T);
}

template <int R, int P, int TX, typename T>
__global__ void __launch_bounds__(128) k_hmom_st(HMomArgs a,
                                                 const __grid_constant__ HMomCoefs<typename AccOf<T>::type> c) {
    using A = typename AccOf<T>::type;
    constexpr int U = 2;
    constexpr int NS = TX + 2 * R;
    constexpr int NR = 2 * R + U;
    constexpr int PQ = P + 1;
    constexpr int NC = kStageWarps * TX + 2 * R;   // tile columns
    constexpr int CH = 32 * (int)sizeof(T) / 16;   // 16-byte chunks per column
    constexpr int TILE = NC * 32;                  // elements per tile
    constexpr int EPC = 16 / (int)sizeof(T);       // elements per chunk
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T* tiles = reinterpret_cast<T*>(smem_raw);
    const unsigned sbase = (unsigned)__cvta_generic_to_shared(smem_raw);
    const int lane = threadIdx.x, warp = threadIdx.y, tid = warp * 32 + lane;
    const int k0 = blockIdx.x * 32;
    const int ib = blockIdx.y * (kStageWarps * TX);
    const int jb = blockIdx.z * a.rows;
    const int je = min(jb + a.rows, a.J);
    const T* gin = static_cast<const T*>(a.in.p);
    const int colmax = a.I + a.halo - 1;  // last readable column of the padded buffer

    auto issue = [&](int jin, int st) {
        const int jr = reflect_half(jin, a.J);
        const T* rowp = gin + a.in.sj * (long long)jr + k0;
        for (int q = tid; q < NC * CH; q += kStageWarps * 32) {
            const int col = q / CH, ch = q - col * CH;
            const int gcol = ib - R + col;
            const bool ok = gcol <= colmax && k0 + ch * EPC < a.nk;
            const T* src = ok ? rowp + a.in.si * (long long)gcol + ch * EPC : gin;
            cp_async16(sbase + (unsigned)(((st * TILE + col * 32) * (int)sizeof(T)) + ch * 16), src, ok ? 16 : 0);
        }
        cp_async_commit();
    };

    const int i0 = ib + warp * TX;
    const bool kv = k0 + lane < a.nk;
    T* outb = static_cast<T*>(a.out.p) + k0 + lane;
    const A scale = static_cast<A>(a.scale);
    A acc[NR][TX];
#pragma unroll
    for (int r = 0; r < NR; ++r)
#pragma unroll
        for (int q = 0; q < TX; ++q) acc[r][q] = A(0);

    auto row = [&](const int st, const int u) {
        const T* tp = tiles + st * TILE + warp * TX * 32 + lane;
        A seg[NS];
#pragma unroll
        for (int s2 = 0; s2 < NS; ++s2) seg[s2] = ldc(tp + s2 * 32);
#pragma unroll
        for (int q = 0; q < TX; ++q) {
            A t[PQ];
            t[0] = seg[R + q];
#pragma unroll
            for (int e = 1; e < PQ; ++e) t[e] = A(0);
#pragma unroll
            for (int m = 0; m <= R; ++m) {
                if (m > 0) {
                    const A pr = seg[R + q + m] + seg[R + q - m];
                    t[0] += pr;
#pragma unroll
                    for (int e = 1; e < PQ; ++e) t[e] = fma(c.upow[m * PQ + e], pr, t[e]);
                }
#pragma unroll
                for (int gy = 0; gy <= R; ++gy) {
                    if (mcanon<R>(gy) == m) {
                        const A Ay = c.coef[gy * PQ];
                        A v = t[0];
#pragma unroll
                        for (int e = 1; e < PQ; ++e) v = fma(v, Ay, t[e]);
                        acc[R + u - gy][q] += v;
                        if (gy) acc[R + u + gy][q] += v;
                    }
                }
            }
        }
    };

    const int nrows = je - jb + 2 * R;  // input rows jb-R .. je+R-1
#pragma unroll
    for (int s2 = 0; s2 < kStages - 1; ++s2) issue(jb - R + s2, s2);
    for (int r0 = 0; r0 < nrows; r0 += U) {
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int r = r0 + u;
            cp_async_wait<kStages - 2>();
            __syncthreads();
            issue(jb - R + r + kStages - 1, (r + kStages - 1) % kStages);
            row(r % kStages, u);
        }
        const int jin0 = jb - R + r0;
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int jo = jin0 - R + u;
            if (kv && jo >= jb && jo < je) {
                T* orow = outb + a.out.sj * (long long)jo;
#pragma unroll
                for (int q = 0; q < TX; ++q) {
                    const int i = i0 + q;
                    if (i < a.I) {
                        const A v = acc[u][q] * scale;
                        stv(orow + a.out.si * (long long)i, v);
                        if (i < a.mirror_hx) stv(orow + a.out.si * (long long)(-1 - i), v);
                        if (i >= a.I - a.mirror_hx) stv(orow + a.out.si * (long long)(2 * a.I - 1 - i), v);
                    }
                }
            }
        }
#pragma unroll
        for (int r = 0; r < NR - U; ++r)
#pragma unroll
            for (int q = 0; q < TX; ++q) acc[r][q] = acc[r + U][q];
#pragma unroll
        for (int r = NR - U; r < NR; ++r)
#pragma unroll
            for (int q = 0; q < TX; ++q) acc[r][q] = A(0);
    }
    cp_async_wait<0>();
}

// Packed variant for FP32 arithmetic (FP32 or BF16 storage): each lane owns
// two adjacent levels (k, k+1) as one float2, so every multiply-add of the
// moment recurrences and of the Horner emission is one f32x2 instruction
// (__ffma2_rn / __fadd2_rn); the block covers 64 levels.  Rows are staged
// through shared memory as in k_hmom_st (DS-deep cp.async ring, 16-byte
// chunks) and U = 4 rows share one ring shift.
template <typename T> struct P2;
template <> struct P2<float> {
    static __device__ __forceinline__ float2 lds(const float* p) { return *reinterpret_cast<const float2*>(p); }
    static __device__ __forceinline__ void st(float* p, float2 v) { *reinterpret_cast<float2*>(p) = v; }
};
template <> struct P2<__nv_bfloat16> {
    static __device__ __forceinline__ float2 lds(const __nv_bfloat16* p) {
        const unsigned u = *reinterpret_cast<const unsigned*>(p);
        return make_float2(__uint_as_float(u << 16), __uint_as_float(u & 0xffff0000u));
    }
    static __device__ __forceinline__ void st(__nv_bfloat16* p, float2 v) {
        *reinterpret_cast<__nv_bfloat162*>(p) = __floats2bfloat162_rn(v.x, v.y);
    }
};

struct HMomCoefs2 {
    float2 coef[kMaxReach + 1];                  // (A(gy), A(gy))
    float2 upow[(kMaxReach + 1) * (kMaxMomP + 1)];  // (c, c) of HMomCoefs::upow
};

template <int R, int TX, typename T>
constexpr size_t hmom_p2_stage_bytes() {
    return (size_t)kStages * (kStageWarps * TX + 2 * R) * 64 * sizeof(T);
}

template <int R, int P, int TX, typename T>
__global__ void __launch_bounds__(128) k_hmom_p2(HMomArgs a, const __grid_constant__ HMomCoefs2 c) {
    constexpr int U = kStages;                     // stage index == u
    constexpr int NS = TX + 2 * R;
    constexpr int NR = 2 * R + U;
    constexpr int PQ = P + 1;
    constexpr int NC = kStageWarps * TX + 2 * R;
    constexpr int CB = 64 * (int)sizeof(T);        // bytes per tile column
    constexpr int CH = CB / 16;
    constexpr int TILE = NC * 64;
    constexpr int EPC = 16 / (int)sizeof(T);
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T* tiles = reinterpret_cast<T*>(smem_raw);
    const unsigned sbase = (unsigned)__cvta_generic_to_shared(smem_raw);
    const int lane = threadIdx.x, warp = threadIdx.y, tid = warp * 32 + lane;
    const int k0 = blockIdx.x * 64;
    const int ib = blockIdx.y * (kStageWarps * TX);
    const int jb = blockIdx.z * a.rows;
    const int je = min(jb + a.rows, a.J);
    const T* gin = static_cast<const T*>(a.in.p);
    const int colmax = a.I + a.halo - 1;

    auto issue = [&](int jin, int st) {
        const int jr = reflect_half(jin, a.J);
        const T* rowp = gin + a.in.sj * (long long)jr + k0;
        for (int q = tid; q < NC * CH; q += kStageWarps * 32) {
            const int col = q / CH, ch = q - col * CH;
            const int gcol = ib - R + col;
            const bool ok = gcol <= colmax && k0 + ch * EPC < a.nk;
            const T* src = ok ? rowp + a.in.si * (long long)gcol + ch * EPC : gin;
            cp_async16(sbase + (unsigned)(((st * TILE + col * 64) * (int)sizeof(T)) + ch * 16), src, ok ? 16 : 0);
        }
        cp_async_commit();
    };

    const int i0 = ib + warp * TX;
    const int kl = k0 + 2 * lane;
    const bool kv = kl < a.nk;                     // nk is even: both levels valid
    T* outb = static_cast<T*>(a.out.p) + kl;
    const float2 scale = make_float2((float)a.scale, (float)a.scale);
    float2 acc[NR][TX];
#pragma unroll
    for (int r = 0; r < NR; ++r)
#pragma unroll
        for (int q = 0; q < TX; ++q) acc[r][q] = make_float2(0.f, 0.f);

    auto row = [&](const int st, const int u) {
        const T* tp = tiles + st * TILE + warp * TX * 64 + 2 * lane;
        float2 seg[NS];
#pragma unroll
        for (int s2 = 0; s2 < NS; ++s2) seg[s2] = P2<T>::lds(tp + s2 * 64);
#pragma unroll
        for (int q = 0; q < TX; ++q) {
            float2 t[PQ];
            t[0] = seg[R + q];
#pragma unroll
            for (int e = 1; e < PQ; ++e) t[e] = make_float2(0.f, 0.f);
#pragma unroll
            for (int m = 0; m <= R; ++m) {
                if (m > 0) {
                    const float2 pr = __fadd2_rn(seg[R + q + m], seg[R + q - m]);
                    t[0] = __fadd2_rn(t[0], pr);
#pragma unroll
                    for (int e = 1; e < PQ; ++e) t[e] = __ffma2_rn(c.upow[m * PQ + e], pr, t[e]);
                }
#pragma unroll
                for (int gy = 0; gy <= R; ++gy) {
                    if (mcanon<R>(gy) == m) {
                        float2 v = t[0];
#pragma unroll
                        for (int e = 1; e < PQ; ++e) v = __ffma2_rn(v, c.coef[gy], t[e]);
                        acc[R + u - gy][q] = __fadd2_rn(acc[R + u - gy][q], v);
                        if (gy) acc[R + u + gy][q] = __fadd2_rn(acc[R + u + gy][q], v);
                    }
                }
            }
        }
    };

    const int nrows = je - jb + 2 * R;
#pragma unroll
    for (int s2 = 0; s2 < kStages - 1; ++s2) issue(jb - R + s2, s2);
    for (int r0 = 0; r0 < nrows; r0 += U) {
#pragma unroll
        for (int u = 0; u < U; ++u) {
            cp_async_wait<kStages - 2>();
            __syncthreads();
            issue(jb - R + r0 + u + kStages - 1, (u + kStages - 1) % kStages);
            row(u, u);
        }
        const int jin0 = jb - R + r0;
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int jo = jin0 - R + u;
            if (kv && jo >= jb && jo < je) {
                T* orow = outb + a.out.sj * (long long)jo;
#pragma unroll
                for (int q = 0; q < TX; ++q) {
                    const int i = i0 + q;
                    if (i < a.I) {
                        const float2 v = __fmul2_rn(acc[u][q], scale);
                        P2<T>::st(orow + a.out.si * (long long)i, v);
                        if (i < a.mirror_hx) P2<T>::st(orow + a.out.si * (long long)(-1 - i), v);
                        if (i >= a.I - a.mirror_hx) P2<T>::st(orow + a.out.si * (long long)(2 * a.I - 1 - i), v);
                    }
                }
            }
        }
#pragma unroll
        for (int r = 0; r < NR - U; ++r)
#pragma unroll
            for (int q = 0; q < TX; ++q) acc[r][q] = acc[r + U][q];
#pragma unroll
        for (int r = NR - U; r < NR; ++r)
#pragma unroll
            for (int q = 0; q < TX; ++q) acc[r][q] = make_float2(0.f, 0.f);
    }
    cp_async_wait<0>();
}

// TMA variant of the packed kernel: one thread issues one
// cp.async.bulk.tensor.3d per input row (box 64 levels x NC columns x 1 row
// of the padded generation buffer; out-of-range levels and columns are
// zero-filled by the copy engine) into a kStages-deep ring of tiles, each
// guarded by an mbarrier with expect_tx.  Consumers wait on the barrier
// parity with a bounded number of polls (a.max_polls); if the bound runs
// out the block records the failure in a.status and leaves through a
// block-uniform exit after a bounded drain of its own copies.
constexpr int kTmaStages = 8;  // rows in flight: kTmaStages - 2

template <int R, int TX, typename T>
constexpr size_t hmom_tma_stage_bytes() {
    return (size_t)kTmaStages * (kStageWarps * TX + 2 * R) * 64 * sizeof(T);
}

// SEQ: the two rows of a barrier are filtered one after the other (the
// registers of one row, as k_hmom_tma1, with half its block barriers);
// otherwise both rows' chains run interleaved for more work in flight.
template <int R, int P, int TX, typename T, bool SEQ>
__global__ void __launch_bounds__(128, SEQ ? 4 : 1) k_hmom_tma(HMomArgs a, const __grid_constant__ CUtensorMap tmap,
                                                  const __grid_constant__ HMomCoefs2 c) {
    constexpr int U = 4;                           // rows per ring shift
    constexpr int NS = TX + 2 * R;
    constexpr int NR = 2 * R + U;
    constexpr int PQ = P + 1;
    constexpr int NC = kStageWarps * TX + 2 * R;
    constexpr int TILE = NC * 64;
    constexpr unsigned TILE_BYTES = TILE * sizeof(T);
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) unsigned long long bars[kTmaStages];
    T* tiles = reinterpret_cast<T*>(smem_raw);
    const unsigned sbase = (unsigned)__cvta_generic_to_shared(smem_raw);
    const unsigned bbase = (unsigned)__cvta_generic_to_shared(bars);
    const int lane = threadIdx.x, warp = threadIdx.y, tid = warp * 32 + lane;
    const int k0 = blockIdx.x * 64;
    const int ib = blockIdx.y * (kStageWarps * TX);
    const int jb = blockIdx.z * a.rows;
    const int je = min(jb + a.rows, a.J);
    const int nrows = je - jb + 2 * R;
    const int nrp = ((nrows + U - 1) / U) * U;  // rows read by the unrolled loop
    if (tid == 0) {
#pragma unroll
        for (int s2 = 0; s2 < kTmaStages; ++s2) mbar_init(bbase + 8 * s2, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    auto issue = [&](int r) {
        if (tid == 0 && r < nrp) {
            const int st = r % kTmaStages;
            const int jr = reflect_half(jb - R + r, a.J);
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            mbar_expect_tx(bbase + 8 * st, TILE_BYTES);
            tma_load_3d(sbase + st * TILE_BYTES, &tmap, k0, ib - R + a.halo, jr, bbase + 8 * st);
        }
    };

    const int i0 = ib + warp * TX;
    const int kl = k0 + 2 * lane;
    const bool kv = kl < a.nk;
    T* outb = static_cast<T*>(a.out.p) + kl;
    const float2 scale = make_float2((float)a.scale, (float)a.scale);
    float2 acc[NR][TX];
#pragma unroll
    for (int r = 0; r < NR; ++r)
#pragma unroll
        for (int q = 0; q < TX; ++q) acc[r][q] = make_float2(0.f, 0.f);

    auto row1 = [&](const int st, const int u) {
        const T* tp = tiles + st * TILE + warp * TX * 64 + 2 * lane;
        float2 seg[NS];
#pragma unroll
        for (int s2 = 0; s2 < NS; ++s2) seg[s2] = P2<T>::lds(tp + s2 * 64);
#pragma unroll
        for (int q = 0; q < TX; ++q) {
            float2 t[PQ];
            t[0] = seg[R + q];
#pragma unroll
            for (int e = 1; e < PQ; ++e) t[e] = make_float2(0.f, 0.f);
#pragma unroll
            for (int m = 0; m <= R; ++m) {
                if (m > 0) {
                    const float2 pr = __fadd2_rn(seg[R + q + m], seg[R + q - m]);
                    t[0] = __fadd2_rn(t[0], pr);
#pragma unroll
                    for (int e = 1; e < PQ; ++e) t[e] = __ffma2_rn(c.upow[m * PQ + e], pr, t[e]);
                }
#pragma unroll
                for (int gy = 0; gy <= R; ++gy) {
                    if (mcanon<R>(gy) == m) {
                        float2 v = t[0];
#pragma unroll
                        for (int e = 1; e < PQ; ++e) v = __ffma2_rn(v, c.coef[gy], t[e]);
                        acc[R + u - gy][q] = __fadd2_rn(acc[R + u - gy][q], v);
                        if (gy) acc[R + u + gy][q] = __fadd2_rn(acc[R + u + gy][q], v);
                    }
                }
            }
        }
    };

    // Two input rows (ring slots u and u+1) at once: their moment chains are
    // independent, which doubles the work in flight per warp.
    auto row2 = [&](const int st0, const int st1, const int u) {
        const T* tp0 = tiles + st0 * TILE + warp * TX * 64 + 2 * lane;
        const T* tp1 = tiles + st1 * TILE + warp * TX * 64 + 2 * lane;
        float2 sa[NS], sb[NS];
#pragma unroll
        for (int s2 = 0; s2 < NS; ++s2) {
            sa[s2] = P2<T>::lds(tp0 + s2 * 64);
            sb[s2] = P2<T>::lds(tp1 + s2 * 64);
        }
#pragma unroll
        for (int q = 0; q < TX; ++q) {
            float2 ta[PQ], tb[PQ];
            ta[0] = sa[R + q];
            tb[0] = sb[R + q];
#pragma unroll
            for (int e = 1; e < PQ; ++e) ta[e] = tb[e] = make_float2(0.f, 0.f);
#pragma unroll
            for (int m = 0; m <= R; ++m) {
                if (m > 0) {
                    const float2 pa = __fadd2_rn(sa[R + q + m], sa[R + q - m]);
                    const float2 pb = __fadd2_rn(sb[R + q + m], sb[R + q - m]);
                    ta[0] = __fadd2_rn(ta[0], pa);
                    tb[0] = __fadd2_rn(tb[0], pb);
#pragma unroll
                    for (int e = 1; e < PQ; ++e) {
                        ta[e] = __ffma2_rn(c.upow[m * PQ + e], pa, ta[e]);
                        tb[e] = __ffma2_rn(c.upow[m * PQ + e], pb, tb[e]);
                    }
                }
#pragma unroll
                for (int gy = 0; gy <= R; ++gy) {
                    if (mcanon<R>(gy) == m) {
                        float2 va = ta[0], vb = tb[0];
#pragma unroll
                        for (int e = 1; e < PQ; ++e) {
                            va = __ffma2_rn(va, c.coef[gy], ta[e]);
                            vb = __ffma2_rn(vb, c.coef[gy], tb[e]);
                        }
                        acc[R + u - gy][q] = __fadd2_rn(acc[R + u - gy][q], va);
                        acc[R + u + 1 - gy][q] = __fadd2_rn(acc[R + u + 1 - gy][q], vb);
                        if (gy) {
                            acc[R + u + gy][q] = __fadd2_rn(acc[R + u + gy][q], va);
                            acc[R + u + 1 + gy][q] = __fadd2_rn(acc[R + u + 1 + gy][q], vb);
                        }
                    }
                }
            }
        }
    };

#pragma unroll
    for (int s2 = 0; s2 < kTmaStages - 2; ++s2) issue(s2);
    bool failed = false;
    int waited = 0;  // rows whose barrier has been waited
    for (int r0 = 0; r0 < nrp && !failed; r0 += U) {
#pragma unroll
        for (int u = 0; u < U; u += 2) {
            const int r = r0 + u;
            const int st0 = r % kTmaStages, st1 = (r + 1) % kTmaStages;
            const unsigned par = (unsigned)((r / kTmaStages) & 1);  // r even: r, r+1 share a phase
            const bool ok = mbar_wait_bounded(bbase + 8 * st0, par, a.max_polls) &&
                            mbar_wait_bounded(bbase + 8 * st1, par, a.max_polls);
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
            waited = r + 2;
            // the previous pair's stages are free now
            issue(r + kTmaStages - 2);
            issue(r + kTmaStages - 1);
            if constexpr (SEQ) {
                row1(st0, u);
                row1(st1, u + 1);
            } else {
                row2(st0, st1, u);
            }
        }
        if (failed) break;
        const int jin0 = jb - R + r0;
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int jo = jin0 - R + u;
            if (kv && jo >= jb && jo < je) {
                T* orow = outb + a.out.sj * (long long)jo;
#pragma unroll
                for (int q = 0; q < TX; ++q) {
                    const int i = i0 + q;
                    if (i < a.I) {
                        const float2 v = __fmul2_rn(acc[u][q], scale);
                        P2<T>::st(orow + a.out.si * (long long)i, v);
                        if (i < a.mirror_hx) P2<T>::st(orow + a.out.si * (long long)(-1 - i), v);
                        if (i >= a.I - a.mirror_hx) P2<T>::st(orow + a.out.si * (long long)(2 * a.I - 1 - i), v);
                    }
                }
            }
        }
#pragma unroll
        for (int r = 0; r < NR - U; ++r)
#pragma unroll
            for (int q = 0; q < TX; ++q) acc[r][q] = acc[r + U][q];
#pragma unroll
        for (int r = NR - U; r < NR; ++r)
#pragma unroll
            for (int q = 0; q < TX; ++q) acc[r][q] = make_float2(0.f, 0.f);
    }
    if (failed) {
        // record, then drain this block's outstanding copies (bounded) before exit
        if (tid == 0) {
            atomicExch(a.status, 1);
            const int issued = min(nrp, waited + kTmaStages - 2);
            for (int r = waited; r < issued; ++r)
                mbar_wait_bounded(bbase + 8 * (r % kTmaStages), (unsigned)((r / kTmaStages) & 1), kDefaultWaitPolls);
        }
        __syncthreads();
    }
}

// One tile of the single-row TMA pipeline (4-deep ring, one input row per
// barrier): levels k0 .. k0+63, the column strip from ib, output rows
// jb .. min(jb + a.rows, a.J) - 1.  The tile reads nrp rows, a multiple of
// kStages; its row r uses ring stage r % kStages and the phase parity of
// row rbase + r, so a persistent block that runs tile after tile continues
// the barriers' phases (rbase is the rows its earlier tiles read).  Returns
// false when a bounded wait ran out, after recording it in a.status and
// draining this block's own copies.
template <int R, int TX>
__host__ __device__ constexpr int hmom_tma1_rows(int out_rows) {
    return ((out_rows + 2 * R + kStages - 1) / kStages) * kStages;
}

template <int R, int P, int TX, typename T, bool MIRROR = false>
__device__ __forceinline__ bool hmom_tma1_tile(const HMomArgs& a, const CUtensorMap* tmap, const HMomCoefs2& c,
                                               int k0, int ib, int jb, unsigned sbase, unsigned bbase, int rbase) {
    constexpr int U = kStages;
    constexpr int NS = TX + 2 * R;
    constexpr int NR = 2 * R + U;
    constexpr int PQ = P + 1;
    constexpr int NC = kStageWarps * TX + 2 * R;
    constexpr int TILE = NC * 64;
    constexpr unsigned TILE_BYTES = TILE * sizeof(T);
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const T* tiles = reinterpret_cast<const T*>(smem_raw);
    const int lane = threadIdx.x, warp = threadIdx.y, tid = warp * 32 + lane;
    const int je = min(jb + a.rows, a.J);
    const int nrp = hmom_tma1_rows<R, TX>(je - jb);  // rows read by the unrolled loop
    auto issue = [&](int r) {
        if (tid == 0 && r < nrp) {
            const int st = r % kStages;
            const int jr = reflect_half(jb - R + r, a.J);
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            mbar_expect_tx(bbase + 8 * st, TILE_BYTES);
            tma_load_3d(sbase + st * TILE_BYTES, tmap, k0, ib - R + a.halo, jr, bbase + 8 * st);
        }
    };

    const int i0 = ib + warp * TX;
    const int kl = k0 + 2 * lane;
    const bool kv = kl < a.nk;
    T* outb = static_cast<T*>(a.out.p) + kl;
    const float2 scale = make_float2((float)a.scale, (float)a.scale);
    float2 acc[NR][TX];
#pragma unroll
    for (int r = 0; r < NR; ++r)
#pragma unroll
        for (int q = 0; q < TX; ++q) acc[r][q] = make_float2(0.f, 0.f);

    auto row = [&](const int st, const int u) {
        const T* tp = tiles + st * TILE + warp * TX * 64 + 2 * lane;
        float2 seg[NS];
#pragma unroll
        for (int s2 = 0; s2 < NS; ++s2) seg[s2] = P2<T>::lds(tp + s2 * 64);
#pragma unroll
        for (int q = 0; q < TX; ++q) {
            float2 t[PQ];
            t[0] = seg[R + q];
#pragma unroll
            for (int e = 1; e < PQ; ++e) t[e] = make_float2(0.f, 0.f);
#pragma unroll
            for (int m = 0; m <= R; ++m) {
                if (m > 0) {
                    const float2 pr = __fadd2_rn(seg[R + q + m], seg[R + q - m]);
                    t[0] = __fadd2_rn(t[0], pr);
#pragma unroll
                    for (int e = 1; e < PQ; ++e) t[e] = __ffma2_rn(c.upow[m * PQ + e], pr, t[e]);
                }
#pragma unroll
                for (int gy = 0; gy <= R; ++gy) {
                    if (mcanon<R>(gy) == m) {
                        float2 v = t[0];
#pragma unroll
                        for (int e = 1; e < PQ; ++e) v = __ffma2_rn(v, c.coef[gy], t[e]);
                        acc[R + u - gy][q] = __fadd2_rn(acc[R + u - gy][q], v);
                        if (gy) acc[R + u + gy][q] = __fadd2_rn(acc[R + u + gy][q], v);
                    }
                }
            }
        }
    };

#pragma unroll
    for (int s2 = 0; s2 < kStages - 1; ++s2) issue(s2);
    bool failed = false;
    int waited = 0;  // rows whose barrier has been waited
    // MIRROR (input without x halo, a.mirror_in): tile column c holds input
    // column g0 + c; the copy engine zero-fills columns outside 0..I-1, and
    // the edge tiles replace those that feed stored outputs (-R..-1 and
    // I..I+R-1) by their half-sample mirrors, which lie inside the same tile
    // (I >= R)
    const bool edge = MIRROR && (ib < R || ib + kStageWarps * TX + R > a.I);  // block-uniform
    auto mirror_edges = [&](int st) {
        constexpr int CH = 64 * (int)sizeof(T) / 16;  // 16-byte chunks per tile column
        constexpr int EPC = 16 / (int)sizeof(T);
        const int g0 = ib - R;
        const int nfl = max(0, min(NC, -g0));                      // tile columns left of column 0
        const int cr0 = a.I - g0;                                  // tile column of input column I
        const int nfr = max(0, min(NC, a.I + R - g0) - cr0);       // needed columns right of I - 1
        T* tw = reinterpret_cast<T*>(smem_raw) + st * TILE;
#pragma unroll 1
        for (int q = tid; q < (nfl + nfr) * CH; q += kStageWarps * 32) {
            const int cc = q / CH, ch = q - cc * CH;
            const int c = cc < nfl ? cc : cr0 + (cc - nfl);
            const int gc = g0 + c;
            const int cs = (gc < 0 ? -1 - gc : 2 * a.I - 1 - gc) - g0;  // in-range source column
            *reinterpret_cast<int4*>(tw + c * 64 + ch * EPC) = *reinterpret_cast<const int4*>(tw + cs * 64 + ch * EPC);
        }
        // these generic writes precede the copy engine's next write of the stage
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncthreads();
    };
    for (int r0 = 0; r0 < nrp && !failed; r0 += U) {
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int r = r0 + u;
            const bool ok = mbar_wait_bounded(bbase + 8 * u, (unsigned)(((rbase + r) / kStages) & 1), a.max_polls);
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
            waited = r + 1;
            if constexpr (MIRROR)
                if (edge) mirror_edges(u);
            issue(r + kStages - 1);
            row(u, u);
        }
        if (failed) break;
        const int jin0 = jb - R + r0;
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int jo = jin0 - R + u;
            if (kv && jo >= jb && jo < je) {
                T* orow = outb + a.out.sj * (long long)jo;
#pragma unroll
                for (int q = 0; q < TX; ++q) {
                    const int i = i0 + q;
                    if (i < a.I) {
                        const float2 v = __fmul2_rn(acc[u][q], scale);
                        P2<T>::st(orow + a.out.si * (long long)i, v);
                        if (i < a.mirror_hx) P2<T>::st(orow + a.out.si * (long long)(-1 - i), v);
                        if (i >= a.I - a.mirror_hx) P2<T>::st(orow + a.out.si * (long long)(2 * a.I - 1 - i), v);
                    }
                }
            }
        }
#pragma unroll
        for (int r = 0; r < NR - U; ++r)
#pragma unroll
            for (int q = 0; q < TX; ++q) acc[r][q] = acc[r + U][q];
#pragma unroll
        for (int r = NR - U; r < NR; ++r)
#pragma unroll
            for (int q = 0; q < TX; ++q) acc[r][q] = make_float2(0.f, 0.f);
    }
    if (failed) {
        // record, then drain this block's outstanding copies (bounded) before exit
        if (tid == 0) {
            atomicExch(a.status, 1);
            const int issued = min(nrp, waited + kStages - 1);
            for (int r = waited; r < issued; ++r)
                mbar_wait_bounded(bbase + 8 * (r % kStages), (unsigned)(((rbase + r) / kStages) & 1), kDefaultWaitPolls);
        }
        __syncthreads();
    }
    return !failed;
}

// Single-row variant of the TMA kernel: one tile per block; fewer registers
// than the two-row kernel, more blocks per SM; the autotuner picks between
// them.
template <int R, int P, int TX, typename T>
__global__ void __launch_bounds__(128) k_hmom_tma1(HMomArgs a, const __grid_constant__ CUtensorMap tmap,
                                                  const __grid_constant__ HMomCoefs2 c) {
    __shared__ __align__(8) unsigned long long bars[kStages];
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const unsigned sbase = (unsigned)__cvta_generic_to_shared(smem_raw);
    const unsigned bbase = (unsigned)__cvta_generic_to_shared(bars);
    if (threadIdx.y == 0 && threadIdx.x == 0) {
#pragma unroll
        for (int s2 = 0; s2 < kStages; ++s2) mbar_init(bbase + 8 * s2, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    hmom_tma1_tile<R, P, TX, T>(a, &tmap, c, blockIdx.x * 64, blockIdx.y * (kStageWarps * TX), blockIdx.z * a.rows, sbase,
                                bbase, 0);
}

// The single-row kernel for an input without x halo (HMomArgs::mirror_in):
// edge tiles fill their half-sample mirror in shared memory.
template <int R, int P, int TX, typename T>
__global__ void __launch_bounds__(128, R <= 8 ? 4 : 1) k_hmom_tma1_mirror(HMomArgs a, const __grid_constant__ CUtensorMap tmap,
                                                                        const __grid_constant__ HMomCoefs2 c) {
    __shared__ __align__(8) unsigned long long bars[kStages];
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const unsigned sbase = (unsigned)__cvta_generic_to_shared(smem_raw);
    const unsigned bbase = (unsigned)__cvta_generic_to_shared(bars);
    if (threadIdx.y == 0 && threadIdx.x == 0) {
#pragma unroll
        for (int s2 = 0; s2 < kStages; ++s2) mbar_init(bbase + 8 * s2, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    hmom_tma1_tile<R, P, TX, T, true>(a, &tmap, c, blockIdx.x * 64, blockIdx.y * (kStageWarps * TX), blockIdx.z * a.rows,
                                      sbase, bbase, 0);
}

// Persistent form of one radial side: every generation's tiles of one
// variable group in one launch.  Blocks (as many as fit on the device at
// once) take tiles from a device counter in order -- the finest
// generation's first -- and run each with hmom_tma1_tile; the generations
// of a side are independent, so any order is correct.  The counter must be
// zero at launch.
template <int R, int P, int TX, typename T>
__global__ void __launch_bounds__(128, R <= 8 ? 4 : 3) k_hmom_persist(const __grid_constant__ HMomPersistArgs pa,
                                                     const __grid_constant__ HMomMaps maps,
                                                     const __grid_constant__ HMomCoefs2 c) {
    __shared__ __align__(8) unsigned long long bars[kStages];
    __shared__ int next_tile;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const unsigned sbase = (unsigned)__cvta_generic_to_shared(smem_raw);
    const unsigned bbase = (unsigned)__cvta_generic_to_shared(bars);
    const int tid = threadIdx.y * 32 + threadIdx.x;
    if (tid == 0) {
#pragma unroll
        for (int s2 = 0; s2 < kStages; ++s2) mbar_init(bbase + 8 * s2, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    int rbase = 0;  // rows read by this block's earlier tiles
    for (;;) {
        if (tid == 0) next_tile = atomicAdd(pa.queue, 1);
        __syncthreads();
        const int t = next_tile;
        __syncthreads();  // every thread has read next_tile before thread 0 writes it again
        if (t >= pa.ntiles) break;
        int sg = 0;
        while (sg + 1 < pa.nseg && t >= pa.seg[sg + 1].first) ++sg;
        const HMomSeg& g = pa.seg[sg];
        int lt = t - g.first;
        const int kx = lt % g.nkb;
        lt /= g.nkb;
        const int iy = lt % g.nstrip;
        const int jz = lt / g.nstrip;
        // the segment's arguments, read once per tile (a dynamic index into
        // the parameter space would reload them at every use)
        const HMomArgs a = g.a;
        const int jb = jz * a.rows;
        if (!hmom_tma1_tile<R, P, TX, T>(a, &maps.m[sg], c, kx * 64, iy * (kStageWarps * TX), jb, sbase, bbase, rbase))
            break;
        rbase += hmom_tma1_rows<R, TX>(min(jb + a.rows, a.J) - jb);
    }
}

// Columns per thread of the packed kernels.
constexpr int hmom_p2_tx(int R) { return hmom_tma_tx(R); }

template <int R, int P, typename T>
static int run_hmom(const HMomArgs& a, const HMomCoefs<double>& cd, cudaStream_t s) {
    using A = typename AccOf<T>::type;
    constexpr int TX = hmom_tx_for((int)sizeof(typename AccOf<T>::type) == 8 ? 8 : 4, R);
    constexpr int U = 2;
    constexpr int NW = 4;
    HMomCoefs<A> c;
    for (int t = 0; t < (kMaxReach + 1) * (kMaxMomP + 1); ++t) {
        c.coef[t] = (A)cd.coef[t];
        c.upow[t] = (A)cd.upow[t];
    }
    const int nstrip = (a.I + TX - 1) / TX;
    const int rows = a.rows > 0 ? a.rows : a.J;
    HMomArgs b = a;
    b.rows = rows;
    dim3 block(32, NW), grid((a.nk + 31) / 32, (nstrip + NW - 1) / NW, (a.J + rows - 1) / rows);
    // columns must start on 16-byte boundaries and 16-byte chunks must not
    // straddle the end of a column: nk * sizeof(T) % 16 == 0
    const bool staged = (a.nk * (int)sizeof(T)) % 16 == 0 && (((uintptr_t)a.in.p) & 15u) == 0 && a.halo >= R;
    if (a.mirror_in) {
        // input without x halo: only the single-row TMA kernel mirrors edge
        // tiles itself (the caller checks these conditions first); reaches
        // up to 16
        if constexpr (sizeof(A) == 4 && R <= 16) {
            if (!a.tmap || !a.status || a.nk % 2 || ((uintptr_t)a.out.p & 7u) || a.I < R || a.halo != 0)
                return (int)cudaErrorInvalidValue;
            constexpr int TX2 = hmom_p2_tx(R);
            HMomCoefs2 c2;
            for (int g = 0; g <= kMaxReach; ++g) c2.coef[g] = make_float2((float)cd.coef[g * (P + 1)], (float)cd.coef[g * (P + 1)]);
            for (int t = 0; t < (kMaxReach + 1) * (kMaxMomP + 1); ++t)
                c2.upow[t] = make_float2((float)cd.upow[t], (float)cd.upow[t]);
            const int nstrip2 = (a.I + TX2 - 1) / TX2;
            dim3 grid2((a.nk + 63) / 64, (nstrip2 + NW - 1) / NW, (a.J + rows - 1) / rows);
            constexpr size_t smt = (size_t)kStages * (kStageWarps * TX2 + 2 * R) * 64 * sizeof(T);
            if (smt + 1024 > 48 * 1024) {
                static unsigned long long done = 0;  // per instantiation
                cudaError_t ea = smem_optin(k_hmom_tma1_mirror<R, P, TX2, T>, smt, done);
                if (ea != cudaSuccess) return (int)ea;
            }
            k_hmom_tma1_mirror<R, P, TX2, T><<<grid2, block, smt, s>>>(b, *static_cast<const CUtensorMap*>(a.tmap), c2);
            cudaError_t e = cudaGetLastError();
            return e == cudaSuccess ? 0 : (int)e;
        } else {
            return (int)cudaErrorInvalidValue;
        }
    }
    if constexpr (sizeof(A) == 4) {
        // packed pairs: nk even and 16-byte aligned columns
        if (staged && a.nk % 2 == 0 && ((uintptr_t)a.out.p & 7u) == 0) {
            constexpr int TX2 = hmom_p2_tx(R);
            HMomCoefs2 c2;
            for (int g = 0; g <= kMaxReach; ++g) c2.coef[g] = make_float2((float)cd.coef[g * (P + 1)], (float)cd.coef[g * (P + 1)]);
            for (int t = 0; t < (kMaxReach + 1) * (kMaxMomP + 1); ++t)
                c2.upow[t] = make_float2((float)cd.upow[t], (float)cd.upow[t]);
            const int nstrip2 = (a.I + TX2 - 1) / TX2;
            dim3 grid2((a.nk + 63) / 64, (nstrip2 + NW - 1) / NW, (a.J + rows - 1) / rows);
            if (a.tmap && a.status && a.variant != 2) {
                static_assert(hmom_tma_tx(R) == TX2, "tile shape");
                const CUtensorMap& tm = *static_cast<const CUtensorMap*>(a.tmap);
                if (a.variant == 1) {  // single-row pipeline
                    constexpr size_t smt = (size_t)kStages * (kStageWarps * TX2 + 2 * R) * 64 * sizeof(T);
                    if (smt + 1024 > 48 * 1024) {
                        static unsigned long long done = 0;  // per instantiation
                        cudaError_t ea = smem_optin(k_hmom_tma1<R, P, TX2, T>, smt, done);
                        if (ea != cudaSuccess) return (int)ea;
                    }
                    k_hmom_tma1<R, P, TX2, T><<<grid2, block, smt, s>>>(b, tm, c2);
                } else if (a.variant == 3) {  // two rows per barrier, filtered one after the other
                    constexpr size_t smt = hmom_tma_stage_bytes<R, TX2, T>();
                    if (smt + 1024 > 48 * 1024) {
                        static unsigned long long done = 0;  // per instantiation
                        cudaError_t ea = smem_optin(k_hmom_tma<R, P, TX2, T, true>, smt, done);
                        if (ea != cudaSuccess) return (int)ea;
                    }
                    k_hmom_tma<R, P, TX2, T, true><<<grid2, block, smt, s>>>(b, tm, c2);
                } else {  // two rows per barrier, interleaved
                    constexpr size_t smt = hmom_tma_stage_bytes<R, TX2, T>();
                    // opt in above the default 48 KB (dynamic + the static mbarriers)
                    if (smt + 1024 > 48 * 1024) {
                        static unsigned long long done = 0;  // per instantiation
                        cudaError_t ea = smem_optin(k_hmom_tma<R, P, TX2, T, false>, smt, done);
                        if (ea != cudaSuccess) return (int)ea;
                    }
                    k_hmom_tma<R, P, TX2, T, false><<<grid2, block, smt, s>>>(b, tm, c2);
                }
                cudaError_t e = cudaGetLastError();
                return e == cudaSuccess ? 0 : (int)e;
            }
            constexpr size_t sm2 = hmom_p2_stage_bytes<R, TX2, T>();
            if (sm2 + 1024 > 48 * 1024) {
                static unsigned long long done = 0;  // per instantiation
                cudaError_t ea = smem_optin(k_hmom_p2<R, P, TX2, T>, sm2, done);
                if (ea != cudaSuccess) return (int)ea;
            }
            k_hmom_p2<R, P, TX2, T><<<grid2, block, sm2, s>>>(b, c2);
            cudaError_t e = cudaGetLastError();
            return e == cudaSuccess ? 0 : (int)e;
        }
    }
    if (staged) {
        static_assert(NW == kStageWarps, "block shape");
        constexpr size_t sm = hmom_stage_bytes<R, TX, T>();
        if (sm + 1024 > 48 * 1024) {
            static unsigned long long done = 0;  // per instantiation
            cudaError_t ea = smem_optin(k_hmom_st<R, P, TX, T>, sm, done);
            if (ea != cudaSuccess) return (int)ea;
        }
        k_hmom_st<R, P, TX, T><<<grid, block, sm, s>>>(b, c);
    } else {
        k_hmom<R, P, TX, U, T><<<grid, block, 0, s>>>(b, c);
    }
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : (int)e;
}

template <int R, int P, typename T>
static int run_hmom_persist(HMomPersistArgs pa, const HMomMaps& maps, const HMomCoefs<double>& cd, cudaStream_t s) {
    if constexpr (sizeof(T) == 8) {
        return -1;
    } else {
        constexpr int TX2 = hmom_p2_tx(R);
        if (pa.nseg <= 0 || pa.nseg > kMaxPersistSegs || !pa.queue) return -1;
        int ntiles = 0;
        for (int i = 0; i < pa.nseg; ++i) {
            HMomSeg& g = pa.seg[i];
            const HMomArgs& a = g.a;
            // the packed TMA pipeline's conditions (as run_hmom)
            if (!a.status || a.rows <= 0 || a.nk % 2 || (a.nk * (int)sizeof(T)) % 16 || a.halo < R ||
                ((uintptr_t)a.in.p & 15u) || ((uintptr_t)a.out.p & 7u))
                return -1;
            g.nkb = (a.nk + 63) / 64;
            g.nstrip = ((a.I + TX2 - 1) / TX2 + kStageWarps - 1) / kStageWarps;
            g.nrowb = (a.J + a.rows - 1) / a.rows;
            g.first = ntiles;
            ntiles += g.nkb * g.nstrip * g.nrowb;
        }
        pa.ntiles = ntiles;
        if (ntiles == 0) return 0;
        HMomCoefs2 c2;
        for (int g = 0; g <= kMaxReach; ++g) c2.coef[g] = make_float2((float)cd.coef[g * (P + 1)], (float)cd.coef[g * (P + 1)]);
        for (int t = 0; t < (kMaxReach + 1) * (kMaxMomP + 1); ++t) c2.upow[t] = make_float2((float)cd.upow[t], (float)cd.upow[t]);
        constexpr size_t smt = (size_t)kStages * (kStageWarps * TX2 + 2 * R) * 64 * sizeof(T);
        static unsigned long long done = 0;  // per instantiation
        if (smt + 1024 > 48 * 1024) {
            cudaError_t ea = smem_optin(k_hmom_persist<R, P, TX2, T>, smt, done);
            if (ea != cudaSuccess) return (int)ea;
        }
        // blocks_per_sm per SM, at most as many as fit on the device at once
        int per_sm = 0;
        cudaError_t eo = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_hmom_persist<R, P, TX2, T>,
                                                                     32 * kStageWarps, smt);
        if (eo != cudaSuccess) return (int)eo;
        per_sm = std::max(per_sm, 1);
        if (pa.blocks_per_sm > 0) per_sm = std::min(per_sm, pa.blocks_per_sm);
        const int grid = std::max(1, std::min(ntiles, per_sm * device_sm_count()));
        cudaError_t em = cudaMemsetAsync(pa.queue, 0, sizeof(int), s);
        if (em != cudaSuccess) return (int)em;
        k_hmom_persist<R, P, TX2, T><<<grid, dim3(32, kStageWarps), smt, s>>>(pa, maps, c2);
        cudaError_t e = cudaGetLastError();
        return e == cudaSuccess ? 0 : (int)e;
    }
}

}  // namespace mgbf
