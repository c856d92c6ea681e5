// Radial beta filter, moment form (sm_103a).
//
// The reference's normalised radial beta weight (vrbeta2, jp_pbfil.f90:888-928)
// is w(gx,gy) = s*(1 - e^2 gy^2 - e^2 gx^2)^p on a disk whose row half-widths
// are m(gy).  For a fixed row gy it is a polynomial of degree p in
// u = (e gx)^2:  w = s * sum_q C(p,q) (-1)^q A(gy)^(p-q) u^q,  A = 1 - (e gy)^2.
// So the row sum  sum_{|gx|<=m(gy)} w a(i+gx)  equals
//   sum_q c_q(gy) T_q^{m(gy)}(i),   T_q^m(i) = sum_{|gx|<=m} (e gx)^(2q) a(i+gx),
// and T_q^m grows from T_q^{m-1} by (e m)^(2q) (a(i+m)+a(i-m)).  One pass over
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

#include <cuda_runtime.h>

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
                        A v = c.coef[gy * PQ] * t[0];
#pragma unroll
                        for (int e = 1; e < PQ; ++e) v = fma(c.coef[gy * PQ + e], t[e], v);
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
    k_hmom<R, P, TX, U, T><<<grid, block, 0, s>>>(b, c);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : (int)e;
}

}  // namespace mgbf
