// filtering_rad3 (procedure 4, mg_filtering.f90:123-257): the 3D radial
// beta filter vrbeta3 (jp_pbfil.f90:930-977) on the 3D variables, as a
// direct sum over its ball of taps (the ball is small: reach <= hz < lm).
//
// Level index L of a 3D variable's column (lm levels, k = v*lm + L) has the
// whole-sample mirror of sup_vrbeta3 (mg_filtering.f90:1923-1980); x and y
// have the half-sample mirror of boco_2d, an index reflection.
// The adjoint side follows the reference's sup_vrbeta3T
// (mg_filtering.f90:1983-2039): the scatter from the interior is folded in
// L and only its x/y interior is kept; bocoT_2d then folds whatever halo the
// generation held, which at generation 1 is the caller's VALL halo.  As a
// gather: target (L, i, j) takes w(g) * x(Ls, i - gx, j - gy) for every tap g
// and every source level Ls whose scatter target Ls + gz folds onto L, with
// sources outside the x/y interior contributing nothing.
#include <cuda_runtime.h>

#include <climits>

#include "mgbf_common.cuh"
#include "mgbf_kernels.cuh"

namespace mgbf {

namespace {

template <typename A> __device__ __forceinline__ A ball_scale(const BallArgs& a);
template <> __device__ __forceinline__ float ball_scale<float>(const BallArgs& a) { return a.scalef; }
template <> __device__ __forceinline__ double ball_scale<double>(const BallArgs& a) { return a.scale; }

// whole-sample mirror of a 0-based level into [0, lm)
__device__ __forceinline__ int mirror_whole(int L, int lm) {
    if (L < 0) L = -L;
    if (L >= lm) L = 2 * (lm - 1) - L;
    return L;
}

template <typename T>
__global__ void __launch_bounds__(128) k_ball(BallArgs a) {
    using A = typename AccOf<T>::type;
    const int n3 = a.ncol * a.lm;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)n3 * a.I * a.J) return;
    const int k = (int)(idx % n3);
    const long long r = idx / n3;
    const int i = (int)(r % a.I), j = (int)(r / a.I);
    const int L = k % a.lm, base = k - L;
    const T* in = static_cast<const T*>(a.in.p) + base;
    const A* w = static_cast<const A*>(a.w);
    A acc = A(0);
    if (!a.adjoint) {
        for (int e = 0; e < a.ntaps; ++e) {
            const int4 g = a.taps[e];
            const int ii = reflect_half(i + g.x, a.I), jj = reflect_half(j + g.y, a.J);
            acc = fma(w[e], ldv(in + a.in.si * ii + a.in.sj * jj + mirror_whole(L + g.z, a.lm)), acc);
        }
    } else {
        const int top = 2 * (a.lm - 1);
        for (int e = 0; e < a.ntaps; ++e) {
            const int4 g = a.taps[e];
            const int is = i - g.x, js = j - g.y;
            if (is < 0 || is >= a.I || js < 0 || js >= a.J) continue;  // scatter source outside the interior
            const T* col = in + a.in.si * is + a.in.sj * js;
            // sources whose target Ls + gz lands on L directly, or folds onto it
            // from below (target -L) or from above (target 2(lm-1) - L)
            A s = A(0);
            int Ls = L - g.z;
            if (Ls >= 0 && Ls < a.lm) s += ldv(col + Ls);
            if (L >= 1) {
                Ls = -L - g.z;
                if (Ls >= 0 && Ls < a.lm) s += ldv(col + Ls);
            }
            if (L <= a.lm - 2) {
                Ls = top - L - g.z;
                if (Ls >= 0 && Ls < a.lm) s += ldv(col + Ls);
            }
            acc = fma(w[e], s, acc);
        }
        if (a.has_prev) {
            // bocoT_2d of the generation's previous halo (width hx, hy): x on
            // every row, then y on the interior columns
            const T* h = static_cast<const T*>(a.prev.p) + k;
            const int px = i < a.hx ? -1 - i : (i >= a.I - a.hx ? 2 * a.I - 1 - i : INT_MIN);
            const int py = j < a.hy ? -1 - j : (j >= a.J - a.hy ? 2 * a.J - 1 - j : INT_MIN);
            if (px != INT_MIN) acc += ldv(h + a.prev.si * px + a.prev.sj * j);
            if (py != INT_MIN) acc += ldv(h + a.prev.si * i + a.prev.sj * py);
            if (px != INT_MIN && py != INT_MIN) acc += ldv(h + a.prev.si * px + a.prev.sj * py);
        }
    }
    stv(static_cast<T*>(a.out.p) + a.out.si * i + a.out.sj * j + k, acc * ball_scale<A>(a));
}

// The same sums in rows along x.  A thread owns LC consecutive x positions
// of one level (consecutive threads: consecutive levels, so every load of a
// warp is one contiguous run).  For each row (gy, gz) of the ball it loads
// the LC + 2R column window of that row once and applies the row's 2R+1 gx
// weights from registers.  The rows keep the taps' order and the weights a
// row lacks are zero (fma(0, x, acc) == acc), so the result is bit-identical
// to k_ball's.
template <typename T, int R, int LC>
__global__ void __launch_bounds__(128) k_ball_rows(BallArgs a) {
    using A = typename AccOf<T>::type;
    constexpr int W = LC + 2 * R, NW = 2 * R + 1;
    const int n3 = a.ncol * a.lm;
    const int nch = (a.I + LC - 1) / LC;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)n3 * nch * a.J) return;
    const int k = (int)(idx % n3);
    const long long r = idx / n3;
    const int i0 = (int)(r % nch) * LC, j = (int)(r / nch);
    const int L = k % a.lm, base = k - L;
    const T* in = static_cast<const T*>(a.in.p) + base;
    const A* rw = static_cast<const A*>(a.rw);
    // column offsets of the window: source x = i0 - R + m; for the adjoint a
    // source outside the interior contributes nothing
    // (32-bit: the launcher checks that si * I fits)
    int xo[W];
#pragma unroll
    for (int m = 0; m < W; ++m) xo[m] = (int)a.in.si * reflect_half(i0 - R + m, a.I);
    auto xv = [&](int m) { return (unsigned)(i0 - R + m) < (unsigned)a.I; };
    A acc[LC];
#pragma unroll
    for (int l = 0; l < LC; ++l) acc[l] = A(0);
    const int top = 2 * (a.lm - 1);
    // adjoint: every source of the window lies in the x interior (uniform
    // over a warp whenever a chunk holds at least 32 levels)
    const bool xin = i0 - R >= 0 && i0 + LC + R <= a.I;
    for (int t = 0; t < a.nrows; ++t) {
        const int2 row = a.rows[t];  // (gy, gz)
        A wl[NW];
#pragma unroll
        for (int d = 0; d < NW; ++d) wl[d] = rw[t * NW + d];
        A win[W];
        if (!a.adjoint) {
            const T* src = in + a.in.sj * reflect_half(j + row.x, a.J) + mirror_whole(L + row.y, a.lm);
#pragma unroll
            for (int m = 0; m < W; ++m) win[m] = ldv(src + xo[m]);
            // target i0 + l reads x = i0 + l + gx: window index l + gx + R
#pragma unroll
            for (int l = 0; l < LC; ++l)
#pragma unroll
                for (int d = 0; d < NW; ++d) acc[l] = fma(wl[d], win[l + d], acc[l]);
        } else {
            const int js = j - row.x;
            if (js < 0 || js >= a.J) continue;  // the whole row's sources lie outside the interior
            const T* src = in + a.in.sj * js;
            // source levels whose target Ls + gz lands on L directly or folds onto it
            const int l1 = L - row.y, l2 = -L - row.y, l3 = top - L - row.y;
            const bool v1 = l1 >= 0 && l1 < a.lm;
            const bool v2 = L >= 1 && l2 >= 0 && l2 < a.lm;
            const bool v3 = L <= a.lm - 2 && l3 >= 0 && l3 < a.lm;
            // direct pre-image, predicated per lane (0 + x == x, so the sum
            // below keeps k_ball's order: direct, then fold from below, then above)
            if (xin) {
#pragma unroll
                for (int m = 0; m < W; ++m) win[m] = v1 ? ldv(src + xo[m] + l1) : A(0);
            } else {
#pragma unroll
                for (int m = 0; m < W; ++m) win[m] = (v1 && xv(m)) ? ldv(src + xo[m] + l1) : A(0);
            }
            // folded pre-images: only lanes within R of a column end, on rows
            // whose gz points out of the column
            if (v2 || v3) {
#pragma unroll
                for (int m = 0; m < W; ++m) {
                    if (xv(m)) {
                        const T* c = src + xo[m];
                        if (v2) win[m] += ldv(c + l2);
                        if (v3) win[m] += ldv(c + l3);
                    }
                }
            }
            // target i0 + l takes x = i0 + l - gx: window index l - gx + R
#pragma unroll
            for (int l = 0; l < LC; ++l)
#pragma unroll
                for (int d = 0; d < NW; ++d) acc[l] = fma(wl[d], win[l + 2 * R - d], acc[l]);
        }
    }
    const A sc = ball_scale<A>(a);
#pragma unroll
    for (int l = 0; l < LC; ++l) {
        const int i = i0 + l;
        if (i >= a.I) break;
        A v = acc[l];
        if (a.adjoint && a.has_prev) {
            const T* h = static_cast<const T*>(a.prev.p) + k;
            const int px = i < a.hx ? -1 - i : (i >= a.I - a.hx ? 2 * a.I - 1 - i : INT_MIN);
            const int py = j < a.hy ? -1 - j : (j >= a.J - a.hy ? 2 * a.J - 1 - j : INT_MIN);
            if (px != INT_MIN) v += ldv(h + a.prev.si * px + a.prev.sj * j);
            if (py != INT_MIN) v += ldv(h + a.prev.si * i + a.prev.sj * py);
            if (px != INT_MIN && py != INT_MIN) v += ldv(h + a.prev.si * px + a.prev.sj * py);
        }
        stv(static_cast<T*>(a.out.p) + a.out.si * i + a.out.sj * j + k, v * sc);
    }
}

// VALL's halo after procedure 4: the 3D variables keep boco_2d's mirror fill
// of the field the ball forward pass read, the 2D variables hold zero.
template <typename T>
__global__ void __launch_bounds__(256) k_rad3_halo(View out, View src, int nk, int n3, int I, int J, int hx, int hy) {
    const int ni = I + 2 * hx;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)nk * ni) return;
    const int i = (int)(idx / nk) - hx;
    const int k = (int)(idx - (long long)(i + hx) * nk);
    const int j = (int)blockIdx.y - hy;
    if (i >= 0 && i < I && j >= 0 && j < J) return;
    T v = T(0);
    if (k < n3) v = static_cast<const T*>(src.p)[src.si * reflect_half(i, I) + src.sj * reflect_half(j, J) + k];
    static_cast<T*>(out.p)[out.sj * j + out.si * i + k] = v;
}

template <typename F>
void dispatch(DType t, F&& f) {
    switch (t) {
        case DType::F64: f(double()); break;
        case DType::F32: f(float()); break;
        case DType::BF16: f(__nv_bfloat16()); break;
    }
}

}  // namespace

int launch_ball(DType t, const BallArgs& args, void* stream) {
    const long long n = (long long)args.ncol * args.lm * args.I * args.J;
    if (n == 0) return 0;
    BallArgs a = args;
    a.scalef = (float)a.scale;  // no FP64 conversion in the threads
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    constexpr int LC = 16;  // x positions per thread (16 measured faster than 8 in every type)
    const long long nr = (long long)args.ncol * args.lm * ((args.I + LC - 1) / LC) * args.J;
    const unsigned gr = (unsigned)((nr + 127) / 128);
    dispatch(t, [&](auto tag) {
        using T = decltype(tag);
        if (a.rows == nullptr || a.nrows <= 0 || a.in.si * a.I >= INT_MAX) a.R = 0;
        switch (a.R) {
            case 1: k_ball_rows<T, 1, LC><<<gr, 128, 0, s>>>(a); break;
            case 2: k_ball_rows<T, 2, LC><<<gr, 128, 0, s>>>(a); break;
            case 3: k_ball_rows<T, 3, LC><<<gr, 128, 0, s>>>(a); break;
            case 4: k_ball_rows<T, 4, LC><<<gr, 128, 0, s>>>(a); break;
            default: k_ball<T><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(a); break;
        }
    });
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : (int)e;
}

int launch_rad3_halo(DType t, View out, View src, int nk, int n3, int I, int J, int hx, int hy, void* stream) {
    const long long n = (long long)nk * (I + 2 * hx);
    if (n == 0 || (hx == 0 && hy == 0)) return 0;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    dim3 grid((unsigned)((n + 255) / 256), J + 2 * hy);
    dispatch(t, [&](auto tag) {
        using T = decltype(tag);
        k_rad3_halo<T><<<grid, 256, 0, s>>>(out, src, nk, n3, I, J, hx, hy);
    });
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : (int)e;
}

}  // namespace mgbf
