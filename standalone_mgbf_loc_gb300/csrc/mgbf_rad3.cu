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
    dispatch(t, [&](auto tag) {
        using T = decltype(tag);
        k_ball<T><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(a);
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
