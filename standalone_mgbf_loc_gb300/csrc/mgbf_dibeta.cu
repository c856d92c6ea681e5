// filtering_lin2_bckg (procedure 2, mg_filtering.f90:683-822): one color of
// its line filters on a generation.  The filter is the "dibeta" of
// jp_pbfil3.f90 (vdibeta2 :1801-1837, vdibeta2t :2345-2382): symmetric
// weights fil[0..h] along the integer generator d = (dx, dy),
//   forward  b(x) = fil0 a(x) + sum_{t=1..h} fil_t (a(x + t d) + a(x - t d))
// on the interior, after boco_2d's half-sample mirror fill (here an index
// reflection per axis), and
//   adjoint  the scatter of the same weights from every interior point,
// followed by bocoT_2d, which adds each halo cell into its mirror image
// (x on all rows, then y on the interior columns).  As a gather: target s
// collects, for every extended point q that folds onto s (s itself and its
// mirror images within the fold widths), every interior source q - t d.
//
// Thread = V consecutive levels of one point, consecutive threads on
// consecutive levels (coalesced loads of every tap).
#include <cuda_runtime.h>

#include "mgbf_common.cuh"
#include "mgbf_kernels.cuh"

namespace mgbf {

namespace {

template <typename A> __device__ __forceinline__ A dib_w(const DibArgs& a, int t);
template <> __device__ __forceinline__ float dib_w<float>(const DibArgs& a, int t) { return a.filf[t]; }
template <> __device__ __forceinline__ double dib_w<double>(const DibArgs& a, int t) { return a.fil[t]; }
template <typename A> __device__ __forceinline__ A dib_scale(const DibArgs& a);
template <> __device__ __forceinline__ float dib_scale<float>(const DibArgs& a) { return a.scalef; }
template <> __device__ __forceinline__ double dib_scale<double>(const DibArgs& a) { return a.scale; }

template <typename T, int V> struct Ld;
template <typename T> struct Ld<T, 4> {
    using A = typename AccOf<T>::type;
    static __device__ __forceinline__ void ld(const T* p, A (&v)[4]) { V4<T>::ld(p, v); }
    static __device__ __forceinline__ void st(T* p, const A (&v)[4]) { V4<T>::st(p, v); }
};
template <typename T> struct Ld<T, 1> {
    using A = typename AccOf<T>::type;
    static __device__ __forceinline__ void ld(const T* p, A (&v)[1]) { v[0] = ldv(p); }
    static __device__ __forceinline__ void st(T* p, const A (&v)[1]) { stv(p, v[0]); }
};

template <typename T, int V>
__global__ void __launch_bounds__(128) k_dibeta(DibArgs a) {
    using A = typename AccOf<T>::type;
    const int nq = a.nk / V;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)nq * a.I * a.J) return;
    const int k = V * (int)(idx % nq);
    const long long r = idx / nq;
    const int i = (int)(r % a.I), j = (int)(r / a.I);
    const T* in = static_cast<const T*>(a.in.p) + k;
    A acc[V], v[V], u[V];
    if (!a.adjoint) {
        Ld<T, V>::ld(in + a.in.si * i + a.in.sj * j, v);
        const A f0 = dib_w<A>(a, 0);
#pragma unroll
        for (int e = 0; e < V; ++e) acc[e] = f0 * v[e];
        for (int t = 1; t <= a.h; ++t) {
            Ld<T, V>::ld(in + a.in.si * reflect_half(i + t * a.dx, a.I) + a.in.sj * reflect_half(j + t * a.dy, a.J), u);
            Ld<T, V>::ld(in + a.in.si * reflect_half(i - t * a.dx, a.I) + a.in.sj * reflect_half(j - t * a.dy, a.J), v);
            const A f = dib_w<A>(a, t);
#pragma unroll
            for (int e = 0; e < V; ++e) acc[e] = fma(f, u[e] + v[e], acc[e]);
        }
    } else {
#pragma unroll
        for (int e = 0; e < V; ++e) acc[e] = A(0);
        // extended points folding onto (i, j): itself, and its mirror in each
        // halo band it lies within (both bands when the grid is narrower
        // than twice the fold width)
        int qx[3], qy[3], nx = 0, ny = 0;
        qx[nx++] = i;
        if (i < a.hx) qx[nx++] = -1 - i;
        if (i >= a.I - a.hx) qx[nx++] = 2 * a.I - 1 - i;
        qy[ny++] = j;
        if (j < a.hy) qy[ny++] = -1 - j;
        if (j >= a.J - a.hy) qy[ny++] = 2 * a.J - 1 - j;
        for (int bx = 0; bx < nx; ++bx)
            for (int by = 0; by < ny; ++by)
                for (int t = -a.h; t <= a.h; ++t) {
                    const int sx = qx[bx] - t * a.dx, sy = qy[by] - t * a.dy;
                    if (sx < 0 || sx >= a.I || sy < 0 || sy >= a.J) continue;  // scatter sources are interior
                    Ld<T, V>::ld(in + a.in.si * sx + a.in.sj * sy, v);
                    const A f = dib_w<A>(a, t < 0 ? -t : t);
#pragma unroll
                    for (int e = 0; e < V; ++e) acc[e] = fma(f, v[e], acc[e]);
                }
    }
    const A sc = dib_scale<A>(a);
#pragma unroll
    for (int e = 0; e < V; ++e) acc[e] *= sc;
    Ld<T, V>::st(static_cast<T*>(a.out.p) + k + a.out.si * i + a.out.sj * j, acc);
}

inline bool al16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

template <typename F>
void dispatch(DType t, F&& f) {
    switch (t) {
        case DType::F64: f(double()); break;
        case DType::F32: f(float()); break;
        case DType::BF16: f(__nv_bfloat16()); break;
    }
}

}  // namespace

int launch_dibeta(DType t, const DibArgs& args, void* stream) {
    if (args.nk == 0 || args.I == 0 || args.J == 0) return 0;
    if (args.h < 0 || args.h > 8) return (int)cudaErrorInvalidValue;
    DibArgs a = args;
    for (int q = 0; q < 9; ++q) a.filf[q] = (float)a.fil[q];  // no FP64 conversion in the threads
    a.scalef = (float)a.scale;
    const size_t es = t == DType::F64 ? 8 : (t == DType::F32 ? 4 : 2);
    const bool vec = a.nk % 4 == 0 && al16(a.in.p) && al16(a.out.p) && (a.in.si * es) % 16 == 0 &&
                     (a.in.sj * es) % 16 == 0 && (a.out.si * es) % 16 == 0 && (a.out.sj * es) % 16 == 0 &&
                     !(t == DType::BF16 && a.nk % 8);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const long long n = (long long)(vec ? a.nk / 4 : a.nk) * a.I * a.J;
    const unsigned grid = (unsigned)((n + 127) / 128);
    dispatch(t, [&](auto tag) {
        using T = decltype(tag);
        if (vec) k_dibeta<T, 4><<<grid, 128, 0, s>>>(a);
        else k_dibeta<T, 1><<<grid, 128, 0, s>>>(a);
    });
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : (int)e;
}

}  // namespace mgbf
