// Transfers between the analysis grid and the first filter generation
// (anal_to_filt_all2 / filt_to_anal_all2, mg_transfer.f90:154-203, 339-464).
//
// Direct (filter -> analysis): each analysis point gathers the separable
// 2/3/4-tap offset interpolation (lin/quad/lsqr_direct_offset,
// mg_interpolate.f90:634-681, 750-795, 858-903) from the filter field, with
// the half-sample mirror of boco_2d as an index reflection.
// Adjoint (analysis -> filter): the reference scatters (..._adjoint_offset,
// mg_interpolate.f90:684-747, 798-855, 906-960); here every target gathers
// its sources from host-built lists, first along y into an intermediate on
// the analysis x-grid, then along x into the extended filter array, so no
// two threads write one element.  bocoT_2d's fold then runs on the halo
// bands only.
// Vertical (lm_a = 2 lm - 1): l_vertical_direct/adjoint_spec2
// (mg_interpolate.f90:963-1044) per point and block of levels.
#include <cuda_runtime.h>

#include <type_traits>

#include "mgbf_common.cuh"
#include "mgbf_kernels.cuh"

namespace mgbf {

namespace {

// V levels per thread: 4 (vector loads) or 1.
template <typename T, int V> struct Lv;
template <typename T> struct Lv<T, 4> {
    using A = typename AccOf<T>::type;
    static __device__ __forceinline__ void ld(const T* p, A (&v)[4]) { V4<T>::ld(p, v); }
    static __device__ __forceinline__ void st(T* p, const A (&v)[4]) { V4<T>::st(p, v); }
};
template <typename T> struct Lv<T, 1> {
    using A = typename AccOf<T>::type;
    static __device__ __forceinline__ void ld(const T* p, A (&v)[1]) { v[0] = ldv(p); }
    static __device__ __forceinline__ void st(T* p, const A (&v)[1]) { stv(p, v[0]); }
};

// Flat thread index -> (level group q, point a, point b), q fastest.
struct Pos3 {
    int q, a, b;
    bool ok;
};
__device__ __forceinline__ Pos3 pos3(int nq, int na, int nb) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    Pos3 r;
    r.q = (int)(idx % nq);
    const long long rest = idx / nq;
    r.a = (int)(rest % na);
    r.b = (int)(rest / na);
    r.ok = r.b < nb;
    return r;
}

// W(k, N, M) = sum_s cy_s(M) sum_t cx_t(N) V(k, reflect(rx(N)+t), reflect(ry(M)+s))
template <typename T, int V, int ORDER>
__global__ void __launch_bounds__(128) k_xfer_direct(XferDirectArgs a) {
    using A = typename AccOf<T>::type;
    const Pos3 p = pos3(a.nk / V, a.nm0, a.mm0);
    if (!p.ok) return;
    const int k = V * p.q;
    constexpr int nt = ORDER + 1;
    const int rx = a.rx[p.a], ry = a.ry[p.b];
    const A* cx = static_cast<const A*>(a.cx) + 4 * p.a;
    const A* cy = static_cast<const A*>(a.cy) + 4 * p.b;
    const T* in = static_cast<const T*>(a.in.p) + k;
    A acc[V], vx[V], v[V];
#pragma unroll
    for (int s = 0; s < nt; ++s) {
        const T* row = in + a.in.sj * reflect_half(ry + s, a.J);
#pragma unroll
        for (int e = 0; e < V; ++e) vx[e] = A(0);
#pragma unroll
        for (int t = 0; t < nt; ++t) {
            Lv<T, V>::ld(row + a.in.si * reflect_half(rx + t, a.I), v);
            const A c = cx[t];
#pragma unroll
            for (int e = 0; e < V; ++e) vx[e] = t ? fma(c, v[e], vx[e]) : c * v[e];
        }
        const A c = cy[s];
#pragma unroll
        for (int e = 0; e < V; ++e) acc[e] = s ? fma(c, vx[e], acc[e]) : c * vx[e];
    }
    Lv<T, V>::st(static_cast<T*>(a.out.p) + k + a.out.si * p.a + a.out.sj * p.b, acc);
}

// Strip form of the direct interpolation: a thread owns V = 4 levels of one
// analysis column N and TM consecutive analysis rows.  The filter rows those
// rows need (first taps ry(M) are nondecreasing in M) are x-interpolated
// once each into the thread's own slice of shared memory, then every output
// row reads its order+1 of them by index.  Loads per output drop from
// (order+1)^2 to about (order+1) * (filter rows per analysis row +
// (order+1)/TM).  No thread reads another's slice: no barrier is needed.
template <typename T, int V, int ORDER, int TM, int NRMAX>
__global__ void __launch_bounds__(128) k_xfer_direct_strip(XferDirectArgs a) {
    using A = typename AccOf<T>::type;
    static_assert(V == 4 && std::is_same<A, float>::value, "strip form: 4 float accumulators per thread");
    constexpr int nt = ORDER + 1;
    extern __shared__ float4 sx[];  // x-interpolated filter rows, [row][thread]: max_strip_rows x 128
    const int nstrip = (a.mm0 + TM - 1) / TM;
    const Pos3 p = pos3(a.nk / V, a.nm0, nstrip);
    if (!p.ok) return;
    const int k = V * p.q;
    const int M0 = p.b * TM, M1 = min(M0 + TM, a.mm0);
    const int j_lo = a.ry[M0];
    const int rx = a.rx[p.a];
    const A* cx = static_cast<const A*>(a.cx) + 4 * p.a;
    const T* in = static_cast<const T*>(a.in.p) + k;
    int coff[nt];
#pragma unroll
    for (int t = 0; t < nt; ++t) coff[t] = reflect_half(rx + t, a.I);
    A c[nt];
#pragma unroll
    for (int t = 0; t < nt; ++t) c[t] = cx[t];
    const int nr = a.ry[M1 - 1] + nt - j_lo;  // filter rows of the strip (<= NRMAX, checked by the launcher)
    float4* mine = sx + threadIdx.x;
#pragma unroll 2
    for (int r = 0; r < nr; ++r) {
        const T* row = in + a.in.sj * reflect_half(j_lo + r, a.J);
        A v[V], vx[V];
#pragma unroll
        for (int t = 0; t < nt; ++t) {
            Lv<T, V>::ld(row + a.in.si * coff[t], v);
#pragma unroll
            for (int e = 0; e < V; ++e) vx[e] = t ? fma(c[t], v[e], vx[e]) : c[t] * v[e];
        }
        mine[r * 128] = make_float4(vx[0], vx[1], vx[2], vx[3]);
    }
    T* outp = static_cast<T*>(a.out.p) + k + a.out.si * p.a;
    for (int M = M0; M < M1; ++M) {
        const float4* rows = mine + (a.ry[M] - j_lo) * 128;
        const A* cy = static_cast<const A*>(a.cy) + 4 * M;
        A acc[V];
#pragma unroll
        for (int e = 0; e < V; ++e) acc[e] = A(0);
#pragma unroll
        for (int s = 0; s < nt; ++s) {
            const float4 f = rows[s * 128];
            const A w = cy[s];
            acc[0] = fma(w, f.x, acc[0]);
            acc[1] = fma(w, f.y, acc[1]);
            acc[2] = fma(w, f.z, acc[2]);
            acc[3] = fma(w, f.w, acc[3]);
        }
        Lv<T, V>::st(outp + a.out.sj * M, acc);
    }
}

// out(k, a, b) = sum over the list of target `lt` of w * in(k, src, b) (dir 0:
// list over the first point index, sources along `in.si`) or
// sum w * in(k, a, src) (dir 1: sources along `in.sj`).  Targets with an
// empty list give 0.
template <typename T, int V>
__global__ void __launch_bounds__(128) k_xfer_gather(XferGatherArgs a) {
    using A = typename AccOf<T>::type;
    const Pos3 p = pos3(a.nk / V, a.na, a.nb);
    if (!p.ok) return;
    const int k = V * p.q;
    const int lt = a.dir ? p.b : p.a;
    const int o0 = a.off[lt], o1 = a.off[lt + 1];
    const A* w = static_cast<const A*>(a.w);
    const T* in = static_cast<const T*>(a.in.p) + k + (a.dir ? a.in.si * p.a : a.in.sj * p.b);
    const long long ls = a.dir ? a.in.sj : a.in.si;
    A acc[V], v[V];
#pragma unroll
    for (int e = 0; e < V; ++e) acc[e] = A(0);
    for (int o = o0; o < o1; ++o) {
        Lv<T, V>::ld(in + ls * a.src[o], v);
        const A c = w[o];
#pragma unroll
        for (int e = 0; e < V; ++e) acc[e] = fma(c, v[e], acc[e]);
    }
    Lv<T, V>::st(static_cast<T*>(a.out.p) + k + a.out.si * (p.a - a.out_a0) + a.out.sj * (p.b - a.out_b0), acc);
}

// Both adjoint gathers of anal_to_filt in one pass.  Block: filter row b
// (blockIdx.y), target columns [tile*ta, tile*ta + ta) (blockIdx.x), level
// lanes [grp*lanes, ...) (blockIdx.z).  Phase 1 y-gathers the analysis
// columns the tile's x lists touch into shared memory (what the separate y
// gather writes to the intermediate, kept in FP32); phase 2 x-gathers each
// target from there.  Both sums run in list order, as the separate gathers'.
template <typename T>
__global__ void __launch_bounds__(256) k_xfer_a2f_fused(XferFusedArgs a) {
    extern __shared__ float4 vs[];  // [column - c0][lane]
    const int tile = blockIdx.x, b = blockIdx.y;
    const int l0 = blockIdx.z * a.lanes;
    const int nlg = min(a.lanes, a.nk / 4 - l0);
    if (nlg <= 0) return;  // uniform over the block
    const int c0 = a.tile_c0[tile], nc = a.tile_nc[tile];
    const int oy0 = a.offy[b], oy1 = a.offy[b + 1];
    const float* wy = static_cast<const float*>(a.wy);
    const T* W = static_cast<const T*>(a.in.p) + 4 * l0;
    for (int p = threadIdx.x; p < nc * nlg; p += blockDim.x) {
        const int e = p % nlg, c = p / nlg;
        const T* col = W + 4 * e + a.in.si * (c0 + c);
        float acc[4] = {0.f, 0.f, 0.f, 0.f}, v[4];
        for (int o = oy0; o < oy1; ++o) {
            V4<T>::ld(col + a.in.sj * a.srcy[o], v);
            const float w = wy[o];
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[q] = fma(w, v[q], acc[q]);
        }
        vs[c * nlg + e] = make_float4(acc[0], acc[1], acc[2], acc[3]);
    }
    __syncthreads();
    const int a0 = tile * a.ta, a1 = min(a0 + a.ta, a.IE);
    const float* wx = static_cast<const float*>(a.wx);
    T* out = static_cast<T*>(a.out.p) + 4 * l0 + a.out.sj * (b - a.ib);
    for (int p = threadIdx.x; p < (a1 - a0) * nlg; p += blockDim.x) {
        const int e = p % nlg, t = a0 + p / nlg;
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        for (int o = a.offx[t]; o < a.offx[t + 1]; ++o) {
            const float4 f = vs[(a.srcx[o] - c0) * nlg + e];
            const float w = wx[o];
            acc[0] = fma(w, f.x, acc[0]);
            acc[1] = fma(w, f.y, acc[1]);
            acc[2] = fma(w, f.z, acc[2]);
            acc[3] = fma(w, f.w, acc[3]);
        }
        V4<T>::st(out + 4 * e + a.out.si * (t - a.ib), acc);
    }
}

// bocoT_2d on the halo band b of an extended array whose view origin is the
// first interior point: x first on every row of the band's range, then y
// on the interior columns.  One thread per (level, row or column, t).
template <typename T>
__global__ void __launch_bounds__(256) k_fold_x(View v, int nk, int I, int J, int b) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = (long long)nk * b * (J + 2 * b);
    if (idx >= n) return;
    const int k = (int)(idx % nk);
    const long long r = idx / nk;
    const int t = (int)(r % b);
    const int j = (int)(r / b) - b;
    T* row = static_cast<T*>(v.p) + k + v.sj * j;
    // west: W(t) += W(1-t); east: W(I-b+t) += W(I+b+1-t)  (1-based, t = 1..b)
    stv(row + v.si * t, ldv(row + v.si * t) + ldv(row + v.si * (-1 - t)));
    stv(row + v.si * (I - 1 - t), ldv(row + v.si * (I - 1 - t)) + ldv(row + v.si * (I + t)));
}
template <typename T>
__global__ void __launch_bounds__(256) k_fold_y(View v, int nk, int I, int J, int b) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = (long long)nk * b * I;
    if (idx >= n) return;
    const int k = (int)(idx % nk);
    const long long r = idx / nk;
    const int t = (int)(r % b);
    const int i = (int)(r / b);
    T* col = static_cast<T*>(v.p) + k + v.si * i;
    stv(col + v.sj * t, ldv(col + v.sj * t) + ldv(col + v.sj * (-1 - t)));
    stv(col + v.sj * (J - 1 - t), ldv(col + v.sj * (J - 1 - t)) + ldv(col + v.sj * (J + t)));
}

// boco_2d on a halo band b: y first on the interior columns, then x on every
// row including the y-halo rows (mg_bocos.f90:225-377).
template <typename T>
__global__ void __launch_bounds__(256) k_fill_y(View v, int nk, int I, int J, int b) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)nk * b * I) return;
    const int k = (int)(idx % nk);
    const long long r = idx / nk;
    const int t = (int)(r % b);
    const int i = (int)(r / b);
    T* col = static_cast<T*>(v.p) + k + v.si * i;
    stv(col + v.sj * (-1 - t), ldv(col + v.sj * t));
    stv(col + v.sj * (J + t), ldv(col + v.sj * (J - 1 - t)));
}
template <typename T>
__global__ void __launch_bounds__(256) k_fill_x(View v, int nk, int I, int J, int b) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)nk * b * (J + 2 * b)) return;
    const int k = (int)(idx % nk);
    const long long r = idx / nk;
    const int t = (int)(r % b);
    const int j = (int)(r / b) - b;
    T* row = static_cast<T*>(v.p) + k + v.sj * j;
    stv(row + v.si * (-1 - t), ldv(row + v.si * t));
    stv(row + v.si * (I + t), ldv(row + v.si * (I - 1 - t)));
}

// l_vertical_direct_spec2 / l_vertical_adjoint_spec2 at every point of an
// (a, b) range: en blocks of lm filter levels <-> en blocks of lm_a = 2lm-1
// analysis levels; levels past the blocks are copied (direct) or left 0.
template <typename T>
__global__ void __launch_bounds__(256) k_vert(XferVertArgs a) {
    using A = typename AccOf<T>::type;
    const int nko = a.adjoint ? a.nkf : a.nka;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)nko * a.na * a.nb) return;
    const int ko = (int)(idx % nko);
    const long long r = idx / nko;
    const int pa = (int)(r % a.na) + a.a0, pb = (int)(r / a.na) + a.b0;
    const T* in = static_cast<const T*>(a.in.p) + a.in.si * pa + a.in.sj * pb;
    T* out = static_cast<T*>(a.out.p) + a.out.si * pa + a.out.sj * pb;
    const int lm = a.lm, lma = 2 * a.lm - 1;
    A v = A(0);
    if (!a.adjoint) {
        if (ko < a.en * lma) {
            const int e = ko / lma, n = ko - e * lma;  // 0-based analysis level
            if (n % 2 == 0) v = ldv(in + e * lm + n / 2);
            else v = A(0.5) * (ldv(in + e * lm + (n - 1) / 2) + ldv(in + e * lm + (n + 1) / 2));
        } else {
            v = ldv(in + ko - a.en * lma + a.en * lm);
        }
    } else {
        if (ko < a.en * lm) {
            const int e = ko / lm, kk = ko - e * lm;
            const T* w = in + e * lma;
            // reference order: the halves of the even levels (increasing), then the odd level
            if (kk >= 1) v += A(0.5) * ldv(w + 2 * kk - 1);
            if (2 * kk + 1 <= lma - 1) v += A(0.5) * ldv(w + 2 * kk + 1);
            v += ldv(w + 2 * kk);
        } else {
            v = ldv(in + ko - a.en * lm + a.en * lma);
        }
    }
    stv(out + ko, v);
}

inline int last_err() {
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : (int)e;
}
inline bool al16(const void* p) { return ((uintptr_t)p & 15u) == 0; }
inline size_t esz(DType t) { return t == DType::F64 ? 8 : (t == DType::F32 ? 4 : 2); }
inline bool vec_ok(DType t, int nk, const View& a, const View& b) {
    const size_t e = esz(t);
    return nk % 4 == 0 && al16(a.p) && al16(b.p) && (a.si * e) % 16 == 0 && (a.sj * e) % 16 == 0 &&
           (b.si * e) % 16 == 0 && (b.sj * e) % 16 == 0;
}
inline unsigned blocks(long long threads, int bs) { return (unsigned)((threads + bs - 1) / bs); }

template <typename F>
void dispatch(DType t, F&& f) {
    switch (t) {
        case DType::F64: f(double()); break;
        case DType::F32: f(float()); break;
        case DType::BF16: f(__nv_bfloat16()); break;
    }
}

}  // namespace

int launch_xfer_direct(DType t, const XferDirectArgs& a, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const bool vec = vec_ok(t, a.nk, a.in, a.out);
    // strip form when every strip's filter rows fit the register window
    constexpr int TM = 8, NRMAX = 16;
    if (vec && a.max_strip_rows > 0 && a.max_strip_rows <= NRMAX && t != DType::F64) {
        const unsigned g = blocks((long long)a.nk / 4 * a.nm0 * ((a.mm0 + TM - 1) / TM), 128);
        const size_t sm = sizeof(float4) * 128 * (size_t)a.max_strip_rows;  // <= 32 KB
        dispatch(t, [&](auto tag) {
            using T = decltype(tag);
            if constexpr (!std::is_same<T, double>::value) {
                switch (a.order) {
                    case 3: k_xfer_direct_strip<T, 4, 3, TM, NRMAX><<<g, 128, sm, s>>>(a); break;
                    case 2: k_xfer_direct_strip<T, 4, 2, TM, NRMAX><<<g, 128, sm, s>>>(a); break;
                    default: k_xfer_direct_strip<T, 4, 1, TM, NRMAX><<<g, 128, sm, s>>>(a); break;
                }
            }
        });
        return last_err();
    }
    dispatch(t, [&](auto tag) {
        using T = decltype(tag);
        const unsigned gv = blocks((long long)a.nk / 4 * a.nm0 * a.mm0, 128), gs = blocks((long long)a.nk * a.nm0 * a.mm0, 128);
        switch (a.order * 2 + (vec ? 1 : 0)) {
            case 7: k_xfer_direct<T, 4, 3><<<gv, 128, 0, s>>>(a); break;
            case 6: k_xfer_direct<T, 1, 3><<<gs, 128, 0, s>>>(a); break;
            case 5: k_xfer_direct<T, 4, 2><<<gv, 128, 0, s>>>(a); break;
            case 4: k_xfer_direct<T, 1, 2><<<gs, 128, 0, s>>>(a); break;
            case 3: k_xfer_direct<T, 4, 1><<<gv, 128, 0, s>>>(a); break;
            default: k_xfer_direct<T, 1, 1><<<gs, 128, 0, s>>>(a); break;
        }
    });
    return last_err();
}

int launch_xfer_gather(DType t, const XferGatherArgs& a, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const bool vec = vec_ok(t, a.nk, a.in, a.out);
    dispatch(t, [&](auto tag) {
        using T = decltype(tag);
        if (vec) k_xfer_gather<T, 4><<<blocks((long long)a.nk / 4 * a.na * a.nb, 128), 128, 0, s>>>(a);
        else k_xfer_gather<T, 1><<<blocks((long long)a.nk * a.na * a.nb, 128), 128, 0, s>>>(a);
    });
    return last_err();
}

int launch_xfer_a2f_fused(DType t, const XferFusedArgs& a, void* stream) {
    if (t == DType::F64 || a.lanes <= 0 || a.ta <= 0 || !vec_ok(t, a.nk, a.in, a.out)) return -1;
    const size_t sm = sizeof(float4) * (size_t)a.ncmax * a.lanes;
    if (sm > 48 * 1024 || a.JE > 65535) return -1;
    const int nl = a.nk / 4;
    dim3 grid((unsigned)((a.IE + a.ta - 1) / a.ta), (unsigned)a.JE, (unsigned)((nl + a.lanes - 1) / a.lanes));
    if (grid.z > 65535) return -1;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    dispatch(t, [&](auto tag) {
        using T = decltype(tag);
        if constexpr (!std::is_same<T, double>::value) k_xfer_a2f_fused<T><<<grid, 256, sm, s>>>(a);
    });
    return last_err();
}

int launch_xfer_fold(DType t, View v, int nk, int I, int J, int b, void* stream) {
    if (b <= 0) return 0;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    dispatch(t, [&](auto tag) {
        using T = decltype(tag);
        k_fold_x<T><<<blocks((long long)nk * b * (J + 2 * b), 256), 256, 0, s>>>(v, nk, I, J, b);
        k_fold_y<T><<<blocks((long long)nk * b * I, 256), 256, 0, s>>>(v, nk, I, J, b);
    });
    return last_err();
}

int launch_xfer_fill(DType t, View v, int nk, int I, int J, int b, void* stream) {
    if (b <= 0) return 0;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    dispatch(t, [&](auto tag) {
        using T = decltype(tag);
        k_fill_y<T><<<blocks((long long)nk * b * I, 256), 256, 0, s>>>(v, nk, I, J, b);
        k_fill_x<T><<<blocks((long long)nk * b * (J + 2 * b), 256), 256, 0, s>>>(v, nk, I, J, b);
    });
    return last_err();
}

int launch_xfer_vert(DType t, const XferVertArgs& a, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const long long n = (long long)(a.adjoint ? a.nkf : a.nka) * a.na * a.nb;
    if (n == 0) return 0;
    dispatch(t, [&](auto tag) {
        using T = decltype(tag);
        k_vert<T><<<blocks(n, 256), 256, 0, s>>>(a);
    });
    return last_err();
}

}  // namespace mgbf
