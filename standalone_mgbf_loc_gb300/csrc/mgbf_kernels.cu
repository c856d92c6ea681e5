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
#include "mgbf_common.cuh"
#include "mgbf_kernels.cuh"

namespace mgbf {

// ------------------------------------------------------------- z filter
// out(k) = sum_d band[L][d+mz] * in(c0+L+d) for z columns (k < nzk), where
// band is the FP64-built matrix of sup_vrbeta1_* / sup_vrbeta1T_*
// (mg_filtering.f90:2042-2262) including the whole-sample mirror and, for
// the adjoint, the edge fold; entries k >= nzk (2D variables) are copied.
template <typename T>
__global__ void __launch_bounds__(256) k_zfilter(ZArgs a) {
    using A = typename AccOf<T>::type;
    extern __shared__ unsigned char smem_raw[];
    A* band = reinterpret_cast<A*>(smem_raw);
    const int bw = 2 * a.mz + 1;
    const int nb = a.lm * bw;
    for (int t = threadIdx.x; t < nb; t += blockDim.x) band[t] = static_cast<const A*>(a.band)[t];
    __syncthreads();
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)a.nk * a.I) return;
    const int i = (int)(t / a.nk);
    const int k = (int)(t - (long long)i * a.nk);
    const int j = blockIdx.y;
    const T* in = static_cast<const T*>(a.in.p) + a.in.sj * j + a.in.si * i;
    A v;
    if (k < a.nzk) {
        const int L = k % a.lm;
        const int c0 = k - L;
        const A* b = band + L * bw + a.mz;
        const int dlo = max(-a.mz, -L), dhi = min(a.mz, a.lm - 1 - L);
        v = A(0);
        for (int d = dlo; d <= dhi; ++d) v = fma(b[d], ldv(in + c0 + L + d), v);
    } else {
        v = ldv(in + k);
    }
    T* out = static_cast<T*>(a.out.p) + a.out.sj * j + k;
    stv(out + a.out.si * i, v);
    if (a.mirror_hx) {
        if (i < a.mirror_hx) stv(out + a.out.si * (-1 - i), v);
        if (i >= a.I - a.mirror_hx) stv(out + a.out.si * (2 * a.I - 1 - i), v);
    }
}

// --------------------------------------------------------- restriction
// coarse(c,d) = sum_b wy[d][b] sum_a wx[c][a] fine(2c-3+a, 2d-3+b): the
// separable transpose of (P o fill2) (adjoint + bocoT_2d(...,2,2),
// mg_generations.f90:1117-1187, mg_bocos.f90:929-1061) with the mirror
// images already merged into the 8-wide weight rows.
template <typename T>
__global__ void __launch_bounds__(256) k_restrict(RestrictArgs a) {
    using A = typename AccOf<T>::type;
    const int Ic = a.If / 2;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)a.nk * Ic) return;
    const int c = (int)(t / a.nk);
    const int k = (int)(t - (long long)c * a.nk);
    const int d = blockIdx.y;
    const A* wx = static_cast<const A*>(a.wx) + c * 8;
    const A* wy = static_cast<const A*>(a.wy) + d * 8;
    const T* fine = static_cast<const T*>(a.fine.p) + k;
    A acc = A(0);
#pragma unroll
    for (int b = 0; b < 8; ++b) {
        const int fj = 2 * d - 3 + b;
        if (fj < 0 || fj >= a.Jf) continue;
        const T* row = fine + a.fine.sj * fj;
        A r = A(0);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int fi = 2 * c - 3 + q;
            if (fi < 0 || fi >= a.If) continue;
            r = fma(wx[q], ldv(row + a.fine.si * fi), r);
        }
        acc = fma(wy[b], r, acc);
    }
    T* out = static_cast<T*>(a.coarse.p) + a.coarse.sj * d + k;
    stv(out + a.coarse.si * c, acc);
    if (a.mirror_hx) {
        if (c < a.mirror_hx) stv(out + a.coarse.si * (-1 - c), acc);
        if (c >= Ic - a.mirror_hx) stv(out + a.coarse.si * (2 * Ic - 1 - c), acc);
    }
}

// -------------------------------------------------------- prolongation
// out(i,j) = base(i,j) + sum_b wy[j][b] sum_a wx[i][a] coarse(ix[i][a], iy[j][b]):
// downsend + boco_2d(...,2,2) + direct1 + add (mg_generations.f90:210-267,
// 1190-1250); x pass inside, y pass outside, as direct1 orders them.
template <typename T>
__global__ void __launch_bounds__(256) k_prolong(ProlongArgs a) {
    using A = typename AccOf<T>::type;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)a.nk * a.If) return;
    const int i = (int)(t / a.nk);
    const int k = (int)(t - (long long)i * a.nk);
    const int j = blockIdx.y;
    const int nt = a.ntap;
    const int* ixp = a.ix + i * nt;
    const int* iyp = a.iy + j * nt;
    const A* wxp = static_cast<const A*>(a.wxp) + i * nt;
    const A* wyp = static_cast<const A*>(a.wyp) + j * nt;
    const T* coarse = static_cast<const T*>(a.coarse.p) + k;
    A acc = A(0);
    for (int b = 0; b < nt; ++b) {
        const T* row = coarse + a.coarse.sj * iyp[b];
        A r = A(0);
        for (int q = 0; q < nt; ++q) r = fma(wxp[q], ldv(row + a.coarse.si * ixp[q]), r);
        acc = fma(wyp[b], r, acc);
    }
    if (a.has_base) {
        const T* base = static_cast<const T*>(a.base.p) + a.base.sj * j + a.base.si * i + k;
        acc = ldc(base) + acc;
    }
    T* out = static_cast<T*>(a.out.p) + a.out.sj * j + a.out.si * i + k;
    stv(out, acc);
}

// ------------------------------------------- direct-sum radial beta filter
// General support table (any aspect, any integer p): the gather form of
// fill_h + vrbeta2 (jp_pbfil.f90:888-928).  Because the radial weights are
// even in gx and gy and the mirror is half-sample, the same gather also
// equals vrbeta2t + fold_h (jp_pbfil.f90:1011-1050); the tests check this
// against the oracle's literal scatter form.  Each lane owns one k and TX
// consecutive columns; the input carries an x halo >= R + TX - 1.
template <typename T, int TX>
__global__ void __launch_bounds__(128) k_hdirect(HDirectArgs a) {
    using A = typename AccOf<T>::type;
    extern __shared__ unsigned char smem_raw[];
    const int W = 2 * a.R + 1;
    A* w = reinterpret_cast<A*>(smem_raw);
    int* mrow = reinterpret_cast<int*>(w + W * W);
    const int nthreads = blockDim.x * blockDim.y;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    for (int t = tid; t < W * W; t += nthreads) w[t] = static_cast<const A*>(a.w)[t];
    for (int t = tid; t < W; t += nthreads) mrow[t] = a.mrow[t];
    __syncthreads();
    int k = blockIdx.x * 32 + threadIdx.x;
    const bool kv = k < a.nk;
    if (!kv) k = a.nk - 1;
    const int i0 = (blockIdx.y * blockDim.y + threadIdx.y) * TX;
    if (i0 >= a.I) return;
    const int j = blockIdx.z;
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

static inline int last_err() {
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : (int)e;
}

int launch_zfilter(DType t, const ZArgs& a, void* stream) {
    const long long n = (long long)a.nk * a.I;
    if (n == 0 || a.J == 0) return 0;
    dim3 block(256), grid((unsigned)((n + 255) / 256), a.J);
    const size_t sm = acc_size(t) * a.lm * (2 * a.mz + 1);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (sm > 48 * 1024) {
        MGBF_DISPATCH(t, (cudaFuncSetAttribute(k_zfilter<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm)));
    }
    MGBF_DISPATCH(t, (k_zfilter<T><<<grid, block, sm, s>>>(a)));
    return last_err();
}

int launch_restrict(DType t, const RestrictArgs& a, void* stream) {
    const long long n = (long long)a.nk * (a.If / 2);
    if (n == 0) return 0;
    dim3 block(256), grid((unsigned)((n + 255) / 256), a.Jf / 2);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    MGBF_DISPATCH(t, (k_restrict<T><<<grid, block, 0, s>>>(a)));
    return last_err();
}

int launch_prolong(DType t, const ProlongArgs& a, void* stream) {
    const long long n = (long long)a.nk * a.If;
    if (n == 0) return 0;
    dim3 block(256), grid((unsigned)((n + 255) / 256), a.Jf);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    MGBF_DISPATCH(t, (k_prolong<T><<<grid, block, 0, s>>>(a)));
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

int launch_hdirect(DType t, const HDirectArgs& a, void* stream) {
    constexpr int TX = 4, NW = 4;
    const int W = 2 * a.R + 1;
    const size_t sm = acc_size(t) * W * W + sizeof(int) * W;
    const int nstrip = (a.I + TX - 1) / TX;
    dim3 block(32, NW), grid((a.nk + 31) / 32, (nstrip + NW - 1) / NW, a.J);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
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
