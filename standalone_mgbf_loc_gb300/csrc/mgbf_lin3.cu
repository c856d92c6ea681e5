// filtering_lin3 (procedure 5, mg_filtering.f90:260-557): the 3D line
// filters of the hexad on the 3D variables of one generation (sm_103a).
//
// The reference copies the 3D variables of a generation into a work array
// W(km3, 1-hx:im+hx, 1-hy:jm+hy, 1-hz:lm+hz) and runs, per color, its 3D
// halo routines and the dibeta line filter along the color's generator
// (jp_pbfil3.f90:1928-1977 vdibetax3, 2475-2525 vdibetax3t;
// mg_bocos.f90:1425-2908 boco_3d / bocoT_3d).  Here the work array lives in
// HBM with the level index fastest, W[(j+hy)][(i+hx)][v][L+hz], so that a
// warp reads 32 consecutive levels of one column whichever direction a
// generator points.  Each stage is its own launch over whole rows, columns
// or cells; the stages keep the reference's order (x before y before z in
// the folds, y before x in the fills), so every element goes through the
// same sequence of additions as in the reference.
#include "mgbf_common.cuh"
#include "mgbf_kernels.cuh"

namespace mgbf {
namespace {

struct W3 {
    long long LX, NV, NI;  // extended levels, variables, extended columns
    int lm, I, J, hx, hy, hz;
    __device__ __forceinline__ long long at(int v, int i, int j, int L) const {
        return (long long)(L + hz) + LX * ((long long)v + NV * ((long long)(i + hx) + NI * (long long)(j + hy)));
    }
    __device__ __forceinline__ bool interior(int i, int j, int L) const {
        return i >= 0 && i < I && j >= 0 && j < J && L >= 0 && L < lm;
    }
};

W3 make_w3(const Lin3Args& a) {
    W3 w;
    w.LX = a.lm + 2 * a.hz;
    w.NV = a.nv;
    w.NI = a.I + 2 * a.hx;
    w.lm = a.lm; w.I = a.I; w.J = a.J; w.hx = a.hx; w.hy = a.hy; w.hz = a.hz;
    return w;
}

// generation buffer (k = v*lm + L, i, j) <-> work array interior; `to`
// multiplies by scale (the generation weight on the adjoint side)
template <typename T>
__global__ void __launch_bounds__(256) k_l3_copy(Lin3Args a, W3 w, int to) {
    using A = typename AccOf<T>::type;
    // 32-bit decode: one row's index space is small, and a 64-bit division
    // by a runtime value costs far more than the copy itself
    const unsigned nlv = (unsigned)(a.nv * a.lm);
    const unsigned x = blockIdx.x * blockDim.x + threadIdx.x;  // (k, i) of row j, k fastest
    if (x >= nlv * (unsigned)a.I) return;
    const int i = (int)(x / nlv), k = (int)(x - (unsigned)i * nlv), j = blockIdx.y;
    const int v = k / a.lm, L = k - v * a.lm;
    T* W = static_cast<T*>(a.w);
    if (to) {
        T* out = static_cast<T*>(a.out.p) + k + a.out.si * i + a.out.sj * j;
        stv(out, static_cast<A>(ldc(W + w.at(v, i, j, L))) * static_cast<A>(a.scale));
    } else {
        const T* in = static_cast<const T*>(a.in.p) + k + a.in.si * i + a.in.sj * j;
        W[w.at(v, i, j, L)] = *in;
    }
}

// One color's dibeta over every cell of the extended array, into t.
// Forward (vdibetax3): interior cells gather fil[0] W(p) + sum_s fil[s]
// (W(p + s d) + W(p - s d)), halo cells are zero.  Adjoint (vdibetax3t,
// the scatter from the interior, written as a gather): cell q collects
// fil[0] W(q) if q is interior and fil[s] W(q -+ s d) from each interior
// q -+ s d.  A color without a line (h = 0, fil[0] = 1) copies the interior.
template <typename T>
__global__ void __launch_bounds__(256) k_l3_dib(Lin3Args a, W3 w, int adj) {
    using A = typename AccOf<T>::type;
    const unsigned lx = (unsigned)w.LX, cell = (unsigned)(w.LX * w.NV);  // extended levels of one column
    const unsigned x = blockIdx.x * blockDim.x + threadIdx.x;  // (L, v, i) of row j, L fastest (32-bit decode)
    if (x >= cell * (unsigned)w.NI) return;
    const unsigned ic = x / cell, r = x - ic * cell;
    const int v = (int)(r / lx), L = (int)(r - (unsigned)v * lx) - a.hz;
    const int i = (int)ic - a.hx, j = (int)blockIdx.y - a.hy;
    const T* W = static_cast<const T*>(a.w);
    T* Tb = static_cast<T*>(a.t);
    A fil[kMaxL3Span + 1];
#pragma unroll
    for (int s = 0; s <= kMaxL3Span; ++s) fil[s] = sizeof(A) == 8 ? (A)a.fil[s] : (A)a.filf[s];
    const bool in_p = w.interior(i, j, L);
    // the cell's index once, and one step along the generator (its
    // neighbours are base +- s * step: no index arithmetic per tap)
    const long long base = w.at(v, i, j, L);
    const long long step = (long long)a.dz + w.LX * (w.NV * ((long long)a.dx + w.NI * (long long)a.dy));
    const T* Wc = W + base;
    A acc = A(0);
    if (!adj) {
        if (in_p) {
            acc = fil[0] * static_cast<A>(ldc(Wc));
#pragma unroll
            for (int s = 1; s <= kMaxL3Span; ++s) {
                if (s > a.h) break;
                acc += fil[s] * (static_cast<A>(ldc(Wc + s * step)) + static_cast<A>(ldc(Wc - s * step)));
            }
        }
    } else {
        if (in_p) acc = fil[0] * static_cast<A>(ldc(Wc));
#pragma unroll
        for (int s = 1; s <= kMaxL3Span; ++s) {
            if (s > a.h) break;
            const int im = i - s * a.dx, jm = j - s * a.dy, Lm = L - s * a.dz;
            const int ip = i + s * a.dx, jp = j + s * a.dy, Lp = L + s * a.dz;
            if (w.interior(im, jm, Lm)) acc += fil[s] * static_cast<A>(ldc(Wc - s * step));
            if (w.interior(ip, jp, Lp)) acc += fil[s] * static_cast<A>(ldc(Wc + s * step));
        }
    }
    stv(Tb + base, acc);
}

// bocoT_3d x part (mg_bocos.f90:2173-2527, 2530-2908): on every row of the
// extended y range and every level 1..lm, west then east; o = 0 for the
// generation-1 form (the east fold reads W(I+hx-i): the edge column is
// added to itself), 1 for coarser generations.
template <typename T>
__global__ void __launch_bounds__(256) k_l3_foldx(Lin3Args a, W3 w, int o) {
    using A = typename AccOf<T>::type;
    const unsigned nlv = (unsigned)(a.lm * a.nv), lm = (unsigned)a.lm;
    const unsigned x = blockIdx.x * blockDim.x + threadIdx.x;  // ((v, L), j), L fastest (32-bit decode)
    if (x >= nlv * (unsigned)(a.J + 2 * a.hy)) return;
    const unsigned jr = x / nlv, r = x - jr * nlv;
    const int v = (int)(r / lm), L = (int)(r - (unsigned)v * lm);
    const int j = (int)jr - a.hy;
    T* const row = static_cast<T*>(a.w) + w.at(v, 0, j, L);  // column c at row + c * cs
    const long long cs = w.LX * w.NV;
    for (int s = 1; s <= a.hx; ++s) {
        T* d = row + (s - 1) * cs;
        stv(d, static_cast<A>(ldc(d)) + static_cast<A>(ldc(row - s * cs)));
    }
    for (int s = 1; s <= a.hx; ++s) {
        T* d = row + (a.I - a.hx + s - 1) * cs;
        stv(d, static_cast<A>(ldc(d)) + static_cast<A>(ldc(row + (a.I + o + a.hx - s - 1) * cs)));
    }
}

// bocoT_3d y part: interior columns, levels 1..lm, south then north.
template <typename T>
__global__ void __launch_bounds__(256) k_l3_foldy(Lin3Args a, W3 w, int o) {
    using A = typename AccOf<T>::type;
    const unsigned nlv = (unsigned)(a.lm * a.nv), lm = (unsigned)a.lm;
    const unsigned x = blockIdx.x * blockDim.x + threadIdx.x;  // ((v, L), i), L fastest (32-bit decode)
    if (x >= nlv * (unsigned)a.I) return;
    const unsigned ir = x / nlv, r = x - ir * nlv;
    const int v = (int)(r / lm), L = (int)(r - (unsigned)v * lm);
    const int i = (int)ir;
    T* const col = static_cast<T*>(a.w) + w.at(v, i, 0, L);  // row r at col + r * rs
    const long long rs = w.LX * w.NV * w.NI;
    for (int s = 1; s <= a.hy; ++s) {
        T* d = col + (s - 1) * rs;
        stv(d, static_cast<A>(ldc(d)) + static_cast<A>(ldc(col - s * rs)));
    }
    for (int s = 1; s <= a.hy; ++s) {
        T* d = col + (a.J - a.hy + s - 1) * rs;
        stv(d, static_cast<A>(ldc(d)) + static_cast<A>(ldc(col + (a.J + o + a.hy - s - 1) * rs)));
    }
}

// bocoT_3d z part: on every column of the extended plane, for L = 1..hz the
// lower halo level into level 1+L, then the upper one into lm-L.
template <typename T>
__global__ void __launch_bounds__(256) k_l3_foldz(Lin3Args a, W3 w) {
    using A = typename AccOf<T>::type;
    const unsigned nv = (unsigned)w.NV;
    const unsigned x = blockIdx.x * blockDim.x + threadIdx.x;  // (v, i), v fastest (32-bit decode)
    if (x >= nv * (unsigned)w.NI) return;
    const int v = (int)(x % nv), i = (int)(x / nv) - a.hx;
    const int j = (int)blockIdx.y - a.hy;
    T* const c0 = static_cast<T*>(a.w) + w.at(v, i, j, 0);  // level L at c0 + L
    for (int s = 1; s <= a.hz; ++s) {
        T* lo = c0 + s;
        stv(lo, static_cast<A>(ldc(lo)) + static_cast<A>(ldc(c0 - s)));
        T* hi = c0 + (a.lm - s - 1);
        stv(hi, static_cast<A>(ldc(hi)) + static_cast<A>(ldc(c0 + (a.lm + s - 1))));
    }
}

// boco_3d y part (interior columns, levels 1..lm): north, then south, as
// half-sample mirrors W(J+j) = W(J+1-j), W(-hy+j) = W(hy+1-j).
template <typename T>
__global__ void __launch_bounds__(256) k_l3_filly(Lin3Args a, W3 w) {
    const unsigned nlv = (unsigned)(a.lm * a.nv), lm = (unsigned)a.lm;
    const unsigned x = blockIdx.x * blockDim.x + threadIdx.x;  // ((v, L), i), L fastest (32-bit decode)
    if (x >= nlv * (unsigned)a.I) return;
    const unsigned ir = x / nlv, r = x - ir * nlv;
    const int v = (int)(r / lm), L = (int)(r - (unsigned)v * lm);
    const int i = (int)ir;
    T* const col = static_cast<T*>(a.w) + w.at(v, i, 0, L);  // row r at col + r * rs
    const long long rs = w.LX * w.NV * w.NI;
    for (int s = 1; s <= a.hy; ++s) col[(a.J + s - 1) * rs] = col[(a.J - s) * rs];
    for (int s = 1; s <= a.hy; ++s) col[(-a.hy + s - 1) * rs] = col[(a.hy - s) * rs];
}

// boco_3d x part (every row of the extended y range, levels 1..lm): west
// W(-hx+i) = W(hx+1-i), then east W(I+i) = W(I-i) at generation 1
// (boco_3d_g1) or W(I+1-i) (boco_3d_gh, o = 1).
template <typename T>
__global__ void __launch_bounds__(256) k_l3_fillx(Lin3Args a, W3 w, int o) {
    const unsigned nlv = (unsigned)(a.lm * a.nv), lm = (unsigned)a.lm;
    const unsigned x = blockIdx.x * blockDim.x + threadIdx.x;  // ((v, L), j), L fastest (32-bit decode)
    if (x >= nlv * (unsigned)(a.J + 2 * a.hy)) return;
    const unsigned jr = x / nlv, r = x - jr * nlv;
    const int v = (int)(r / lm), L = (int)(r - (unsigned)v * lm);
    const int j = (int)jr - a.hy;
    T* const row = static_cast<T*>(a.w) + w.at(v, 0, j, L);  // column c at row + c * cs
    const long long cs = w.LX * w.NV;
    for (int s = 1; s <= a.hx; ++s) row[(-a.hx + s - 1) * cs] = row[(a.hx - s) * cs];
    for (int s = 1; s <= a.hx; ++s) row[(a.I + s - 1) * cs] = row[(a.I - s - 1 + o) * cs];
}

// Whole-sample mirror of the z halo on every column of the extended plane:
// W(1-L) = W(1+L), W(lm+L) = W(lm-L), L = 1..hz.
template <typename T>
__global__ void __launch_bounds__(256) k_l3_zmirror(Lin3Args a, W3 w) {
    const unsigned nv = (unsigned)w.NV;
    const unsigned x = blockIdx.x * blockDim.x + threadIdx.x;  // (v, i), v fastest (32-bit decode)
    if (x >= nv * (unsigned)w.NI) return;
    const int v = (int)(x % nv), i = (int)(x / nv) - a.hx;
    const int j = (int)blockIdx.y - a.hy;
    T* const c0 = static_cast<T*>(a.w) + w.at(v, i, j, 0);  // level L at c0 + L
    for (int s = 1; s <= a.hz; ++s) {
        c0[-s] = c0[s];
        c0[a.lm + s - 1] = c0[a.lm - s - 1];
    }
}

// Zero every halo cell of the extended array (x, y and z halos) in place:
// what the dibeta of a color without a line (h = 0, fil[0] = 1) leaves,
// since it copies the interior exactly and writes zero elsewhere.
template <typename T>
__global__ void __launch_bounds__(256) k_l3_halo_zero(Lin3Args a, W3 w) {
    const unsigned lx = (unsigned)w.LX, cell = (unsigned)(w.LX * w.NV);
    const unsigned x = blockIdx.x * blockDim.x + threadIdx.x;  // (L, v, i) of row j, L fastest (32-bit decode)
    if (x >= cell * (unsigned)w.NI) return;
    const unsigned ic = x / cell, r = x - ic * cell;
    const int v = (int)(r / lx), L = (int)(r - (unsigned)v * lx) - a.hz;
    const int i = (int)ic - a.hx, j = (int)blockIdx.y - a.hy;
    if (!w.interior(i, j, L)) static_cast<T*>(a.w)[w.at(v, i, j, L)] = T(0.0f);
}

template <typename T>
int launch_lin3_t(const Lin3Args& a0, int op, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Lin3Args a = a0;
    for (int q = 0; q <= kMaxL3Span; ++q) a.filf[q] = (float)a.fil[q];
    const W3 w = make_w3(a);
    const int NI = a.I + 2 * a.hx, NJ = a.J + 2 * a.hy;
    const long long nlv = (long long)a.lm * a.nv;
    const long long ncol = (long long)a.nv * NI;
    auto blocks = [](long long n) { return (unsigned)((n + 255) / 256); };
    switch (op) {
        case kL3From:
        case kL3To:
            k_l3_copy<T><<<dim3(blocks(nlv * a.I), a.J), 256, 0, s>>>(a, w, op == kL3To);
            break;
        case kL3DibFwd:
        case kL3DibAdj:
            k_l3_dib<T><<<dim3(blocks(w.LX * w.NV * NI), NJ), 256, 0, s>>>(a, w, op == kL3DibAdj);
            break;
        case kL3FoldX: k_l3_foldx<T><<<blocks(nlv * NJ), 256, 0, s>>>(a, w, a.gh); break;
        case kL3FoldY: k_l3_foldy<T><<<blocks(nlv * a.I), 256, 0, s>>>(a, w, a.gh); break;
        case kL3FoldZ: k_l3_foldz<T><<<dim3(blocks(ncol), NJ), 256, 0, s>>>(a, w); break;
        case kL3FillY: k_l3_filly<T><<<blocks(nlv * a.I), 256, 0, s>>>(a, w); break;
        case kL3FillX: k_l3_fillx<T><<<blocks(nlv * NJ), 256, 0, s>>>(a, w, a.gh); break;
        case kL3ZMirror: k_l3_zmirror<T><<<dim3(blocks(ncol), NJ), 256, 0, s>>>(a, w); break;
        case kL3HaloZero: k_l3_halo_zero<T><<<dim3(blocks(w.LX * w.NV * NI), NJ), 256, 0, s>>>(a, w); break;
        default: return (int)cudaErrorInvalidValue;
    }
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : (int)e;
}

}  // namespace

int launch_lin3(DType t, const Lin3Args& a, int op, void* stream) {
    switch (t) {
        case DType::F64: return launch_lin3_t<double>(a, op, stream);
        case DType::F32: return launch_lin3_t<float>(a, op, stream);
        case DType::BF16: return launch_lin3_t<__nv_bfloat16>(a, op, stream);
    }
    return (int)cudaErrorInvalidValue;
}

}  // namespace mgbf
