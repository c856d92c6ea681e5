// Device helpers shared by the sm_103a kernels.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace mgbf {

// Arithmetic type for a storage type: FP64 storage computes in FP64,
// FP32 and BF16 storage compute in FP32.
template <typename T> struct AccOf { using type = float; };
template <> struct AccOf<double> { using type = double; };

__device__ __forceinline__ float ldv(const float* p) { return __ldg(p); }
__device__ __forceinline__ double ldv(const double* p) { return __ldg(p); }
__device__ __forceinline__ float ldv(const __nv_bfloat16* p) { return __bfloat162float(__ldg(p)); }

// Plain (coherent) loads for buffers the same kernel also writes.
__device__ __forceinline__ float ldc(const float* p) { return *p; }
__device__ __forceinline__ double ldc(const double* p) { return *p; }
__device__ __forceinline__ float ldc(const __nv_bfloat16* p) { return __bfloat162float(*p); }

__device__ __forceinline__ void stv(float* p, float v) { *p = v; }
__device__ __forceinline__ void stv(double* p, double v) { *p = v; }
__device__ __forceinline__ void stv(__nv_bfloat16* p, float v) { *p = __float2bfloat16_rn(v); }

// Four consecutive level values (k, k+1, k+2, k+3; k % 4 == 0) as one
// vector access: float4, two double2, or four bf16 in 8 bytes.
template <typename T> struct V4;
template <> struct V4<float> {
    static __device__ __forceinline__ void ld(const float* p, float (&v)[4]) {
        const float4 x = __ldg(reinterpret_cast<const float4*>(p));
        v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
    }
    static __device__ __forceinline__ void ldc(const float* p, float (&v)[4]) {
        const float4 x = *reinterpret_cast<const float4*>(p);
        v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
    }
    static __device__ __forceinline__ void st(float* p, const float (&v)[4]) {
        *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
    }
};
template <> struct V4<double> {
    static __device__ __forceinline__ void ld(const double* p, double (&v)[4]) {
        const double2 a = __ldg(reinterpret_cast<const double2*>(p));
        const double2 b = __ldg(reinterpret_cast<const double2*>(p) + 1);
        v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
    }
    static __device__ __forceinline__ void ldc(const double* p, double (&v)[4]) {
        const double2 a = *reinterpret_cast<const double2*>(p);
        const double2 b = *(reinterpret_cast<const double2*>(p) + 1);
        v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
    }
    static __device__ __forceinline__ void st(double* p, const double (&v)[4]) {
        reinterpret_cast<double2*>(p)[0] = make_double2(v[0], v[1]);
        reinterpret_cast<double2*>(p)[1] = make_double2(v[2], v[3]);
    }
};
template <> struct V4<__nv_bfloat16> {
    static __device__ __forceinline__ void unpack(uint2 u, float (&v)[4]) {
        v[0] = __uint_as_float(u.x << 16);
        v[1] = __uint_as_float(u.x & 0xffff0000u);
        v[2] = __uint_as_float(u.y << 16);
        v[3] = __uint_as_float(u.y & 0xffff0000u);
    }
    static __device__ __forceinline__ void ld(const __nv_bfloat16* p, float (&v)[4]) {
        unpack(__ldg(reinterpret_cast<const uint2*>(p)), v);
    }
    static __device__ __forceinline__ void ldc(const __nv_bfloat16* p, float (&v)[4]) {
        unpack(*reinterpret_cast<const uint2*>(p), v);
    }
    static __device__ __forceinline__ void st(__nv_bfloat16* p, const float (&v)[4]) {
        const __nv_bfloat162 a = __floats2bfloat162_rn(v[0], v[1]);
        const __nv_bfloat162 b = __floats2bfloat162_rn(v[2], v[3]);
        uint2 u;
        u.x = *reinterpret_cast<const unsigned*>(&a);
        u.y = *reinterpret_cast<const unsigned*>(&b);
        *reinterpret_cast<uint2*>(p) = u;
    }
};

// 16-byte asynchronous global -> shared copy (L1 bypassed); `bytes` < 16
// zero-fills the rest of the destination.
__device__ __forceinline__ void cp_async16(unsigned saddr, const void* g, int bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(saddr), "l"(g), "r"(bytes) : "memory");
}
// 8-byte form (cp.async.ca); bytes < 8 zero-fills the rest
__device__ __forceinline__ void cp_async8(unsigned saddr, const void* g, int bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(saddr), "l"(g), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// mbarrier and TMA (cp.async.bulk.tensor) primitives.  A consumer waits on a
// barrier's phase parity with a bounded number of polls; the caller decides
// what a wait that gives up means.
__device__ __forceinline__ void mbar_init(unsigned addr, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(addr), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned addr, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(addr), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned addr, unsigned parity) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    return done != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(unsigned addr, unsigned parity, int max_polls) {
    for (int it = 0; it < max_polls; ++it)
        if (mbar_try_wait(addr, parity)) return true;
    return false;
}
__device__ __forceinline__ void tma_load_3d(unsigned dst, const void* tmap, int c0, int c1, int c2, unsigned bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(dst),
        "l"(tmap), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
        : "memory");
}

// Half-sample mirror of a 0-based index into [0, n): -1 -> 0, n -> n-1
// (the reference's physical-boundary halo fill, mg_bocos.f90:225-377),
// clamped so that rows only used for discarded outputs stay in range.
__device__ __forceinline__ int reflect_half(int j, int n) {
    j = j < 0 ? -1 - j : j;
    j = j >= n ? 2 * n - 1 - j : j;
    return j < 0 ? 0 : (j >= n ? n - 1 : j);
}

// Streaming multiprocessors of the current device (queried once per device;
// grid sizing targets whole waves of them).  Falls back to GB300's 152 if
// the query fails.
inline int device_sm_count() {
    static int cache[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return 152;
    }
    if (!cache[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
            cudaGetLastError();
            n = 152;
        }
        cache[dev] = n;
    }
    return cache[dev];
}

// Opts a kernel into more than 48 KB of dynamic shared memory, once per
// device (the attribute persists, so graph captures later need no API call).
template <typename K>
inline cudaError_t smem_optin(K kernel, size_t bytes, unsigned long long& done /* one bit per device */) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev >= 64) return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (done >> dev & 1ull) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) done |= 1ull << dev;
    return e;
}

}  // namespace mgbf
