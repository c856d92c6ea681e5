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

// Half-sample mirror of a 0-based index into [0, n): -1 -> 0, n -> n-1
// (the reference's physical-boundary halo fill, mg_bocos.f90:225-377),
// clamped so that rows only used for discarded outputs stay in range.
__device__ __forceinline__ int reflect_half(int j, int n) {
    j = j < 0 ? -1 - j : j;
    j = j >= n ? 2 * n - 1 - j : j;
    return j < 0 ? 0 : (j >= n ? n - 1 : j);
}

}  // namespace mgbf
