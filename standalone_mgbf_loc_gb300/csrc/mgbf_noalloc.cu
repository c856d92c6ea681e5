// Radial beta filtering of one field without any device allocation.
//
// Some callers cannot allocate device memory: code running while a CUDA
// stream is being captured into a graph (where cudaMalloc is not allowed
// for the captured work), an application that hands out all device memory
// through its own pool and forbids other allocators, or a host program whose
// memory budget is fixed in advance.  mgbf_radial_filter_noalloc serves them:
// it computes y = weight * B(B(x)) -- the generation-1 radial filtering that
// filtering_procedure performs with one generation and no vertical filter --
// and keeps its two intermediate fields in a file-scope device array instead
// of memory obtained from cudaMalloc.  The caller still provides x and y.
//
// The array is static: every GPU that loads this library holds its
// 64 MiB until the process exits.  Its device address is looked up with
// cudaGetSymbolAddress once per device, by the first call made with that
// device current; that first call should come before any stream capture
// (a lookup that fails is retried by the next call).
// All calls share the array and it keeps the last call's contents (nothing
// in it has to start at zero: each call overwrites every element it later
// reads).  Calls that overlap on the GPU (different streams, or different
// host threads on the same device) race on the array and must be ordered by
// the caller.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "../../include/mgbf.h"
#include "mgbf_common.cuh"
#include "mgbf_kernels.cuh"
#include "mgbf_setup.hpp"

namespace {

// 16 Mi FP32 elements = 64 MiB: two buffers of up to 8 Mi elements each,
// i.e. nk * (im + 2*(reach+8)) * jm <= MGBF_NOALLOC_MAX_ELEMS.
constexpr size_t kNoAllocElems = (size_t)2 * MGBF_NOALLOC_MAX_ELEMS;
static __device__ __align__(256) float g_noalloc_scratch[kNoAllocElems];

constexpr int kMaxDevices = 64;
float* g_scratch_addr[kMaxDevices];  // set only once a lookup has succeeded
std::mutex g_scratch_mutex[kMaxDevices];

// Moment coefficients of the canonical radial disk, computed on the stack
// (the same FP64 formulas as the handle's setup: cholaspect2, getlinesum2).
int moment_setup(int p, double ampl02, int hx, int hy, mgbf::HMomCoefs<double>& c, int& R, double& s) {
    using mgbf::report_error;
    if (!(ampl02 > 0.0)) return report_error(MGBF_ERR_CONFIG, "mg_ampl02 must be positive");
    if (p != 2) return report_error(MGBF_ERR_UNSUPPORTED, "the allocation-free filter needs p = 2");
    const double e = std::sqrt(1.0 / ampl02) * (1.0 / std::sqrt(2.0 * p + 4.0));
    const double y = 1.0 / e;
    const int gyl = (int)std::ceil(-y + mgbf::kEps), gym = (int)std::floor(y - mgbf::kEps);
    if (gyl < -hy || gym > hy) return report_error(MGBF_ERR_REACH, "getlinesum2: filter reach exceeds hy");
    R = gym;
    double sum = 0.0;
    for (int gy = gyl; gy <= gym; ++gy) {
        const double rrx = (gy * e) * (gy * e);
        const double x = std::sqrt(1.0 - rrx);
        const int lo = (int)std::ceil(-x / e + mgbf::kEps), hi = (int)std::floor(x / e - mgbf::kEps);
        if (lo < -hx || hi > hx) return report_error(MGBF_ERR_REACH, "getlinesum2: filter reach exceeds hx");
        if (lo != -hi || hi != mgbf::canonical_width(gym, gy < 0 ? -gy : gy) || gyl != -gym)
            return report_error(MGBF_ERR_UNSUPPORTED,
                                "the allocation-free filter needs the disk of radius reach+1/2 "
                                "(mg_ampl02 = (reach+1/2)^2/(2p+4))");
        for (int gx = lo; gx <= hi; ++gx) {
            const double rrc = 1.0 - (rrx + (gx * e) * (gx * e));
            sum += rrc * rrc;
        }
    }
    if (!mgbf::hmom_available(mgbf::DType::F32, R, p))
        return report_error(MGBF_ERR_UNSUPPORTED, "no compiled moment kernel for this reach");
    s = 1.0 / sum;
    c = mgbf::HMomCoefs<double>{};
    for (int gy = 0; gy <= R; ++gy) c.coef[gy * 3] = 1.0 - (gy * e) * (gy * e);
    for (int m = 0; m <= R; ++m) {
        const double u = (m * e) * (m * e);
        c.upow[m * 3 + 0] = 1.0;
        c.upow[m * 3 + 1] = -2.0 * u;
        c.upow[m * 3 + 2] = u * u;
    }
    return MGBF_OK;
}

}  // namespace

extern "C" int mgbf_radial_filter_noalloc(const float* x, float* y, int nk, int im, int jm, int p, double mg_ampl02,
                                          int hx, int hy, double weight, void* stream) {
    using mgbf::report_error;
    if (!x || !y || nk <= 0 || im <= 0 || jm <= 0) return report_error(MGBF_ERR_ARG, "null field or non-positive size");
    mgbf::HMomCoefs<double> coefs;
    int R = 0;
    double s = 0.0;
    int rc = moment_setup(p, mg_ampl02, hx, hy, coefs, R, s);
    if (rc) return rc;
    if (R > im || R > jm) return report_error(MGBF_ERR_DIVISIBILITY, "filter reach exceeds the grid");
    const int halo = R + 8;  // mirrored x halo of the intermediate fields
    const size_t per = (size_t)nk * (size_t)(im + 2 * halo) * (size_t)jm;
    if (per > MGBF_NOALLOC_MAX_ELEMS)
        return report_error(MGBF_ERR_ARG,
                            "field too large for the allocation-free filter: nk*(im+2*(reach+8))*jm must not exceed "
                            "MGBF_NOALLOC_MAX_ELEMS (8388608)");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return report_error(MGBF_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return report_error(MGBF_ERR_ARG, "device ordinal out of range");
    // Host code must not use g_noalloc_scratch as an address: look the device
    // address up with that device current, and keep it once the lookup has
    // succeeded.  A failed lookup (for instance one attempted during a stream
    // capture) is not remembered: the next call tries again.
    float* A = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_scratch_mutex[dev]);
        if (!g_scratch_addr[dev]) {
            void* p_ = nullptr;
            e = cudaGetSymbolAddress(&p_, g_noalloc_scratch);
            if (e != cudaSuccess || !p_) {
                cudaGetLastError();
                return report_error(MGBF_ERR_CUDA, e != cudaSuccess ? cudaGetErrorString(e)
                                                                    : "cudaGetSymbolAddress returned no address");
            }
            g_scratch_addr[dev] = static_cast<float*>(p_);
        }
        A = g_scratch_addr[dev];
    }
    float* B = A + per;
    mgbf::View vin, vA, vB, vout;
    vin.p = const_cast<float*>(x); vin.si = nk; vin.sj = (long long)nk * im;
    vA.p = A + (size_t)nk * halo; vA.si = nk; vA.sj = (long long)nk * (im + 2 * halo);
    vB.p = B + (size_t)nk * halo; vB.si = nk; vB.sj = vA.sj;
    vout.p = y; vout.si = nk; vout.sj = (long long)nk * im;
    // padded copy of x (mirrored x halo), then the two radial passes
    rc = mgbf::launch_copy(mgbf::DType::F32, vin, vA, nk, im, jm, R, stream);
    if (rc) return report_error(MGBF_ERR_CUDA, cudaGetErrorString((cudaError_t)rc));
    mgbf::HMomArgs a;
    a.in = vA; a.out = vB; a.nk = nk; a.I = im; a.J = jm;
    a.mirror_hx = R; a.halo = halo; a.scale = weight * s; a.tmap = nullptr; a.status = nullptr;
    const int tx = mgbf::hmom_tx_for(4, R);
    const long long w0 = (long long)((nk + 31) / 32) * ((im + tx - 1) / tx);
    const long long nz = ((long long)mgbf::device_sm_count() * 24 + w0 - 1) / w0;
    int rows = (int)((jm + nz - 1) / nz);
    a.rows = rows > 4 * R ? rows : (jm < 4 * R ? jm : 4 * R);
    rc = mgbf::launch_hmom(mgbf::DType::F32, R, p, a, coefs, stream);
    if (rc) return report_error(MGBF_ERR_CUDA, rc > 0 ? cudaGetErrorString((cudaError_t)rc) : "radial kernel launch");
    a.in = vB; a.out = vout; a.mirror_hx = 0; a.scale = s;
    rc = mgbf::launch_hmom(mgbf::DType::F32, R, p, a, coefs, stream);
    if (rc) return report_error(MGBF_ERR_CUDA, rc > 0 ? cudaGetErrorString((cudaError_t)rc) : "radial kernel launch");
    return MGBF_OK;
}
