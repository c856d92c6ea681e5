// Moment-form radial beta kernels for __nv_bfloat16 storage, reaches 10-24 (the
// other half of mgbf_hbeta_bf16.cu, split so the build compiles them in
// parallel).
#include "mgbf_hbeta.cuh"

namespace mgbf {

int hmom_dispatch_bf16_b(int R, const HMomArgs& a, const HMomCoefs<double>& c, cudaStream_t s) {
    switch (R) {
#define MGBF_CASE(r) \
    case r:          \
        return run_hmom<r, 2, __nv_bfloat16>(a, c, s);
        MGBF_HMOM_REACHES_B(MGBF_CASE)
#undef MGBF_CASE
        default:
            return -1;
    }
}

int hmom_persist_dispatch_bf16_b(int R, const HMomPersistArgs& pa, const HMomMaps& maps, const HMomCoefs<double>& c,
                                cudaStream_t s) {
    switch (R) {
#define MGBF_CASE(r) \
    case r:          \
        return run_hmom_persist<r, 2, __nv_bfloat16>(pa, maps, c, s);
        MGBF_HMOM_REACHES_B(MGBF_CASE)
#undef MGBF_CASE
        default:
            return -1;
    }
}

}  // namespace mgbf
