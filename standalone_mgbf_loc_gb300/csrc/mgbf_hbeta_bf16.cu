// Moment-form radial beta kernels for __nv_bfloat16 storage, reaches 4-8; reaches
// 10-24 are in mgbf_hbeta_bf16_b.cu (separate translation units compile in
// parallel).
#include "mgbf_hbeta.cuh"

namespace mgbf {

int hmom_dispatch_bf16_b(int R, const HMomArgs& a, const HMomCoefs<double>& c, cudaStream_t s);
int hmom_persist_dispatch_bf16_b(int R, const HMomPersistArgs& pa, const HMomMaps& maps, const HMomCoefs<double>& c,
                                cudaStream_t s);

int hmom_dispatch_bf16(int R, const HMomArgs& a, const HMomCoefs<double>& c, cudaStream_t s) {
    switch (R) {
#define MGBF_CASE(r) \
    case r:          \
        return run_hmom<r, 2, __nv_bfloat16>(a, c, s);
        MGBF_HMOM_REACHES_A(MGBF_CASE)
#undef MGBF_CASE
        default:
            return hmom_dispatch_bf16_b(R, a, c, s);
    }
}

int hmom_persist_dispatch_bf16(int R, const HMomPersistArgs& pa, const HMomMaps& maps, const HMomCoefs<double>& c,
                              cudaStream_t s) {
    switch (R) {
#define MGBF_CASE(r) \
    case r:          \
        return run_hmom_persist<r, 2, __nv_bfloat16>(pa, maps, c, s);
        MGBF_HMOM_REACHES_A(MGBF_CASE)
#undef MGBF_CASE
        default:
            return hmom_persist_dispatch_bf16_b(R, pa, maps, c, s);
    }
}

}  // namespace mgbf
