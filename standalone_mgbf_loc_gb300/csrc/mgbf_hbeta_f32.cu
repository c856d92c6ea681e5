// Moment-form radial beta kernels instantiated for float storage (one
// translation unit per storage type so the build compiles them in parallel).
#include "mgbf_hbeta.cuh"

namespace mgbf {

int hmom_dispatch_f32(int R, const HMomArgs& a, const HMomCoefs<double>& c, cudaStream_t s) {
    switch (R) {
#define MGBF_CASE(r) \
    case r:          \
        return run_hmom<r, 2, float>(a, c, s);
        MGBF_HMOM_REACHES(MGBF_CASE)
#undef MGBF_CASE
        default:
            return -1;
    }
}

}  // namespace mgbf
