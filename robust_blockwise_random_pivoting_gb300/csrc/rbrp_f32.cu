// FP32-storage instantiation of the RBRP block loop (the mixed-precision form:
// FP32 A, Q and projections; double-float (pairs of FP32) panel factorisation,
// sums and T solve; FP64 sampler weights).
#include "rbrp_driver.cuh"

namespace rbrp {
template rbrp_status run_rbrp<float>(rbrp_handle, int, int, const float*, int64_t, const rbrp_params&,
                                     int*, rbrp_result*);
}
