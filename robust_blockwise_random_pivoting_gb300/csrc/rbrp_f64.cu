// FP64 instantiation of the RBRP block loop (the plain form).
#include "rbrp_driver.cuh"

namespace rbrp {
template rbrp_status run_rbrp<double>(rbrp_handle, int, int, const double*, int64_t, const rbrp_params&,
                                      int*, rbrp_result*);
}
