/*
 * rbrp_gb300_testing.h - diagnostic entry points of the GB300 RBRP library.
 *
 * Not part of the reference's interface (no counterpart in gpu/rbrp.hpp or
 * gpu/rid.hpp): they let tests and benchmarks select between the kernel
 * variants that compute the same quantity, so each can be checked against
 * the other and against the CPU oracle, and shorten the limit of the bounded
 * device-side waits so that the timeout path can be tested.
 */
#ifndef RBRP_GB300_TESTING_H
#define RBRP_GB300_TESTING_H

#include "rbrp_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Projection and update kernels of the FP32 residual form: 0 = tcgen05 /
 * TMEM / TMA 3xTF32 (default), 1 = CUDA-core FFMA.  Both accumulate to
 * ~1e-8 relative. */
rbrp_status rbrp_set_variant(rbrp_handle h, int variant);

/* T = R11^{-1} R12 block updates: 0 = double-float on the FP32 pipe (default,
 * ~48 significant bits), 1 = FP64 pipe. */
rbrp_status rbrp_set_tsolve_fp64(rbrp_handle h, int on);

/* Limit, in SM clock cycles, of the bounded device-side waits of kernels launched
 * through this handle: the grid barrier of the LU pivots (rbrp_lupp_pivots_f64)
 * and the mbarrier waits of the tcgen05 kernels (projection, update, the
 * adjoint's and the sketch's GEMMs).  0 restores the default
 * (~2 s).  A limit of a few cycles makes a wait run out: the kernel then exits
 * cleanly and the call returns RBRP_ERR_DEVICE_TIMEOUT, which is how the tests
 * exercise that path without faulting or hanging a GPU.  The waits that let an
 * aborting kernel's own copies and MMAs finish keep the default limit. */
rbrp_status rbrp_set_wait_budget(rbrp_handle h, long long cycles);

#ifdef __cplusplus
}
#endif
#endif /* RBRP_GB300_TESTING_H */
