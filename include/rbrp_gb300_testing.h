/*
 * rbrp_gb300_testing.h - diagnostic entry points of the GB300 RBRP library.
 *
 * Not part of the reference's interface (no counterpart in gpu/rbrp.hpp or
 * gpu/rid.hpp): they let tests and benchmarks select between the kernel
 * variants that compute the same quantity, so each can be checked against
 * the other and against the CPU oracle.
 */
#ifndef RBRP_GB300_TESTING_H
#define RBRP_GB300_TESTING_H

#include "rbrp_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Projection kernel of the FP32 residual form: 0 = tcgen05 / TMEM / TMA
 * (default), 1 = CUDA-core FFMA.  Both accumulate to ~1e-8 relative. */
rbrp_status rbrp_set_variant(rbrp_handle h, int variant);

/* T = R11^{-1} R12 block updates: 0 = double-float on the FP32 pipe (default,
 * ~48 significant bits), 1 = FP64 pipe. */
rbrp_status rbrp_set_tsolve_fp64(rbrp_handle h, int on);

#ifdef __cplusplus
}
#endif
#endif /* RBRP_GB300_TESTING_H */
