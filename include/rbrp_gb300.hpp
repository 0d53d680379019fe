/*
 * rbrp_gb300.hpp - C++ drop-in shims over the C ABI of rbrp_gb300.h.
 *
 * Same names, argument meaning and output containers as the reference's
 * gpu/rbrp.hpp:6-8 (RBRP), gpu/rid.hpp:5-7 (RandAdapLUPP's contract, here
 * with RBRP pivoting), gpu/rid.hpp (RandLUPP_OS, RandCPQR_OS) and
 * gpu/id_cpqr.hpp (CPQR).  Errors are reported by return value (the reference
 * asserts or exits, gpu/util.hpp:16-24,79-84).  Header-only; link librbrp_gb300.so.
 */
#ifndef RBRP_GB300_HPP
#define RBRP_GB300_HPP

#include <vector>

#include "rbrp_gb300.h"

namespace rbrp_gb300 {

/* gpu/rbrp.hpp:6-8.  A: device FP64, m x n, ld = m.  Runs to rank min(m, n);
 * ranks/error/t_ranks are cumulative per block, error is the squared relative
 * residual, times in seconds. */
inline rbrp_status RBRP(int m, int n, double* A, int blk, std::vector<int>& ranks, std::vector<double>& error,
                        std::vector<double>& t_ranks, double& t_rbrp, double& flops) {
  const int cap = m < n ? m : n;
  ranks.assign(cap, 0);
  error.assign(cap, 0.0);
  t_ranks.assign(cap, 0.0);
  int nb = 0;
  rbrp_status s = rbrp_RBRP(m, n, A, blk, ranks.data(), error.data(), t_ranks.data(), cap, &nb, &t_rbrp, &flops);
  ranks.resize(s == RBRP_OK ? nb : 0);
  error.resize(ranks.size());
  t_ranks.resize(ranks.size());
  return s;
}

/* gpu/rid.hpp:5-7 contract (tol = squared relative tolerance, blk = block size):
 * sk, rd and T are device arrays allocated here; free them with rbrp_free. */
inline rbrp_status RandAdapRBRP(const double* A, int m, int n, int*& sk, int*& rd, double*& T, int& rank,
                                double& flops, double tol = 1e-8, int blk = 16) {
  return rbrp_RandAdapRBRP(A, m, n, &sk, &rd, &T, &rank, &flops, tol, blk);
}
/* The name gpu/rid.hpp:5-7 declares, so a caller written against it compiles
 * unchanged; same arguments and results as RandAdapRBRP (RBRP pivoting). */
inline rbrp_status RandAdapLUPP(const double* A, int m, int n, int*& sk, int*& rd, double*& T, int& rank,
                                double& flops, double tol = 1e-8, int blk = 16) {
  return RandAdapRBRP(A, m, n, sk, rd, T, rank, flops, tol, blk);
}

/* gpu/rid.hpp: RandLUPP_OS and RandCPQR_OS with the reference's arguments; each
 * call draws a new sketch (Philox key = call count, as the reference's RNG
 * counter advances per call).  sk, rd (RandLUPP_OS) and T are device arrays
 * allocated here; free them with rbrp_free.  h_sk, h_rd are the caller's host
 * arrays of k and n - k ints. */
inline uint64_t& sketch_calls() {
  static uint64_t calls = 0;
  return calls;
}
inline rbrp_status RandLUPP_OS(const double* A, int m, int n, int rank, int*& sk, int*& rd, double*& T,
                               double& flops) {
  return rbrp_RandLUPP_OS(A, m, n, rank, &sk, &rd, &T, &flops, sketch_calls()++);
}
inline rbrp_status RandCPQR_OS(const double* A, int m, int n, int rank, int* h_sk, int* h_rd, double*& T,
                               double& flops) {
  return rbrp_RandCPQR_OS(A, m, n, rank, h_sk, h_rd, &T, &flops, sketch_calls()++);
}

/* gpu/id_cpqr.hpp: CPQR to the given ranks; err holds the squared relative ID
 * error at each rank, t_ranks the cumulative seconds. */
inline rbrp_status CPQR(int m, int n, double* A, const std::vector<int> ranks, std::vector<double>& err,
                        std::vector<double>& t_ranks, double& t_cpqr, double& flops) {
  err.assign(ranks.size(), 0.0);
  t_ranks.assign(ranks.size(), 0.0);
  if (ranks.empty()) return RBRP_ERR_INVALID_ARG;
  return rbrp_CPQR(m, n, A, ranks.data(), (int)ranks.size(), err.data(), t_ranks.data(), &t_cpqr, &flops);
}

}  // namespace rbrp_gb300

#endif /* RBRP_GB300_HPP */
