/*
 * rbrp_gb300.hpp - C++ drop-in shims over the C ABI of rbrp_gb300.h.
 *
 * Same names, argument meaning and output containers as the reference's
 * gpu/rbrp.hpp:6-8 (RBRP) and gpu/rid.hpp:5-7 (RandAdapLUPP's contract, here
 * with RBRP pivoting).  Errors are reported by return value (the reference
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

}  // namespace rbrp_gb300

#endif /* RBRP_GB300_HPP */
