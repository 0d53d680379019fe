// driver_dropin.cpp - a caller of the reference's C++ entry points, linked to
// librbrp_gb300.so through include/rbrp_gb300.hpp.
//
// It calls RBRP (gpu/rbrp.hpp:6-8) and RandAdapLUPP (gpu/rid.hpp:5-7) the way
// the reference's driver does (gpu/driver.cpp:177: a statement whose result is
// ignored, a device matrix from cudaMalloc, host std::vectors for the trace),
// so it also shows that such a caller compiles unchanged against the shims.
//
//   driver_dropin MATRIX BLK TOL OUT
// MATRIX: int32 m, int32 n, then m*n FP64 column major.  Prints the RBRP trace
// ("rank squared-relative-residual" per block) on stdout and writes the
// RandAdapLUPP results to OUT: int32 rank, int32 sk[rank], int32 rd[n-rank],
// FP64 T[rank*(n-rank)] (column major, ld = rank).
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "rbrp_gb300.hpp"

using namespace rbrp_gb300;

#define CHECK_CUDA(x)                                                   \
  do {                                                                  \
    cudaError_t e_ = (x);                                               \
    if (e_ != cudaSuccess) {                                            \
      std::fprintf(stderr, "%s: %s\n", #x, cudaGetErrorString(e_));     \
      return 2;                                                         \
    }                                                                   \
  } while (0)

int main(int argc, char** argv) {
  if (argc != 5) {
    std::fprintf(stderr, "usage: driver_dropin MATRIX BLK TOL OUT\n");
    return 1;
  }
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 1;
  int m = 0, n = 0;
  if (std::fread(&m, 4, 1, f) != 1 || std::fread(&n, 4, 1, f) != 1 || m < 1 || n < 1) return 1;
  std::vector<double> hA((size_t)m * n);
  if (std::fread(hA.data(), 8, hA.size(), f) != hA.size()) return 1;
  std::fclose(f);
  const int blk = std::atoi(argv[2]);
  const double tol = std::atof(argv[3]);

  double* dA = nullptr;
  CHECK_CUDA(cudaMalloc(&dA, hA.size() * sizeof(double)));
  CHECK_CUDA(cudaMemcpy(dA, hA.data(), hA.size() * sizeof(double), cudaMemcpyHostToDevice));

  // gpu/driver.cpp:177
  std::vector<int> ranks;
  std::vector<double> error, t_ranks;
  double t_rbrp = 0.0, flops = 0.0;
  RBRP(m, n, dA, blk, ranks, error, t_ranks, t_rbrp, flops);
  if (ranks.empty()) {
    std::fprintf(stderr, "RBRP returned no blocks\n");
    return 3;
  }
  std::printf("blocks %zu t_rbrp %.6f flops %.6e\n", ranks.size(), t_rbrp, flops);
  for (size_t i = 0; i < ranks.size(); ++i) std::printf("%d %.17g\n", ranks[i], error[i]);

  // gpu/rid.hpp:5-7
  int *sk = nullptr, *rd = nullptr;
  double* T = nullptr;
  int rank = 0;
  double fl = 0.0;
  if (RandAdapLUPP(dA, m, n, sk, rd, T, rank, fl, tol, blk) != RBRP_OK) {
    std::fprintf(stderr, "RandAdapLUPP failed\n");
    return 4;
  }
  std::vector<int> hsk(rank), hrd(n - rank);
  std::vector<double> hT((size_t)rank * (n - rank));
  if (rank > 0) CHECK_CUDA(cudaMemcpy(hsk.data(), sk, rank * sizeof(int), cudaMemcpyDeviceToHost));
  if (n - rank > 0) CHECK_CUDA(cudaMemcpy(hrd.data(), rd, (n - rank) * sizeof(int), cudaMemcpyDeviceToHost));
  if (!hT.empty()) CHECK_CUDA(cudaMemcpy(hT.data(), T, hT.size() * sizeof(double), cudaMemcpyDeviceToHost));
  rbrp_free(sk);
  rbrp_free(rd);
  rbrp_free(T);
  cudaFree(dA);

  FILE* o = std::fopen(argv[4], "wb");
  if (!o) return 1;
  std::fwrite(&rank, 4, 1, o);
  std::fwrite(hsk.data(), 4, hsk.size(), o);
  std::fwrite(hrd.data(), 4, hrd.size(), o);
  std::fwrite(hT.data(), 8, hT.size(), o);
  std::fclose(o);
  std::printf("rank %d\n", rank);
  return 0;
}
