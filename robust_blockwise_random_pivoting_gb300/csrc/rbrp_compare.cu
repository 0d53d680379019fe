// rbrp_compare.cu - the reference's comparison IDs behind its own C++ signatures:
// RandLUPP_OS and RandCPQR_OS (gpu/rid.hpp, gpu/randLUPP_OS.cu:14-119,
// gpu/randCPQR_OS.cu:20-111) and the CPQR baseline (gpu/id_cpqr.hpp,
// gpu/id_cpqr.cu:30-172), composed from this library's kernels:
//
//  * sketch Y = G A with 2k rows, G ~ N(0, 1/m) (rbrp_sketch_gaussian_f32 on an
//    FP32 copy of A), widened to FP64;
//  * the skeleton: LU pivots of Y(1:k, :)^T (rbrp_lupp_pivots_f64) or greedy
//    column-pivoted QR of Y(1:k, :) (rbrp_id_f64, b = 1);
//  * T = Y(:, S)^+ Y(:, rd) by the fixed-skeleton run on Y (rbrp_fixed_id_f64),
//    rows in skeleton order and columns in rd order, as the reference's
//    Compute_interpolation_matrix returns them (gpu/interp.cu:45-105).
#include <algorithm>
#include <cmath>
#include <vector>

#include "rbrp_internal.h"

namespace rbrp {
namespace {

__global__ void k_to_f32(const double* __restrict__ A, int64_t lda, int m, int n, float* __restrict__ B) {
  const int64_t total = (int64_t)m * n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e % m, c = e / m;
    B[e] = (float)A[r + c * lda];
  }
}

__global__ void k_to_f64(const float* __restrict__ A, int64_t count, double* __restrict__ B) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count; e += (int64_t)gridDim.x * blockDim.x)
    B[e] = (double)A[e];
}

// pos[perm[p]] = p
__global__ void k_inverse_perm(const int* __restrict__ perm, int n, int* __restrict__ pos) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) pos[perm[p]] = p;
}

// Tout(a, j) = Trun(pos[S[a]], pos[rd[j]] - k): T of a run (rows and columns in the
// run's own order) with rows in S order and columns in rd order.  Both k x (n - k), ld k.
__global__ void k_reorder_T(const double* __restrict__ Trun, const int* __restrict__ pos, const int* __restrict__ S,
                            const int* __restrict__ rd, int k, int nc, double* __restrict__ Tout) {
  const int64_t total = (int64_t)k * nc;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int a = (int)(e % k), j = (int)(e / k);
    Tout[e] = Trun[pos[S[a]] + (int64_t)(pos[rd[j]] - k) * k];
  }
}

int grid_for(int64_t count) { return (int)std::max<int64_t>(1, std::min<int64_t>(4864, (count + 255) / 256)); }

// Device scratch freed on scope exit.
struct Scratch {
  std::vector<void*> ptrs;
  template <typename T>
  T* get(size_t count) {
    void* p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(1, count) * sizeof(T)) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    ptrs.push_back(p);
    return static_cast<T*>(p);
  }
  ~Scratch() {
    for (void* p : ptrs) cudaFree(p);
  }
};

// Y64 (2k x n, ld 2k) = G A for A (m x n FP64, ld m), G 2k x m ~ N(0, 1/m).
rbrp_status sketch_f64(rbrp_handle h, Scratch& sc, const double* dA, int m, int n, int k, uint64_t seed,
                       double** Y64) {
  const int r = 2 * k;
  float* A32 = sc.get<float>((size_t)m * n);
  float* Y32 = sc.get<float>((size_t)r * n);
  *Y64 = sc.get<double>((size_t)r * n);
  if (!A32 || !Y32 || !*Y64) return set_error(h, RBRP_ERR_ALLOC, "cudaMalloc(sketch buffers)");
  k_to_f32<<<grid_for((int64_t)m * n), 256, 0, h->stream>>>(dA, m, m, n, A32);
  rbrp_status s = rbrp_sketch_gaussian_f32(h, r, m, n, A32, m, seed, (float)(1.0 / std::sqrt((double)m)), Y32, r);
  if (s != RBRP_OK) return s;
  k_to_f64<<<grid_for((int64_t)r * n), 256, 0, h->stream>>>(Y32, (int64_t)r * n, *Y64);
  return cuda_check(h, cudaGetLastError(), "sketch conversion kernels");
}

// T (k x (n - k), rows in S order, columns in rd order) of the fixed-skeleton run on
// Y64 (2k x n) with the skeleton dS = perm[:k] and rd = perm[k:] of dPerm.
rbrp_status interpolation_on_sketch(rbrp_handle h, Scratch& sc, const double* Y64, int k, int n, const int* dPerm,
                                    double* dT) {
  const int r = 2 * k, nc = n - k;
  int* perm_run = sc.get<int>(n);
  int* pos = sc.get<int>(n);
  if (!perm_run || !pos) return set_error(h, RBRP_ERR_ALLOC, "cudaMalloc(run permutation)");
  rbrp_result res;
  rbrp_status s = rbrp_fixed_id_f64(h, r, n, Y64, r, dPerm, k, std::min(64, k), perm_run, &res);
  if (s != RBRP_OK) return s;
  if (res.k != k) return set_error(h, RBRP_ERR_NUMERIC, "the sketch's skeleton columns are linearly dependent");
  if (nc > 0) {
    k_inverse_perm<<<grid_for(n), 256, 0, h->stream>>>(perm_run, n, pos);
    k_reorder_T<<<grid_for((int64_t)k * nc), 256, 0, h->stream>>>(static_cast<const double*>(h->T), pos, dPerm,
                                                                   dPerm + k, k, nc, dT);
  }
  return cuda_check(h, cudaStreamSynchronize(h->stream), "interpolation on the sketch");
}

rbrp_status check_args(const double* dA, int m, int n, int k) {
  if (!dA || m < 1 || n < 1 || k < 1 || k > std::min(m, n)) return RBRP_ERR_INVALID_ARG;
  return RBRP_OK;
}

}  // namespace
}  // namespace rbrp

using namespace rbrp;

extern "C" rbrp_status rbrp_RandLUPP_OS(const double* dA, int m, int n, int k, int** sk, int** rd, double** T,
                                        double* flops, uint64_t seed) {
  if (!sk || !rd || !T) return RBRP_ERR_INVALID_ARG;
  *sk = nullptr;
  *rd = nullptr;
  *T = nullptr;
  rbrp_status s = check_args(dA, m, n, k);
  if (s != RBRP_OK) return s;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return RBRP_ERR_CUDA;
  rbrp_handle h = nullptr;
  if ((s = rbrp_create(&h, dev)) != RBRP_OK) return s;
  const int nc = n - k;
  {
    Scratch sc;
    double* Y64 = nullptr;
    int* perm = sc.get<int>(n);
    s = perm ? sketch_f64(h, sc, dA, m, n, k, seed, &Y64) : RBRP_ERR_ALLOC;
    if (s == RBRP_OK) s = rbrp_lupp_pivots_f64(h, k, n, Y64, 2 * k, perm, nullptr);
    double* Tout = nullptr;
    if (s == RBRP_OK) {
      if (cudaMalloc((void**)sk, sizeof(int) * (size_t)k) != cudaSuccess ||
          cudaMalloc((void**)rd, sizeof(int) * (size_t)std::max(nc, 1)) != cudaSuccess ||
          cudaMalloc((void**)&Tout, sizeof(double) * std::max<size_t>(1, (size_t)k * nc)) != cudaSuccess) {
        cudaGetLastError();
        s = RBRP_ERR_ALLOC;
      }
    }
    if (s == RBRP_OK) s = interpolation_on_sketch(h, sc, Y64, k, n, perm, Tout);
    if (s == RBRP_OK) {
      cudaMemcpy(*sk, perm, sizeof(int) * (size_t)k, cudaMemcpyDeviceToDevice);
      if (nc > 0) cudaMemcpy(*rd, perm + k, sizeof(int) * (size_t)nc, cudaMemcpyDeviceToDevice);
      *T = Tout;
      // the reference's count (gpu/randLUPP_OS.cu:102)
      if (flops) *flops = 2.0 * m * n * k + 2.0 * m * k * k / 3.0 + 1.0 * k * k * (double)(m - k);
      if (cudaDeviceSynchronize() != cudaSuccess) s = RBRP_ERR_CUDA;
    }
    if (s != RBRP_OK) {
      if (*sk) cudaFree(*sk);
      if (*rd) cudaFree(*rd);
      if (Tout) cudaFree(Tout);
      *sk = nullptr;
      *rd = nullptr;
      *T = nullptr;
    }
  }
  rbrp_destroy(h);
  return s;
}

extern "C" rbrp_status rbrp_RandCPQR_OS(const double* dA, int m, int n, int k, int* h_sk, int* h_rd, double** T,
                                        double* flops, uint64_t seed) {
  if (!h_sk || !h_rd || !T) return RBRP_ERR_INVALID_ARG;
  *T = nullptr;
  rbrp_status s = check_args(dA, m, n, k);
  if (s != RBRP_OK) return s;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return RBRP_ERR_CUDA;
  rbrp_handle h = nullptr;
  if ((s = rbrp_create(&h, dev)) != RBRP_OK) return s;
  const int nc = n - k;
  {
    Scratch sc;
    double* Y64 = nullptr;
    int* perm = sc.get<int>(n);
    s = perm ? sketch_f64(h, sc, dA, m, n, k, seed, &Y64) : RBRP_ERR_ALLOC;
    if (s == RBRP_OK) {
      // the skeleton: column-pivoted QR of the first k rows of the sketch (greedy b = 1)
      rbrp_params p;
      rbrp_params_default(&p);
      p.b = 1;
      p.sampler = RBRP_SAMPLER_GREEDY;
      p.tol = 0.0;
      p.kmax = k;
      p.compute_T = 0;
      rbrp_result r;
      s = rbrp_id_f64(h, k, n, Y64, 2 * k, &p, perm, &r);
      if (s == RBRP_OK && r.k != k) s = set_error(h, RBRP_ERR_NUMERIC, "the sketch has rank below k");
    }
    double* Tout = nullptr;
    if (s == RBRP_OK && cudaMalloc((void**)&Tout, sizeof(double) * std::max<size_t>(1, (size_t)k * nc)) != cudaSuccess) {
      cudaGetLastError();
      s = RBRP_ERR_ALLOC;
    }
    if (s == RBRP_OK) s = interpolation_on_sketch(h, sc, Y64, k, n, perm, Tout);
    if (s == RBRP_OK) {
      cudaMemcpy(h_sk, perm, sizeof(int) * (size_t)k, cudaMemcpyDeviceToHost);
      if (nc > 0) cudaMemcpy(h_rd, perm + k, sizeof(int) * (size_t)nc, cudaMemcpyDeviceToHost);
      *T = Tout;
      // sketch GEMM, QR of the k x n panel, and the interpolation solve on the 2k x n sketch
      if (flops) *flops = 2.0 * (2.0 * k) * m * n + 4.0 * k * k * (double)n + 2.0 * k * k * (double)nc;
    } else if (Tout) {
      cudaFree(Tout);
    }
  }
  rbrp_destroy(h);
  return s;
}

extern "C" rbrp_status rbrp_CPQR(int m, int n, const double* dA, const int* ranks, int nranks, double* err,
                                 double* t_ranks, double* t_cpqr, double* flops) {
  if (!dA || m < 1 || n < 1 || nranks < 1 || !ranks || !err) return RBRP_ERR_INVALID_ARG;
  int kmax = 0;
  for (int q = 0; q < nranks; ++q) {
    if (ranks[q] < 0 || ranks[q] > std::min(m, n)) return RBRP_ERR_INVALID_ARG;
    kmax = std::max(kmax, ranks[q]);
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return RBRP_ERR_CUDA;
  rbrp_handle h = nullptr;
  rbrp_status s = rbrp_create(&h, dev);
  if (s != RBRP_OK) return s;
  rbrp_params p;
  rbrp_params_default(&p);
  p.b = 1;
  p.sampler = RBRP_SAMPLER_GREEDY;
  p.tol = 0.0;
  p.kmax = std::max(kmax, 1);
  p.compute_T = 0;
  rbrp_result r;
  s = rbrp_id_f64(h, m, n, dA, m, &p, nullptr, &r);
  if (s == RBRP_OK) {
    // one block per pivot: trace entry t holds rank t + 1 (squared relative residual, seconds)
    int nb = 0;
    s = rbrp_get_trace(h, nullptr, nullptr, nullptr, 0, &nb);
    std::vector<int> tr_rank(std::max(nb, 1));
    std::vector<double> tr_err(std::max(nb, 1)), tr_t(std::max(nb, 1));
    if (s == RBRP_OK) s = rbrp_get_trace(h, tr_rank.data(), tr_err.data(), tr_t.data(), nb, &nb);
    for (int q = 0; s == RBRP_OK && q < nranks; ++q) {
      const int kq = ranks[q];
      double e = 1.0, t = 0.0;
      for (int b = 0; b < nb; ++b)
        if (tr_rank[b] == kq) { e = tr_err[b]; t = tr_t[b] * 1e-3; }
      if (kq == 0) e = 1.0;
      else if (kq > r.k) e = 0.0;   // the residual vanished before rank kq
      err[q] = e;
      if (t_ranks) t_ranks[q] = t;
    }
    if (t_cpqr) *t_cpqr = nb > 0 ? tr_t[nb - 1] * 1e-3 : 0.0;
    if (flops) *flops = 4.0 * m * (double)n * r.k - 2.0 * (double)r.k * r.k * (m + n) + 4.0 * std::pow((double)r.k, 3) / 3.0;
  }
  rbrp_destroy(h);
  return s;
}
