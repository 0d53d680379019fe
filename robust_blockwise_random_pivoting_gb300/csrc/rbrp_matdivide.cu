// rbrp_matdivide.cu - interpolation through a truncated-SVD pseudo-inverse.
//
// The notebook's matdivide (python/RBRP.ipynb cell 2 lines 111-126) computes
// A * pinv(B) from the SVD of B, keeping the singular values above an absolute
// cutoff tol (TOL_FP = 1e-12, cell 0 line 26); get_rpid_error uses it for the
// interpolation matrix of every blocked run (cell 11 lines 226-232), where L1
// is only block triangular and may be ill-conditioned.  Here R11 is exactly
// triangular and T = R11^{-1} R12 is a triangular solve, but a skeleton given
// from outside (fixed-skeleton runs) can be rank deficient; this is the
// rank-revealing form for it: X = pinv_tol(B) C.
//
// The SVD is a one-sided Jacobi (Hestenes) iteration in FP64: column pairs of
// B are rotated until every pair is orthogonal to working precision, then the
// column norms are the singular values (to high relative accuracy, so small
// ones are resolved as LAPACK's gesdd resolves them), B V = U diag(s).  Pairs
// follow a round-robin schedule (q/2 disjoint pairs per launch, q - 1 launches
// per sweep), one warp per pair.  Then X = V diag(w) B^T C with w_j = 1/s_j^2
// for s_j > tol and 0 otherwise (B_j / s_j = U_j), by two small FP64 GEMMs.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "rbrp_internal.h"

namespace rbrp {
namespace {

constexpr int MD_THREADS = 256;
constexpr int MD_PAIRS = MD_THREADS / 32;  // one warp per column pair
constexpr int MD_MAX_SWEEPS = 60;

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Pair i of round r of the round-robin schedule over qq (even) players: player
// qq - 1 meets r, and (r + i, r - i) mod (qq - 1) otherwise.
__device__ __forceinline__ void rr_pair(int qq, int r, int i, int& a, int& b) {
  const int m = qq - 1;
  if (i == 0) {
    a = m;
    b = r;
  } else {
    a = (r + i) % m;
    b = (r - i + m) % m;
  }
}

// One round: every pair (a, b) of columns of B (p x q, ld ldb) is rotated so
// that b_a . b_b = 0; V (q x q, ld q) takes the same rotation.  The largest
// |b_a . b_b| / (|b_a| |b_b|) seen before rotating is folded into *off (its bit
// pattern: non-negative doubles order like their bits).  A column whose squared
// norm is at most floor2 (rounding noise of ||B||_F, what an exactly dependent
// column leaves) counts as orthogonal to every other.
__global__ void __launch_bounds__(MD_THREADS) k_jacobi_round(double* __restrict__ B, int64_t ldb,
                                                             double* __restrict__ V, int p, int q, int qq, int r,
                                                             double thresh, double floor2,
                                                             unsigned long long* __restrict__ off) {
  const int lane = threadIdx.x & 31;
  const int pair = blockIdx.x * MD_PAIRS + (threadIdx.x >> 5);
  if (pair >= qq / 2) return;
  int a, b;
  rr_pair(qq, r, pair, a, b);
  if (a >= q || b >= q) return;  // the padding player of an odd q
  if (a > b) {
    const int t = a;
    a = b;
    b = t;
  }
  double* x = B + (int64_t)a * ldb;
  double* y = B + (int64_t)b * ldb;
  double al = 0.0, be = 0.0, ga = 0.0;
  for (int i = lane; i < p; i += 32) {
    const double u = x[i], v = y[i];
    al = fma(u, u, al);
    be = fma(v, v, be);
    ga = fma(u, v, ga);
  }
  al = warp_sum_d(al);
  be = warp_sum_d(be);
  ga = warp_sum_d(ga);
  if (al <= floor2 || be <= floor2 || ga == 0.0) return;
  const double rel = fabs(ga) / (sqrt(al) * sqrt(be));
  if (lane == 0) atomicMax(off, (unsigned long long)__double_as_longlong(rel));
  if (!(rel > thresh)) return;
  // rotation angle that zeroes the off-diagonal entry of [al ga; ga be]
  const double zeta = (be - al) / (2.0 * ga);
  const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
  const double c = 1.0 / sqrt(1.0 + t * t), s = c * t;
  for (int i = lane; i < p; i += 32) {
    const double u = x[i], v = y[i];
    x[i] = c * u - s * v;
    y[i] = s * u + c * v;
  }
  double* va = V + (int64_t)a * q;
  double* vb = V + (int64_t)b * q;
  for (int i = lane; i < q; i += 32) {
    const double u = va[i], v = vb[i];
    va[i] = c * u - s * v;
    vb[i] = s * u + c * v;
  }
}

// V = I (q x q); off = 0.
__global__ void k_md_init(double* __restrict__ V, int q, unsigned long long* __restrict__ off) {
  const int64_t total = (int64_t)q * q;
  for (int64_t z = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; z < total; z += (int64_t)gridDim.x * blockDim.x)
    V[z] = (z % q) == (z / q) ? 1.0 : 0.0;
  if (blockIdx.x == 0 && threadIdx.x == 0) *off = 0ull;
}

// Copy of B (p x q, ld ldb) into the workspace (ld p).
__global__ void k_md_copy(const double* __restrict__ B, int64_t ldb, int p, int q, double* __restrict__ W) {
  const int64_t total = (int64_t)p * q;
  for (int64_t z = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; z < total; z += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = z / p, r = z % p;
    W[z] = B[r + c * ldb];
  }
}

// ||B||_F^2 of the workspace copy (one CTA, fixed order).
__global__ void __launch_bounds__(MD_THREADS) k_md_fro(const double* __restrict__ B, int64_t total,
                                                       double* __restrict__ out) {
  __shared__ double red[32];
  double s = 0.0;
  for (int64_t z = threadIdx.x; z < total; z += MD_THREADS) s = fma(B[z], B[z], s);
  s = block_sum(s, red);
  if (threadIdx.x == 0) *out = s;
}

// R11 (k x k, upper part of the row-major R, ld n) and R12 (k x (n - k)) as
// column-major matrices with leading dimension k.
__global__ void k_md_split_R(const double* __restrict__ R, int n, int k, double* __restrict__ R11,
                             double* __restrict__ R12) {
  const int64_t total = (int64_t)k * n;
  for (int64_t z = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; z < total; z += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(z % k);
    const int64_t c = z / k;
    const double v = R[(int64_t)r * n + c];
    if (c < k)
      R11[r + c * k] = r <= c ? v : 0.0;
    else
      R12[r + (c - k) * k] = v;
  }
}

// w_j = 1 / |b_j|^2 for |b_j| > tol, else 0 (one warp per column); rank count.
__global__ void __launch_bounds__(MD_THREADS) k_md_weights(const double* __restrict__ B, int p, int q, double tol,
                                                           double* __restrict__ w, int* __restrict__ rank) {
  const int lane = threadIdx.x & 31;
  const int j = blockIdx.x * MD_PAIRS + (threadIdx.x >> 5);
  if (j >= q) return;
  const double* x = B + (int64_t)j * p;
  double s = 0.0;
  for (int i = lane; i < p; i += 32) s = fma(x[i], x[i], s);
  s = warp_sum_d(s);
  if (lane == 0) {
    const bool keep = sqrt(s) > tol;
    w[j] = keep ? 1.0 / s : 0.0;
    if (keep) atomicAdd(rank, 1);
  }
}

// Z (M x N, ld ldz) = diag(scale) X^T Y or X Y, FP64, 32 x 32 output tiles.
//   TRANS: Z = diag(scale) X^T Y with X (K x M, ld ldx): Y = C (K x N).
//   !TRANS: Z = X Y with X (M x K, ld ldx), scale unused.
template <bool TRANS>
__global__ void __launch_bounds__(256) k_md_gemm(const double* __restrict__ X, int64_t ldx, const double* __restrict__ Y,
                                                 int64_t ldy, const double* __restrict__ scale, int M, int N, int K,
                                                 double* __restrict__ Z, int64_t ldz) {
  __shared__ double Xs[32][33];  // Xs[kk][row]
  __shared__ double Ys[32][33];  // Ys[kk][col]
  const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;  // 8 rows of 4
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int k0 = 0; k0 < K; k0 += 32) {
    for (int z = tid; z < 32 * 32; z += 256) {
      const int u = z & 31, v = z >> 5;  // u fast
      // X element (row r0 + ., kk): TRANS reads X[kk + row * ldx] with kk fast
      if (TRANS) {
        const int kk = u, row = v;
        Xs[kk][row] = (k0 + kk < K && r0 + row < M) ? X[(k0 + kk) + (int64_t)(r0 + row) * ldx] : 0.0;
      } else {
        const int row = u, kk = v;
        Xs[kk][row] = (k0 + kk < K && r0 + row < M) ? X[(r0 + row) + (int64_t)(k0 + kk) * ldx] : 0.0;
      }
      const int kk = u, col = v;
      Ys[kk][col] = (k0 + kk < K && c0 + col < N) ? Y[(k0 + kk) + (int64_t)(c0 + col) * ldy] : 0.0;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < 32; ++kk) {
      const double yv = Ys[kk][tx];
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[q] = fma(Xs[kk][ty + 8 * q], yv, acc[q]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int row = r0 + ty + 8 * q, col = c0 + tx;
    if (row < M && col < N) Z[row + (int64_t)col * ldz] = TRANS ? scale[row] * acc[q] : acc[q];
  }
}

// Columns perm[c0 + c] of A (m x ?, ld lda), c < nc, as an FP64 column-major
// matrix (m x nc, ld m): exact for FP32 and FP64 A.
template <typename T>
__global__ void k_md_gather(const T* __restrict__ A, int64_t lda, const int* __restrict__ perm, int c0, int m,
                            int nc, double* __restrict__ out) {
  const int64_t total = (int64_t)m * nc;
  for (int64_t z = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; z < total; z += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = z / m, r = z % m;
    out[z] = (double)A[r + (int64_t)perm[c0 + c] * lda];
  }
}

// y = x - y (elementwise, n entries)
__global__ void k_md_xmy(const double* __restrict__ x, double* __restrict__ y, int64_t n) {
  for (int64_t z = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; z < n; z += (int64_t)gridDim.x * blockDim.x)
    y[z] = x[z] - y[z];
}

// T += D (k x nc, T with leading dimension ldt, D with k); partial sums of |D|^2 and |T|^2
// per CTA into parts[2 * blockIdx.x + {0, 1}] (fixed order).
__global__ void __launch_bounds__(256) k_md_add(double* __restrict__ T, int64_t ldt, const double* __restrict__ D,
                                                int k, int nc, double* __restrict__ parts) {
  __shared__ double red[32];
  const int64_t total = (int64_t)k * nc;
  double dd = 0.0, tt = 0.0;
  for (int64_t z = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; z < total; z += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = z / k, r = z % k;
    const double d = D[z];
    const double t = T[r + c * ldt] + d;
    T[r + c * ldt] = t;
    dd = fma(d, d, dd);
    tt = fma(t, t, tt);
  }
  dd = block_sum(dd, red);
  tt = block_sum(tt, red);
  if (threadIdx.x == 0) {
    parts[2 * blockIdx.x] = dd;
    parts[2 * blockIdx.x + 1] = tt;
  }
}

}  // namespace
}  // namespace rbrp

namespace rbrp {

// X (q x nc, ld ldx) = pinv_tol(B) C for B (p x q, ld ldb) and C (p x nc, ld ldc), all
// on the handle's device; *rank = the number of singular values of B above tol.
rbrp_status matdivide(rbrp_handle h, int p, int q, int nc, const double* dB, int64_t ldb, const double* dC,
                      int64_t ldc, double tol, double* dX, int64_t ldx, int* rank) {
  // workspace: B copy (p x q) | V (q x q) | w (q) | off | rank
  auto up = [](size_t x) { return (x + 255) / 256 * 256; };
  const size_t o_v = up((size_t)p * q * sizeof(double));
  const size_t o_w = o_v + up((size_t)q * q * sizeof(double));
  const size_t o_off = o_w + up((size_t)q * sizeof(double));
  const size_t o_rank = o_off + 256;
  const size_t o_y = o_rank + 256;
  const size_t bytes = o_y + up((size_t)q * (size_t)nc * sizeof(double));
  if (h->md_bytes < bytes) {
    if (h->md_ws) cudaFree(h->md_ws);
    h->md_ws = nullptr;
    h->md_bytes = 0;
    rbrp_status s = cuda_check(h, cudaMalloc(&h->md_ws, bytes), "cudaMalloc(matdivide workspace)");
    if (s != RBRP_OK) return s;
    h->md_bytes = bytes;
  }
  unsigned char* ws = static_cast<unsigned char*>(h->md_ws);
  double* Bw = reinterpret_cast<double*>(ws);
  double* V = reinterpret_cast<double*>(ws + o_v);
  double* w = reinterpret_cast<double*>(ws + o_w);
  unsigned long long* off = reinterpret_cast<unsigned long long*>(ws + o_off);
  int* d_rank = reinterpret_cast<int*>(ws + o_rank);
  double* Y = reinterpret_cast<double*>(ws + o_y);
  cudaStream_t st = h->stream;

  k_md_copy<<<std::min<int64_t>(1216, ((int64_t)p * q + 255) / 256), 256, 0, st>>>(dB, ldb, p, q, Bw);
  k_md_init<<<std::min<int64_t>(1216, ((int64_t)q * q + 255) / 256), 256, 0, st>>>(V, q, off);
  k_md_fro<<<1, MD_THREADS, 0, st>>>(Bw, (int64_t)p * q, w);
  double fro2 = 0.0;
  rbrp_status s = cuda_check(h, cudaGetLastError(), "matdivide set-up");
  if (s == RBRP_OK) s = cuda_check(h, cudaMemcpyAsync(&fro2, w, sizeof(double), cudaMemcpyDeviceToHost, st), "norm");
  if (s == RBRP_OK) s = cuda_check(h, cudaStreamSynchronize(st), "matdivide set-up");
  if (s != RBRP_OK) return s;
  if (!std::isfinite(fro2)) return set_error(h, RBRP_ERR_NUMERIC, "matdivide: non-finite entries in B");
  const double noise = 8.0 * q * 2.220446049250313e-16;
  const double floor2 = noise * noise * fro2;
  // sweeps until no pair is further from orthogonal than sqrt(q) units of FP64 rounding
  const int qq = q + (q & 1);
  const double thresh = std::sqrt((double)q) * 2.220446049250313e-16;
  const int grid = (qq / 2 + MD_PAIRS - 1) / MD_PAIRS;
  bool converged = q == 1;
  unsigned long long h_off = 0;
  for (int sweep = 0; sweep < MD_MAX_SWEEPS && !converged; ++sweep) {
    s = cuda_check(h, cudaMemsetAsync(off, 0, sizeof(unsigned long long), st), "matdivide sweep reset");
    if (s != RBRP_OK) return s;
    for (int r = 0; r < qq - 1; ++r)
      k_jacobi_round<<<grid, MD_THREADS, 0, st>>>(Bw, p, V, p, q, qq, r, thresh, floor2, off);
    s = cuda_check(h, cudaMemcpyAsync(&h_off, off, sizeof(h_off), cudaMemcpyDeviceToHost, st), "matdivide sweep");
    if (s == RBRP_OK) s = cuda_check(h, cudaStreamSynchronize(st), "matdivide sweep");
    if (s != RBRP_OK) return s;
    double worst;
    std::memcpy(&worst, &h_off, sizeof(worst));
    if (!std::isfinite(worst)) return set_error(h, RBRP_ERR_NUMERIC, "matdivide: non-finite entries in B");
    converged = worst <= thresh;
  }
  if (!converged) return set_error(h, RBRP_ERR_NUMERIC, "matdivide: the Jacobi SVD did not converge");
  s = cuda_check(h, cudaMemsetAsync(d_rank, 0, sizeof(int), st), "matdivide rank");
  if (s != RBRP_OK) return s;
  k_md_weights<<<(q + MD_PAIRS - 1) / MD_PAIRS, MD_THREADS, 0, st>>>(Bw, p, q, tol, w, d_rank);
  if (nc > 0) {
    // Y = diag(w) B^T C (q x nc), then X = V Y (q x nc)
    k_md_gemm<true><<<dim3((nc + 31) / 32, (q + 31) / 32), 256, 0, st>>>(Bw, p, dC, ldc, w, q, nc, p, Y, q);
    k_md_gemm<false><<<dim3((nc + 31) / 32, (q + 31) / 32), 256, 0, st>>>(V, q, Y, q, nullptr, q, nc, q, dX, ldx);
  }
  int h_rank = 0;
  s = cuda_check(h, cudaMemcpyAsync(&h_rank, d_rank, sizeof(int), cudaMemcpyDeviceToHost, st), "matdivide rank");
  if (s == RBRP_OK) s = cuda_check(h, cudaStreamSynchronize(st), "matdivide");
  if (s != RBRP_OK) return s;
  if (rank) *rank = h_rank;
  return RBRP_OK;
}

}  // namespace rbrp

using namespace rbrp;

extern "C" rbrp_status rbrp_matdivide_f64(rbrp_handle h, int p, int q, int nc, const double* dB, int64_t ldb,
                                          const double* dC, int64_t ldc, double tol, double* dX, int64_t ldx,
                                          int* rank) {
  if (!h) return RBRP_ERR_INVALID_ARG;
  if (p < 1 || q < 1 || nc < 0 || !dB || ldb < p || (nc > 0 && (!dC || ldc < p || !dX || ldx < q)) ||
      !(tol >= 0.0) || !std::isfinite(tol))
    return set_error(h, RBRP_ERR_INVALID_ARG, "matdivide: need p, q >= 1, nc >= 0, ldb, ldc >= p, ldx >= q, tol >= 0");
  DeviceGuard g(h->device);
  return matdivide(h, p, q, nc, dB, ldb, dC, ldc, tol, dX, ldx, rank);
}

extern "C" rbrp_status rbrp_T_matdivide(rbrp_handle h, double tol, int* rank) {
  if (!h) return RBRP_ERR_INVALID_ARG;
  if (!h->have_result) return set_error(h, RBRP_ERR_NOT_COMPUTED, "no successful run");
  if (!(tol >= 0.0) || !std::isfinite(tol)) return set_error(h, RBRP_ERR_INVALID_ARG, "matdivide: tol must be >= 0");
  const int k = h->k, n = h->n;
  if (k <= 0 || k >= n) {
    if (rank) *rank = k;
    return RBRP_OK;  // T is empty
  }
  DeviceGuard g(h->device);
  const int nc = n - k;
  const size_t tbytes = (size_t)k * nc * sizeof(double);
  if (tbytes > h->T_bytes) {
    if (h->T) cudaFree(h->T);
    h->T = nullptr;
    h->T_bytes = 0;
    rbrp_status s = cuda_check(h, cudaMalloc((void**)&h->T, tbytes), "cudaMalloc(T)");
    if (s != RBRP_OK) return s;
    h->T_bytes = tbytes;
  }
  const size_t abytes = (size_t)k * n * sizeof(double);  // R11 | R12, column major
  if (h->md_aux_bytes < abytes) {
    if (h->md_aux) cudaFree(h->md_aux);
    h->md_aux = nullptr;
    h->md_aux_bytes = 0;
    rbrp_status s = cuda_check(h, cudaMalloc(&h->md_aux, abytes), "cudaMalloc(matdivide operands)");
    if (s != RBRP_OK) return s;
    h->md_aux_bytes = abytes;
  }
  double* R11 = static_cast<double*>(h->md_aux);
  double* R12 = R11 + (size_t)k * k;
  k_md_split_R<<<1216, 256, 0, h->stream>>>(h->R, n, k, R11, R12);
  rbrp_status s = cuda_check(h, cudaGetLastError(), "matdivide gather");
  if (s != RBRP_OK) return s;
  return matdivide(h, k, k, nc, R11, k, R12, k, tol, h->T, k, rank);
}

namespace rbrp {

// One or more refinement steps of the last run's T against the matrix A it was
// computed from: T += pinv(A_S) (A_rd - A_S T), in FP64 on the exact values of A.
template <typename T>
rbrp_status refine_T(rbrp_handle h, int m, int n, const T* dA, int64_t lda, int steps, double tol, double* change) {
  if (!h || !dA || lda < m || steps < 1 || !(tol >= 0.0) || !std::isfinite(tol)) return RBRP_ERR_INVALID_ARG;
  if (!h->have_result) return set_error(h, RBRP_ERR_NOT_COMPUTED, "no successful run");
  if (m != h->m || n != h->n) return set_error(h, RBRP_ERR_INVALID_ARG, "shape differs from the last run");
  const int k = h->k, nc = n - k;
  if (change) *change = 0.0;
  if (k <= 0 || nc <= 0) return RBRP_OK;  // T is empty
  if (!h->T) return set_error(h, RBRP_ERR_NOT_COMPUTED, "T was not computed");
  DeviceGuard g(h->device);
  // operands: A_S (m x k) | A_rd (m x nc) | E (m x nc) | D (k x nc) | CTA partials
  constexpr int NP = 512;
  const size_t bytes = ((size_t)m * k + 2 * (size_t)m * nc + (size_t)k * nc + 2 * NP) * sizeof(double);
  if (h->md_aux_bytes < bytes) {
    if (h->md_aux) cudaFree(h->md_aux);
    h->md_aux = nullptr;
    h->md_aux_bytes = 0;
    rbrp_status s = cuda_check(h, cudaMalloc(&h->md_aux, bytes), "cudaMalloc(refinement operands)");
    if (s != RBRP_OK) return s;
    h->md_aux_bytes = bytes;
  }
  double* As = static_cast<double*>(h->md_aux);
  double* Ard = As + (size_t)m * k;
  double* E = Ard + (size_t)m * nc;
  double* D = E + (size_t)m * nc;
  double* parts = D + (size_t)k * nc;
  cudaStream_t st = h->stream;
  k_md_gather<T><<<1216, 256, 0, st>>>(dA, lda, h->perm, 0, m, k, As);
  k_md_gather<T><<<1216, 256, 0, st>>>(dA, lda, h->perm, k, m, nc, Ard);
  // numerical-rank cutoff of A_S: the caller's, or max(m, k) units of rounding of |A_S|_F
  k_md_fro<<<1, MD_THREADS, 0, st>>>(As, (int64_t)m * k, parts);
  double fro2 = 0.0;
  rbrp_status s = cuda_check(h, cudaGetLastError(), "refinement gather");
  if (s == RBRP_OK) s = cuda_check(h, cudaMemcpyAsync(&fro2, parts, 8, cudaMemcpyDeviceToHost, st), "norm");
  if (s == RBRP_OK) s = cuda_check(h, cudaStreamSynchronize(st), "refinement gather");
  if (s != RBRP_OK) return s;
  if (!std::isfinite(fro2)) return set_error(h, RBRP_ERR_NUMERIC, "refinement: non-finite entries in A");
  const double cut = std::max(tol, std::max(m, k) * 2.220446049250313e-16 * std::sqrt(fro2));
  std::vector<double> hp(2 * NP);
  for (int it = 0; it < steps; ++it) {
    // E = A_rd - A_S T
    k_md_gemm<false><<<dim3((nc + 31) / 32, (m + 31) / 32), 256, 0, st>>>(As, m, h->T, k, nullptr, m, nc, k, E, m);
    k_md_xmy<<<1216, 256, 0, st>>>(Ard, E, (int64_t)m * nc);
    s = cuda_check(h, cudaGetLastError(), "refinement residual");
    if (s != RBRP_OK) return s;
    // D = pinv(A_S) E, T += D
    int rank = 0;
    s = matdivide(h, m, k, nc, As, m, E, m, cut, D, k, &rank);
    if (s != RBRP_OK) return s;
    k_md_add<<<NP, 256, 0, st>>>(h->T, k, D, k, nc, parts);
    s = cuda_check(h, cudaMemcpyAsync(hp.data(), parts, 2 * NP * sizeof(double), cudaMemcpyDeviceToHost, st), "refine");
    if (s == RBRP_OK) s = cuda_check(h, cudaStreamSynchronize(st), "refinement step");
    if (s != RBRP_OK) return s;
    double dd = 0.0, tt = 0.0;
    for (int z = 0; z < NP; ++z) {
      dd += hp[2 * z];
      tt += hp[2 * z + 1];
    }
    if (change) *change = tt > 0.0 ? std::sqrt(dd / tt) : 0.0;
  }
  return RBRP_OK;
}

}  // namespace rbrp

extern "C" rbrp_status rbrp_refine_T_f64(rbrp_handle h, int m, int n, const double* dA, int64_t lda, int steps,
                                         double tol, double* change) {
  return rbrp::refine_T<double>(h, m, n, dA, lda, steps, tol, change);
}

extern "C" rbrp_status rbrp_refine_T_f32(rbrp_handle h, int m, int n, const float* dA, int64_t lda, int steps,
                                         double tol, double* change) {
  return rbrp::refine_T<float>(h, m, n, dA, lda, steps, tol, change);
}
