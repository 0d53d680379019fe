// rbrp_adjoint.cu - loss and adjoint of the fixed-skeleton interpolative
// decomposition, FP32 kernels (no counterpart in the reference).
//
// With the skeleton S held fixed, C = A(:, S) (m x k), B = A(:, rd) (m x nc)
// and T = C^+ B (the k x nc interpolation matrix of the last fixed-skeleton
// run, T = R11^{-1} R12), the loss is
//     L = ||E||_F^2 + ||T w||^2,   E = B - C T,   w = dW(rd).
// Its gradient (T optimal for the first term, so only the second term sees
// dT = -C^+ dC T + (C^T C)^{-1} dC^T E + C^+ dB), with u = T w and
// z = (C^T C)^{-1} u = R11^{-1} R11^{-T} u:
//     dL/dB = 2 E + 2 (C z) w^T
//     dL/dC = -2 E T^T - 2 (C z) u^T + 2 (E w) z^T.
// Nothing of the forward factorisation is stored: R11 and T come from the
// handle's last run (the caller recomputes it for the backward), C and B are
// read from A through perm.  The two products E = B - C T and E T^T run on the
// tensor cores (tcgen05, 3xTF32, rbrp_gemm_tc.cuh) with the loss terms, E w and
// the rank-one terms fused into their epilogues (the handle's variant 1 keeps
// them as 128 x 128-tiled FP32 FFMA GEMMs); z is a double-float triangular
// solve.
//
// Tensor-core operand layouts (K-major, leading dimensions rounded up to 4
// floats for TMA):
//   E = B - C T:  M = rd columns c, N = rows r, K = skeleton index t
//                 X = T (k x nc, ld kp), Y = C^T (k x m, ld kp, TF32 hi / lo)
//                 written as E^T (nc x m, ld ncp): the drain lanes run along c
//   E T^T:        M = rows r, N = skeleton index t, K = rd columns c
//                 X = E^T, Y = T^T (nc x k, ld ncp, TF32 hi / lo)
#include <algorithm>
#include <cmath>

#include "rbrp_internal.h"
#include "rbrp_df.cuh"
#include "rbrp_gemm.cuh"
#include "rbrp_gemm_tc.cuh"

namespace rbrp {
namespace {

constexpr int PARTS = 16;      // split of the GEMV contractions

// Tr[t * nc + c] = T[t + c * k] (row major copy) and Tc = FP32 T (column major);
// wr[c] = W[perm[k + c]].
__global__ void k_adj_prep(const double* __restrict__ T, int k, int nc, const float* __restrict__ W,
                           const int* __restrict__ perm, float* __restrict__ Tr, float* __restrict__ Tc,
                           float* __restrict__ wr) {
  __shared__ float tile[32][33];
  const int t0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads
  for (int q = ty; q < 32; q += 8) {
    const int t = t0 + tx, c = c0 + q;
    float v = 0.f;
    if (t < k && c < nc) {
      v = (float)T[t + (int64_t)c * k];
      Tc[t + (int64_t)c * k] = v;
    }
    tile[q][tx] = v;
  }
  __syncthreads();
  for (int q = ty; q < 32; q += 8) {
    const int t = t0 + q, c = c0 + tx;
    if (t < k && c < nc) Tr[(int64_t)t * nc + c] = tile[tx][q];
  }
  if (blockIdx.x == 0)
    for (int c = c0 + threadIdx.x; c < min(nc, c0 + 32); c += blockDim.x) wr[c] = W[perm[k + c]];
}

// upart[p][t] = sum over columns c of part p of T[t, c] wr[c] (double-float, as float2);
// T is FP32, k x nc, column major with leading dimension ldt >= k
__global__ void k_adj_u(const float* __restrict__ Tc, int64_t ldt, int k, int nc, const float* __restrict__ wr,
                        float2* __restrict__ upart) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int p = blockIdx.y, chunk = (nc + PARTS - 1) / PARTS;
  const int cb = p * chunk, ce = min(nc, cb + chunk);
  if (t >= k) return;
  float hi = 0.f, lo = 0.f;
  for (int c = cb; c < ce; ++c) {
    const float prod = Tc[t + (int64_t)c * ldt] * wr[c];
    const float e = fmaf(Tc[t + (int64_t)c * ldt], wr[c], -prod);
    const float s = hi + prod, z = s - hi;
    lo += ((hi - (s - z)) + (prod - z)) + e;
    hi = s;
  }
  upart[(int64_t)p * k + t] = make_float2(hi, lo);
}

// out[i] = sum of the PARTS partials (fixed order), as float and (if out_df)
// double-float.
__global__ void k_adj_sum_parts(const float2* __restrict__ part, int len, float* __restrict__ out,
                                float2* __restrict__ out_df) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= len) return;
  dfl s = {part[i].x, part[i].y};
  for (int p = 1; p < PARTS; ++p) {
    const float2 v = part[(int64_t)p * len + i];
    s = df_add(s, {v.x, v.y});
  }
  s = df_two_sum(s.hi, s.lo);
  out[i] = s.hi;
  if (out_df) out_df[i] = make_float2(s.hi, s.lo);
}

// out[i] = sum over p < nparts of part[p][i] (fixed order, double-float).
__global__ void k_adj_sum_rows(const float2* __restrict__ part, int nparts, int len, float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= len) return;
  dfl s = {0.f, 0.f};
  for (int p = 0; p < nparts; ++p) {
    const float2 v = part[(int64_t)p * len + i];
    s = df_add(s, {v.x, v.y});
  }
  out[i] = df_two_sum(s.hi, s.lo).hi;
}

// R11 (FP64, row major, ld ldr, upper) as double-float pairs, row major ld k.
__global__ void k_adj_split_r(const double* __restrict__ R, int64_t ldr, int k, float2* __restrict__ Rdf) {
  const int64_t total = (int64_t)k * k;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int a = (int)(idx / k), c = (int)(idx % k);
    const double x = c >= a ? R[(int64_t)a * ldr + c] : 0.0;
    const float hi = (float)x;
    Rdf[idx] = make_float2(hi, (float)(x - (double)hi));
  }
}

// z = R11^{-1} R11^{-T} u in double-float, by 32-row blocks, one launch per block
// and direction.  In every CTA warp 0 solves the block's 32 x 32 triangle from the
// right-hand side rhs (lane-parallel: the lane of row i finishes x_i, every later
// lane subtracts its term), CTA 0 stores it in sol, and all CTAs subtract the
// block's contribution from their share of the remaining rows of rhs.  No CTA
// writes what another reads in the same launch: the block's rhs rows are only
// read, its solution goes to sol.
__device__ __forceinline__ dfl r_df(const float2* __restrict__ R, int k, int a, int c) {
  const float2 v = R[(int64_t)a * k + c];
  return dfl{v.x, v.y};
}

// forward step: R11^T y = u for rows [j0, j0 + 32): y(j0..) into sol, rhs(j) for j >= j0 + 32
__global__ void __launch_bounds__(256) k_adj_zf_step(const float2* __restrict__ R, int k, int j0,
                                                     float2* __restrict__ rhs, float2* __restrict__ sol) {
  __shared__ dfl xb[32];
  __shared__ dfl Rb[32][33];  // the block's diagonal 32 x 32 of R, staged once
  const int tid = threadIdx.x, lane = tid & 31;
  const int jl = min(32, k - j0);
  for (int e = tid; e < 32 * 32; e += blockDim.x) {
    const int a = e >> 5, c = e & 31;
    Rb[a][c] = (a < jl && c < jl) ? r_df(R, k, j0 + a, j0 + c) : dfl{1.f, 0.f};
  }
  __syncthreads();
  if (tid < 32) {
    dfl b = {0.f, 0.f};
    if (lane < jl) {
      const float2 v = rhs[j0 + lane];
      b = {v.x, v.y};
    }
    dfl x = {0.f, 0.f};
    for (int i = 0; i < jl; ++i) {
      if (lane == i) x = df_mul(b, df_recip(Rb[i][i]));
      const dfl xi = {__shfl_sync(0xffffffffu, x.hi, i), __shfl_sync(0xffffffffu, x.lo, i)};
      if (lane > i && lane < jl) b = df_fms(b, Rb[i][lane], xi);
    }
    xb[lane] = x;
  }
  __syncthreads();
  if (blockIdx.x == 0 && tid < jl) sol[j0 + tid] = make_float2(xb[tid].hi, xb[tid].lo);
  for (int j = j0 + jl + blockIdx.x * blockDim.x + tid; j < k; j += gridDim.x * blockDim.x) {
    const float2 w0 = rhs[j];
    dfl v = {w0.x, w0.y};
    for (int ii = 0; ii < jl; ++ii) v = df_fms(v, r_df(R, k, j0 + ii, j), xb[ii]);
    rhs[j] = make_float2(v.hi, v.lo);
  }
}

// backward step: R11 z = y for rows [i0, i0 + il): z(i0..) into sol, rhs(i) for i < i0
__global__ void __launch_bounds__(256) k_adj_zb_step(const float2* __restrict__ R, int k, int i0, int il,
                                                     float2* __restrict__ rhs, float2* __restrict__ sol) {
  __shared__ dfl xb[32];
  __shared__ dfl Rb[32][33];  // the block's diagonal il x il of R, staged once
  const int tid = threadIdx.x, lane = tid & 31;
  for (int e = tid; e < 32 * 32; e += blockDim.x) {
    const int a = e >> 5, c = e & 31;
    Rb[a][c] = (a < il && c < il) ? r_df(R, k, i0 + a, i0 + c) : dfl{1.f, 0.f};
  }
  __syncthreads();
  if (tid < 32) {
    dfl b = {0.f, 0.f};
    if (lane < il) {
      const float2 v = rhs[i0 + lane];
      b = {v.x, v.y};
    }
    dfl x = {0.f, 0.f};
    for (int i = il - 1; i >= 0; --i) {
      if (lane == i) x = df_mul(b, df_recip(Rb[i][i]));
      const dfl xi = {__shfl_sync(0xffffffffu, x.hi, i), __shfl_sync(0xffffffffu, x.lo, i)};
      if (lane < i) b = df_fms(b, Rb[lane][i], xi);
    }
    xb[lane] = x;
  }
  __syncthreads();
  if (blockIdx.x == 0 && tid < il) sol[i0 + tid] = make_float2(xb[tid].hi, xb[tid].lo);
  for (int i = blockIdx.x * blockDim.x + tid; i < i0; i += gridDim.x * blockDim.x) {
    const float2 w0 = rhs[i];
    dfl v = {w0.x, w0.y};
    for (int jj = 0; jj < il; ++jj) v = df_fms(v, r_df(R, k, i, i0 + jj), xb[jj]);
    rhs[i] = make_float2(v.hi, v.lo);
  }
}

__global__ void k_adj_copy_df(const float2* __restrict__ in, float2* __restrict__ out, int k) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < k) out[i] = in[i];
}

__global__ void k_adj_z_out(const float2* __restrict__ zdf, float* __restrict__ z, int k) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < k) z[i] = zdf[i].x;
}

// z (FP32) = R11^{-1} R11^{-T} u; work and ys are k double-float scratch vectors each.
void solve_z(cudaStream_t st, int sms, const float2* Rdf, int k, const float2* udf, float2* work, float2* ys,
             float* z) {
  const int grid = std::max(1, std::min((k + 255) / 256, 2 * sms));
  k_adj_copy_df<<<(k + 255) / 256, 256, 0, st>>>(udf, work, k);
  for (int j0 = 0; j0 < k; j0 += 32) k_adj_zf_step<<<grid, 256, 0, st>>>(Rdf, k, j0, work, ys);
  // backward: the right-hand side is y (ys, updated in place), the solution goes to work
  for (int i1 = k; i1 > 0; i1 -= 32) {
    const int i0 = std::max(0, i1 - 32);
    k_adj_zb_step<<<grid, 256, 0, st>>>(Rdf, k, i0, i1 - i0, ys, work);
  }
  k_adj_z_out<<<(k + 255) / 256, 256, 0, st>>>(work, z, k);
}

// czpart[p][r] = sum over the part-p skeleton columns t of A[r, perm[t]] z[t]
__global__ void k_adj_cz(const float* __restrict__ A, int64_t lda, int m, int k, const int* __restrict__ perm,
                         const float* __restrict__ z, float2* __restrict__ czpart) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int p = blockIdx.y, chunk = (k + PARTS - 1) / PARTS;
  const int tb = p * chunk, te = min(k, tb + chunk);
  if (r >= m) return;
  float hi = 0.f, lo = 0.f;
  for (int t = tb; t < te; ++t) {
    const float a = A[r + (int64_t)perm[t] * lda];
    const float prod = a * z[t];
    const float e = fmaf(a, z[t], -prod);
    const float s = hi + prod, zz = s - hi;
    lo += ((hi - (s - zz)) + (prod - zz)) + e;
    hi = s;
  }
  czpart[(int64_t)p * m + r] = make_float2(hi, lo);
}

// E = B - C T for a 128 x 128 tile: E stored (if Eout), ||E||^2 and E w row
// sums as per-tile partials, and G(:, rd) = scale * 2 (E + (C z) w^T).
__global__ void __launch_bounds__(GT) k_adj_gemm1(const float* __restrict__ A, int64_t lda, int m, int k, int nc,
                                                  const int* __restrict__ perm, const float* __restrict__ Tr,
                                                  const float* __restrict__ wr, const float* __restrict__ cz,
                                                  float* __restrict__ Eout, float* __restrict__ G, int64_t ldg,
                                                  float scale, float2* __restrict__ loss_part,
                                                  float2* __restrict__ ew_part) {
  __shared__ GemmSmem sm;
  __shared__ float2 red[GT];
  const int r0 = blockIdx.x * GTILE, c0 = blockIdx.y * GTILE;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  float acc[8][8];
  gemm_tile(sm, LoadC{A, lda, perm, m, k}, LoadRowMajor{Tr, k, nc}, k, r0, c0, acc);
  dfl sq = {0.f, 0.f};
  float ew[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) ew[i] = 0.f;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int c = c0 + tile_col(tx, j);
    if (c >= nc) continue;
    const int col = perm[k + c];
    const float w = wr[c];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int r = r0 + tile_row(ty, i);
      if (r >= m) continue;
      const float e = A[r + (int64_t)col * lda] - acc[i][j];
      df_acc_prod(sq, e, e);
      ew[i] = fmaf(e, w, ew[i]);
      if (Eout) Eout[r + (int64_t)c * m] = e;
      if (G) G[r + (int64_t)col * ldg] = scale * 2.f * fmaf(cz[r], w, e);
    }
  }
  // row sums of E w over the tile's 16 column groups: through shared memory, fixed order
  float* ews = reinterpret_cast<float*>(&sm);  // the staging buffers are idle now
#pragma unroll
  for (int i = 0; i < 8; ++i) ews[tile_row(ty, i) * 16 + tx] = ew[i];
  red[tid] = make_float2(sq.hi, sq.lo);
  __syncthreads();
  if (tid < GTILE) {
    float s = 0.f;
    for (int q = 0; q < 16; ++q) s += ews[tid * 16 + q];
    if (r0 + tid < m) ew_part[(int64_t)blockIdx.y * m + r0 + tid] = make_float2(s, 0.f);
  }
  if (tid == 0) {
    dfl t = {red[0].x, red[0].y};
    for (int q = 1; q < GT; ++q) t = df_add(t, {red[q].x, red[q].y});
    loss_part[blockIdx.y * gridDim.x + blockIdx.x] = make_float2(t.hi, t.lo);
  }
}

// G(:, S) = scale * (-2 E T^T - 2 (C z) u^T + 2 (E w) z^T) for a 128 x 128 tile.
__global__ void __launch_bounds__(GT) k_adj_gemm2(const float* __restrict__ E, int m, int k, int nc,
                                                  const int* __restrict__ perm, const float* __restrict__ Tc,
                                                  const float* __restrict__ cz, const float* __restrict__ ew,
                                                  const float* __restrict__ u, const float* __restrict__ z,
                                                  float* __restrict__ G, int64_t ldg, float scale) {
  __shared__ GemmSmem sm;
  const int r0 = blockIdx.x * GTILE, c0 = blockIdx.y * GTILE;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  float acc[8][8];
  // E T^T: contraction over the nc rd columns; T^T (nc x k) row major is T column major
  gemm_tile(sm, LoadE{E, m, nc}, LoadRowMajor{Tc, nc, k}, nc, r0, c0, acc);
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int t = c0 + tile_col(tx, j);
    if (t >= k) continue;
    const int col = perm[t];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int r = r0 + tile_row(ty, i);
      if (r >= m) continue;
      const float g = -2.f * acc[i][j] - 2.f * cz[r] * u[t] + 2.f * ew[r] * z[t];
      G[r + (int64_t)col * ldg] = scale * g;
    }
  }
}

__global__ void k_adj_loss(const float2* __restrict__ loss_part, int nparts, const float2* __restrict__ udf, int k,
                           double* __restrict__ out) {
  __shared__ float2 red[256];
  dfl s = {0.f, 0.f};
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) s = df_add(s, {loss_part[i].x, loss_part[i].y});
  dfl su = {0.f, 0.f};
  for (int i = threadIdx.x; i < k; i += blockDim.x) {
    const dfl v = {udf[i].x, udf[i].y};
    su = df_add(su, df_mul(v, v));
  }
  red[threadIdx.x] = make_float2(s.hi, s.lo);
  __syncthreads();
  if (threadIdx.x == 0) {
    dfl t = {red[0].x, red[0].y};
    for (int q = 1; q < (int)blockDim.x; ++q) t = df_add(t, {red[q].x, red[q].y});
    out[0] = (double)t.hi + (double)t.lo;
  }
  __syncthreads();
  red[threadIdx.x] = make_float2(su.hi, su.lo);
  __syncthreads();
  if (threadIdx.x == 0) {
    dfl t = {red[0].x, red[0].y};
    for (int q = 1; q < (int)blockDim.x; ++q) t = df_add(t, {red[q].x, red[q].y});
    out[1] = (double)t.hi + (double)t.lo;
  }
}

// ---------------------------------------------------------------------------
// tensor-core path
// ---------------------------------------------------------------------------
// Tx (k x nc, ld kp) = FP32 T; T^T hi / lo (nc x k, ld ncp) = tf32_rn(t), tf32_rn(t - hi)
// from the FP64 T; wr[c] = W[perm[k + c]].  32 x 32 tiles through shared memory.
__global__ void k_adj_prep_tc(const double* __restrict__ T, int k, int nc, int kp, int ncp,
                              const float* __restrict__ W, const int* __restrict__ perm, float* __restrict__ Tx,
                              float* __restrict__ Trh, float* __restrict__ Trl, float* __restrict__ wr) {
  __shared__ double tile[32][33];
  const int t0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads
  for (int q = ty; q < 32; q += 8) {
    const int t = t0 + tx, c = c0 + q;
    double v = 0.0;
    if (t < k && c < nc) {
      v = T[t + (int64_t)c * k];
      Tx[t + (int64_t)c * kp] = (float)v;
    }
    tile[q][tx] = v;
  }
  __syncthreads();
  for (int q = ty; q < 32; q += 8) {
    const int t = t0 + q, c = c0 + tx;
    if (t < k && c < nc) {
      const double v = tile[tx][q];
      const float h = tf32_rn((float)v);
      Trh[c + (int64_t)t * ncp] = h;
      Trl[c + (int64_t)t * ncp] = tf32_rn((float)(v - (double)h));
    }
  }
  if (blockIdx.x == 0)
    for (int c = c0 + threadIdx.x; c < min(nc, c0 + 32); c += blockDim.x) wr[c] = W[perm[k + c]];
}

// C^T hi / lo (k x m, ld kp): element (t, r) = A[r, perm[t]] split by tf32_split.
__global__ void k_adj_gather_ct(const float* __restrict__ A, int64_t lda, const int* __restrict__ perm, int k,
                                int m, int kp, float* __restrict__ Cth, float* __restrict__ Ctl) {
  __shared__ float tile[32][33];
  const int r0 = blockIdx.x * 32, t0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int q = ty; q < 32; q += 8) {
    const int r = r0 + tx, t = t0 + q;
    tile[q][tx] = (r < m && t < k) ? A[r + (int64_t)perm[t] * lda] : 0.f;
  }
  __syncthreads();
  for (int q = ty; q < 32; q += 8) {
    const int t = t0 + tx, r = r0 + q;
    if (t < k && r < m) {
      float h, l;
      tf32_split(tile[tx][q], h, l);
      Cth[t + (int64_t)r * kp] = h;
      Ctl[t + (int64_t)r * kp] = l;
    }
  }
}

// Per-CTA reduction buffers of the E epilogue (one instance per CTA).
__device__ __forceinline__ float* epi_ew_buf() {
  __shared__ float buf[64 * 4];  // [row slot][lane quarter]
  return buf;
}
__device__ __forceinline__ float2* epi_sq_buf() {
  __shared__ float2 buf[8];      // [drain warp]
  return buf;
}

// E = B - C T on a (128 rd columns) x (64 rows) tile: E^T stored (when Et), ||E||^2
// and the row sums of E w as per-CTA partials, G(:, rd) = scale * 2 (E + (C z) w^T).
struct EpiE {
  const float* A;
  int64_t lda;
  const int* perm;
  int k, m, nc;
  const float* wr;
  const float* cz;
  float* Et;
  int64_t ldet;
  float* G;
  int64_t ldg;
  float scale;
  float2* loss_part;
  float2* ew_part;

  __device__ void operator()(int c, int r0, const float (&hi)[32], const float (&lo)[32], int dw) const {
    float* s_ew = epi_ew_buf();
    float2* s_sq = epi_sq_buf();
    const int lane = threadIdx.x & 31, quarter = (c & 127) >> 5, ch = dw >> 2;
    const bool vc = c < nc;
    const float w = vc ? wr[c] : 0.f;
    const int64_t col = vc ? (int64_t)perm[k + c] : 0;
    dfl sq = {0.f, 0.f};
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      const int r = r0 + j;
      float e = 0.f;
      if (vc && r < m) {
        e = (A[r + col * lda] - hi[j]) - lo[j];
        df_acc_prod(sq, e, e);
        if (Et) Et[c + (int64_t)r * ldet] = e;
        if (G) G[r + col * ldg] = scale * 2.f * fmaf(cz[r], w, e);
      }
      float ew = e * w;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) ew += __shfl_xor_sync(0xffffffffu, ew, o);
      if (lane == 0) s_ew[(ch * 32 + j) * 4 + quarter] = ew;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const dfl t = {__shfl_xor_sync(0xffffffffu, sq.hi, o), __shfl_xor_sync(0xffffffffu, sq.lo, o)};
      sq = df_add(sq, t);
    }
    if (lane == 0) s_sq[dw] = make_float2(sq.hi, sq.lo);
  }

  // after the CTA barrier: fixed-order sums of the shared partials
  __device__ void finish(bool ok) const {
    if (!ok) return;
    const float* s_ew = epi_ew_buf();
    const float2* s_sq = epi_sq_buf();
    const int t = threadIdx.x;
    if (t < 64) {
      const int r = blockIdx.y * 64 + t;
      if (r < m) {
        const float s = ((s_ew[t * 4] + s_ew[t * 4 + 1]) + s_ew[t * 4 + 2]) + s_ew[t * 4 + 3];
        ew_part[(int64_t)blockIdx.x * m + r] = make_float2(s, 0.f);
      }
    } else if (t == 64) {
      dfl a = {s_sq[0].x, s_sq[0].y};
      for (int q = 1; q < 8; ++q) a = df_add(a, {s_sq[q].x, s_sq[q].y});
      loss_part[(int64_t)blockIdx.y * gridDim.x + blockIdx.x] = make_float2(a.hi, a.lo);
    }
  }
};

// G(:, S) = scale * (-2 E T^T - 2 (C z) u^T + 2 (E w) z^T) on a (128 rows) x (64 skeleton) tile.
struct EpiG {
  const int* perm;
  int m, k;
  const float* cz;
  const float* ew;
  const float* u;
  const float* z;
  float* G;
  int64_t ldg;
  float scale;

  __device__ void operator()(int r, int a0, const float (&hi)[32], const float (&lo)[32], int) const {
    if (r >= m) return;
    const float czr = cz[r], ewr = ew[r];
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      const int a = a0 + j;
      if (a < k) {
        const float g = -2.f * (hi[j] + lo[j]) - 2.f * czr * u[a] + 2.f * ewr * z[a];
        G[r + (int64_t)perm[a] * ldg] = scale * g;
      }
    }
  }
  __device__ void finish(bool) const {}
};

size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace
}  // namespace rbrp

namespace rbrp {
namespace {

// The tensor-core form of the loss and gradient (same outputs as the FFMA kernels).
rbrp_status adjoint_tc(rbrp_handle h, int m, int k, int nc, int kp, int ncp, const float* dA, int64_t lda,
                       const float* dW, float scale, float* dG, int64_t ldg, double* loss, float* Trh, float* Trl,
                       float* Tx, float* wr, float2* up, float* u, float2* udf, float* z, float2* Rdf, float2* wk,
                       float2* ys, float2* czp, float* cz, float* Et, float2* ewp, float* ew, float2* lp, double* lout,
                       float* Cth, float* Ctl, int* dstatus) {
  cudaStream_t st = h->stream;
  const int n = h->n;
  if (!h->smem_attr_gemm_tc) {
    rbrp_status s = cuda_check(h, cudaFuncSetAttribute(tc::k_gemm_tc<EpiE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       (int)tc::GEMM_SMEM), "cudaFuncSetAttribute(k_gemm_tc<E>)");
    if (s == RBRP_OK)
      s = cuda_check(h, cudaFuncSetAttribute(tc::k_gemm_tc<EpiG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)tc::GEMM_SMEM), "cudaFuncSetAttribute(k_gemm_tc<G>)");
    if (s != RBRP_OK) return s;
    h->smem_attr_gemm_tc = true;
  }
  const long long budget = h->wait_budget > 0 ? h->wait_budget : kWaitBudgetDefault;
  CUtensorMap tmX1, tmY1h, tmY1l;
  rbrp_status s = make_tmap_f32(h, &tmX1, Tx, k, nc, kp, tc::BK, tc::BM);
  if (s == RBRP_OK) s = make_tmap_f32(h, &tmY1h, Cth, k, m, kp, tc::BK, tc::BN);
  if (s == RBRP_OK) s = make_tmap_f32(h, &tmY1l, Ctl, k, m, kp, tc::BK, tc::BN);
  if (s != RBRP_OK) return s;
  s = cuda_check(h, cudaMemsetAsync(dstatus, 0, sizeof(int), st), "clear status");
  if (s != RBRP_OK) return s;

  k_adj_prep_tc<<<dim3((k + 31) / 32, (nc + 31) / 32), 256, 0, st>>>(h->T, k, nc, kp, ncp, dW, h->perm, Tx, Trh,
                                                                     Trl, wr);
  k_adj_gather_ct<<<dim3((m + 31) / 32, (k + 31) / 32), 256, 0, st>>>(dA, lda, h->perm, k, m, kp, Cth, Ctl);
  k_adj_u<<<dim3((k + 255) / 256, PARTS), 256, 0, st>>>(Tx, kp, k, nc, wr, up);
  k_adj_sum_parts<<<(k + 255) / 256, 256, 0, st>>>(up, k, u, udf);
  if (dG) {
    k_adj_split_r<<<1216, 256, 0, st>>>(h->R, n, k, Rdf);
    solve_z(st, h->sms, Rdf, k, udf, wk, ys, z);
    k_adj_cz<<<dim3((m + 255) / 256, PARTS), 256, 0, st>>>(dA, lda, m, k, h->perm, z, czp);
    k_adj_sum_parts<<<(m + 255) / 256, 256, 0, st>>>(czp, m, cz, nullptr);
  }
  const int tx1 = (nc + tc::BM - 1) / tc::BM, ty1 = (m + tc::BN - 1) / tc::BN;
  EpiE e1{dA, lda, h->perm, k, m, nc, wr, cz, dG ? Et : nullptr, ncp, dG, ldg, scale, lp, ewp};
  tc::k_gemm_tc<EpiE><<<dim3(tx1, ty1), tc::NTHREADS, tc::GEMM_SMEM, st>>>(tmX1, tmY1h, tmY1l, nc, m, k, budget,
                                                                       dstatus, e1);
  if (dG) k_adj_sum_rows<<<(m + 255) / 256, 256, 0, st>>>(ewp, tx1, m, ew);
  k_adj_loss<<<1, 256, 0, st>>>(lp, tx1 * ty1, udf, k, lout);
  if (dG) {
    CUtensorMap tmX2, tmY2h, tmY2l;
    s = make_tmap_f32(h, &tmX2, Et, nc, m, ncp, tc::BK, tc::BM);
    if (s == RBRP_OK) s = make_tmap_f32(h, &tmY2h, Trh, nc, k, ncp, tc::BK, tc::BN);
    if (s == RBRP_OK) s = make_tmap_f32(h, &tmY2l, Trl, nc, k, ncp, tc::BK, tc::BN);
    if (s != RBRP_OK) return s;
    EpiG e2{h->perm, m, k, cz, ew, u, z, dG, ldg, scale};
    tc::k_gemm_tc<EpiG><<<dim3((m + tc::BM - 1) / tc::BM, (k + tc::BN - 1) / tc::BN), tc::NTHREADS, tc::GEMM_SMEM, st>>>(
        tmX2, tmY2h, tmY2l, m, k, nc, budget, dstatus, e2);
  }
  s = cuda_check(h, cudaGetLastError(), "adjoint kernels");
  if (s != RBRP_OK) return s;
  double hl[2] = {0.0, 0.0};
  int hs = 0;
  s = cuda_check(h, cudaMemcpyAsync(hl, lout, sizeof(hl), cudaMemcpyDeviceToHost, st), "copy loss");
  if (s == RBRP_OK) s = cuda_check(h, cudaMemcpyAsync(&hs, dstatus, sizeof(int), cudaMemcpyDeviceToHost, st), "status");
  if (s == RBRP_OK) s = cuda_check(h, cudaStreamSynchronize(st), "adjoint kernels");
  if (s != RBRP_OK) return s;
  if (hs == tc::ST_ERR_TIMEOUT)
    return set_error(h, RBRP_ERR_DEVICE_TIMEOUT, "a device-side wait of the adjoint GEMMs timed out; they aborted cleanly");
  if (loss) *loss = hl[0] + hl[1];
  return RBRP_OK;
}

}  // namespace
}  // namespace rbrp

using namespace rbrp;

extern "C" rbrp_status rbrp_fixed_id_adjoint_f32(rbrp_handle h, int m, int n, const float* dA, int64_t lda,
                                                 const float* dW, float scale, float* dG, int64_t ldg,
                                                 double* loss) {
  if (!h) return RBRP_ERR_INVALID_ARG;
  if (!h->have_result || h->prec != RBRP_PREC_F32_MIXED)
    return set_error(h, RBRP_ERR_NOT_COMPUTED, "needs a preceding FP32 run (rbrp_fixed_id_f32) on this matrix");
  if (m != h->m || n != h->n || !dA || lda < m || !dW)
    return set_error(h, RBRP_ERR_INVALID_ARG, "A / W do not match the last run");
  if (dG && ldg < m) return set_error(h, RBRP_ERR_INVALID_ARG, "ldg < m");
  const int k = h->k, nc = n - k;
  if (k < 1 || nc < 1 || !h->T) return set_error(h, RBRP_ERR_NOT_COMPUTED, "the last run has no T (k = 0 or n)");
  DeviceGuard g(h->device);
  cudaStream_t st = h->stream;
  // workspace: Tr, Tc (k x nc), wr (nc), u parts / u / udf, z, Rdf (k x k), work (k), cz parts / cz,
  // E (m x nc), E w parts / E w, loss parts, loss out
  const bool use_tc = h->variant == 0;
  const int gx = (m + GTILE - 1) / GTILE, gy1 = (nc + GTILE - 1) / GTILE, gy2 = (k + GTILE - 1) / GTILE;
  const int kp = (k + 3) & ~3, ncp = (nc + 3) & ~3;           // TMA leading dimensions (16-byte rows)
  const int tx1 = (nc + tc::BM - 1) / tc::BM, ty1 = (m + tc::BN - 1) / tc::BN;   // E tiles
  const size_t kn = (size_t)k * nc;
  size_t off = 0;
  auto take = [&](size_t bytes) { const size_t o = off; off += al(bytes); return o; };
  const size_t o_Tr = take(4 * (use_tc ? (size_t)ncp * k : kn)), o_Tc = take(4 * (use_tc ? (size_t)kp * nc : kn));
  const size_t o_wr = take(4 * (size_t)nc);
  const size_t o_up = take(8 * (size_t)PARTS * k), o_u = take(4 * (size_t)k), o_udf = take(8 * (size_t)k);
  const size_t o_z = take(4 * (size_t)k), o_R = take(8 * (size_t)k * k), o_wk = take(8 * (size_t)k);
  const size_t o_ys = take(8 * (size_t)k);
  const size_t o_czp = take(8 * (size_t)PARTS * m), o_cz = take(4 * (size_t)m);
  const size_t o_E = take(4 * (use_tc ? (size_t)ncp * m : (size_t)m * nc)), o_ewp = take(8 * (size_t)gy1 * m);
  const size_t o_ew = take(4 * (size_t)m);
  const size_t o_lp = take(8 * std::max((size_t)gx * gy1, (size_t)tx1 * ty1)), o_loss = take(16);
  // tensor-core operands: T^T lo, C^T hi / lo, the timeout status
  const size_t o_Trl = use_tc ? take(4 * (size_t)ncp * k) : 0;
  const size_t o_Cth = use_tc ? take(4 * (size_t)kp * m) : 0, o_Ctl = use_tc ? take(4 * (size_t)kp * m) : 0;
  const size_t o_st = take(16);
  if (h->adj_bytes < off) {
    if (h->adj_ws) cudaFree(h->adj_ws);
    h->adj_ws = nullptr;
    h->adj_bytes = 0;
    rbrp_status s = cuda_check(h, cudaMalloc(&h->adj_ws, off), "cudaMalloc(adjoint workspace)");
    if (s != RBRP_OK) return s;
    h->adj_bytes = off;
  }
  unsigned char* w = static_cast<unsigned char*>(h->adj_ws);
  float* Tr = reinterpret_cast<float*>(w + o_Tr);
  float* Tc = reinterpret_cast<float*>(w + o_Tc);
  float* wr = reinterpret_cast<float*>(w + o_wr);
  float2* up = reinterpret_cast<float2*>(w + o_up);
  float* u = reinterpret_cast<float*>(w + o_u);
  float2* udf = reinterpret_cast<float2*>(w + o_udf);
  float* z = reinterpret_cast<float*>(w + o_z);
  float2* Rdf = reinterpret_cast<float2*>(w + o_R);
  float2* wk = reinterpret_cast<float2*>(w + o_wk);
  float2* ys = reinterpret_cast<float2*>(w + o_ys);
  float2* czp = reinterpret_cast<float2*>(w + o_czp);
  float* cz = reinterpret_cast<float*>(w + o_cz);
  float* E = reinterpret_cast<float*>(w + o_E);
  float2* ewp = reinterpret_cast<float2*>(w + o_ewp);
  float* ew = reinterpret_cast<float*>(w + o_ew);
  float2* lp = reinterpret_cast<float2*>(w + o_lp);
  double* lout = reinterpret_cast<double*>(w + o_loss);
  int* dstatus = reinterpret_cast<int*>(w + o_st);

  if (use_tc) return adjoint_tc(h, m, k, nc, kp, ncp, dA, lda, dW, scale, dG, ldg, loss, Tr /* T^T hi */,
                                reinterpret_cast<float*>(w + o_Trl), Tc /* Tx */, wr, up, u, udf, z, Rdf, wk, ys, czp,
                                cz, E /* E^T */, ewp, ew, lp, lout, reinterpret_cast<float*>(w + o_Cth),
                                reinterpret_cast<float*>(w + o_Ctl), dstatus);
  k_adj_prep<<<dim3((k + 31) / 32, (nc + 31) / 32), 256, 0, st>>>(h->T, k, nc, dW, h->perm, Tr, Tc, wr);
  k_adj_u<<<dim3((k + 255) / 256, PARTS), 256, 0, st>>>(Tc, k, k, nc, wr, up);
  k_adj_sum_parts<<<(k + 255) / 256, 256, 0, st>>>(up, k, u, udf);
  if (dG) {
    k_adj_split_r<<<1216, 256, 0, st>>>(h->R, n, k, Rdf);
    solve_z(st, h->sms, Rdf, k, udf, wk, ys, z);
    k_adj_cz<<<dim3((m + 255) / 256, PARTS), 256, 0, st>>>(dA, lda, m, k, h->perm, z, czp);
    k_adj_sum_parts<<<(m + 255) / 256, 256, 0, st>>>(czp, m, cz, nullptr);
  }
  k_adj_gemm1<<<dim3(gx, gy1), GT, 0, st>>>(dA, lda, m, k, nc, h->perm, Tr, wr, cz, dG ? E : nullptr, dG, ldg, scale,
                                            lp, ewp);
  if (dG) k_adj_sum_rows<<<(m + 255) / 256, 256, 0, st>>>(ewp, gy1, m, ew);
  k_adj_loss<<<1, 256, 0, st>>>(lp, gx * gy1, udf, k, lout);
  if (dG) {
    k_adj_gemm2<<<dim3(gx, gy2), GT, 0, st>>>(E, m, k, nc, h->perm, Tc, cz, ew, u, z, dG, ldg, scale);
  }
  double hl[2] = {0.0, 0.0};
  rbrp_status s = cuda_check(h, cudaMemcpyAsync(hl, lout, sizeof(hl), cudaMemcpyDeviceToHost, st), "copy loss");
  if (s == RBRP_OK) s = cuda_check(h, cudaStreamSynchronize(st), "adjoint kernels");
  if (s != RBRP_OK) return s;
  if (loss) *loss = hl[0] + hl[1];
  return RBRP_OK;
}
