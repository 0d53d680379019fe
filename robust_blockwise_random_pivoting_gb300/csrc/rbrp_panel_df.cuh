// rbrp_panel_df.cuh - panel CPQR of the FP32 residual form in double-float
// arithmetic (one CholQR pass: ~48-bit arithmetic keeps the basis orthogonal to
// far below its FP32 rounding).
//
// GB300's FP64 pipe issues ~1/64 of the FP32 pipe's rate, and the panel work
// (the Gram matrix, a pivoted Cholesky factorisation and a row solve per block)
// is FP64-class arithmetic.  Here every FP64 quantity is a pair of floats
// (hi + lo, ~48 significant bits) computed on the FP32 pipe with error-free
// transformations: products by FMA splitting, sums by TwoSum.  The steps are
// those of the FP64 panel kernels in rbrp_kernels.cuh (same pivot rule, same
// robust filter, same swap), so the FP64 path keeps its own kernels and these
// serve the mixed-precision path.
//
// The pivoted Cholesky never moves rows or columns: the Schur complement
// stays indexed by panel column, a slot -> column map (ord) carries LAPACK's
// swap order, so the argmax still picks the first maximal slot.
#pragma once
#include "rbrp_common.cuh"
#include "rbrp_df.cuh"
#include "rbrp_pchol_df.cuh"

namespace rbrp {
namespace {

constexpr int DF_ROWS = 128;  // panel rows per CTA of the Gram kernel

// V = A_res(:, J) (FP32, exact) for 128 rows per CTA, and the tile's Gram partial V^T V
// (upper triangle, mirrored) in double-float, stored as FP64.
__global__ void __launch_bounds__(256)
k_gram_df(const float* __restrict__ Ares, int64_t ld, const int* __restrict__ js, const State* __restrict__ st,
          int m, float* __restrict__ V, double* __restrict__ Gpart) {
  __shared__ float Vs[DF_ROWS][MAXB + 1];
  __shared__ int cs[MAXB];
  const int tid = threadIdx.x;
  const int bss = st->bs_sampled;
  const int r0 = blockIdx.x * DF_ROWS;
  if (tid < MAXB) cs[tid] = tid < bss ? js[tid] : -1;
  __syncthreads();
  for (int idx = tid; idx < DF_ROWS * MAXB; idx += 256) {
    const int rr = idx % DF_ROWS, c = idx / DF_ROWS, r = r0 + rr;
    const float v = (r < m && cs[c] >= 0) ? Ares[r + (int64_t)cs[c] * ld] : 0.f;
    Vs[rr][c] = v;
    if (r < m && c < bss) V[r + (int64_t)c * m] = v;
  }
  __syncthreads();
  double* G = Gpart + (int64_t)blockIdx.x * MAXB * MAXB;
  const int c1 = tid >> 2;
  dfl acc[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) acc[q] = {0.f, 0.f};
  if (c1 < bss) {
    for (int rr = 0; rr < DF_ROWS; ++rr) {
      const float x = Vs[rr][c1];
#pragma unroll
      for (int q = 0; q < 16; ++q) df_acc_prod(acc[q], x, Vs[rr][(tid & 3) + 4 * q]);
    }
  }
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    const int c2 = (tid & 3) + 4 * q;
    const double g = (c1 < bss && c2 < bss) ? df_dbl(acc[q]) : 0.0;
    G[c1 * MAXB + c2] = g;
  }
}

using PcholDfSmem = PcholDfSmemT<MAXB>;

// Pivoted Cholesky of the panel Gram matrix with the robust filter (same rule as
// pivoted_chol_filter), LEAN_THREADS threads, no data movement for the swaps.  Publishes
// R11 (slot order, double-float pairs), ord, the kept count and performs the block swap.
__global__ void __launch_bounds__(LEAN_THREADS)
k_pchol_df(const double* __restrict__ G, int m, State* st, double tol_loc, const int* __restrict__ js,
           int* __restrict__ perm, double* __restrict__ diags, float2* __restrict__ R11g, float2* __restrict__ Rinvg,
           int* __restrict__ ordg, int* __restrict__ Jg, int* __restrict__ K1g, int* __restrict__ K2g) {
  extern __shared__ __align__(16) unsigned char dyn_smem[];
  PcholDfSmem& sm = *reinterpret_cast<PcholDfSmem*>(dyn_smem);
  const int tid = threadIdx.x;
  const int nb = st->bs_sampled, i = st->i;
  const int rows = min(nb, m);
  for (int idx = tid; idx < MAXB * MAXB; idx += blockDim.x) {
    const int a = idx / MAXB, c = idx % MAXB;
    sm.S[a][c] = (a < nb && c < nb) ? df_of(G[a * MAXB + c]) : dfl{0.f, 0.f};
  }
  if (tid < MAXB) {
    sm.ord[tid] = tid;
    sm.alive[tid] = tid < nb;
  }
  __syncthreads();
  static_assert(MAXB == 64, "the lean factorization is written for 64-column panels");
  const int kept = pchol_filter_df_lean(sm, nb, rows, tol_loc);
  // R11 in slot order: R11[a][c] = R[a][ord[c]] for c >= a
  for (int idx = tid; idx < MAXB * MAXB; idx += blockDim.x) {
    const int a = idx / MAXB, c = idx % MAXB;
    const dfl v = (a < kept && c < kept && c >= a) ? sm.R[a][sm.ord[c]] : dfl{0.f, 0.f};
    R11g[idx] = make_float2(v.hi, v.lo);
  }
  // R11^{-1} (upper triangular, slot order) by columns: 16 threads per column c solve
  // R11 x = e_c from the bottom, the dot products split over the 16 lanes.  The Schur
  // array is free now and holds x; the column groups of a warp are independent.
  __shared__ dfl invd[MAXB];
  if (tid < kept) invd[tid] = df_recip_lean(sm.R[tid][sm.ord[tid]]);
  __syncthreads();
  {
    const int c = tid >> 4, l = tid & 15;
    dfl(*X)[MAXB + 1] = sm.S;
    if (c < kept) {
      const unsigned mask = 0xFFFFu << (threadIdx.x & 16);
      if (l == 0) X[c][c] = invd[c];
      __syncwarp(mask);
      for (int a = c - 1; a >= 0; --a) {
        dfl acc = {0.f, 0.f};
        for (int u = a + 1 + l; u <= c; u += 16) acc = df_fma2(acc, sm.R[a][sm.ord[u]], X[u][c]);
#pragma unroll
        for (int o = 8; o > 0; o >>= 1)
          acc = df_add(acc, {__shfl_xor_sync(mask, acc.hi, o), __shfl_xor_sync(mask, acc.lo, o)});
        if (l == 0) X[a][c] = df_mul(df_neg(acc), invd[a]);
        __syncwarp(mask);
      }
    }
    __syncthreads();
    for (int idx = tid; idx < MAXB * MAXB; idx += blockDim.x) {
      const int a = idx / MAXB, cc = idx % MAXB;
      const dfl v = (a < kept && cc < kept && cc >= a) ? X[a][cc] : dfl{0.f, 0.f};
      Rinvg[idx] = make_float2(v.hi, v.lo);
    }
  }
  if (tid < MAXB) ordg[tid] = sm.ord[tid];
  block_swap_parallel(sm, i, kept, js, perm, diags, Jg, K1g, K2g, st);
}

// Q_blk = V(:, ord[:kept]) R11^{-1} in double-float as the product with the explicit
// inverse (k_pchol_df), written as the FP32 basis and its TF32 split (Qh = Q
// rounded to the nearest TF32 value, Ql = fp32(q - Qh); zero beyond the kept
// columns), by columns for the projection and by rows for the update.  Every output is an
// independent dot product: a CTA takes 32 rows, warp w the outputs s = w + 8q of
// every row (lane = row, so the stores coalesce), eight chains per thread.  One
// CholQR pass suffices here: with ~48-bit arithmetic the loss of orthogonality,
// ~2^-48 cond(V_kept)^2, stays far below the FP32 rounding of the stored basis for
// the conditioning the robust filter admits.
constexpr int QS_ROWS = 32;
struct QSolveSmem {
  dfl Ri[MAXB][MAXB + 1];
  float W[MAXB][QS_ROWS + 1];
  float Hr[QS_ROWS][MAXB + 1];  // the tile's hi / lo parts by rows, for the row-major copies
  float Lr[QS_ROWS][MAXB + 1];
  int ord[MAXB];
};

__global__ void __launch_bounds__(256)
k_panel_q_df(const float* __restrict__ V, int m, const State* __restrict__ st, const float2* __restrict__ Rinvg,
             const int* __restrict__ ordg, float* __restrict__ Q, int64_t ldq, float* __restrict__ Qh,
             float* __restrict__ Ql, int64_t ldh, float* __restrict__ Qrh, float* __restrict__ Qrl) {
  extern __shared__ __align__(16) unsigned char dyn_smem[];
  QSolveSmem& sm = *reinterpret_cast<QSolveSmem*>(dyn_smem);
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int kept = st->bs;
  if (kept == 0) return;
  for (int idx = tid; idx < kept * kept; idx += 256) {
    const int u = idx / kept, s = idx % kept;
    const float2 v = Rinvg[u * MAXB + s];
    sm.Ri[u][s] = dfl{v.x, v.y};
  }
  if (tid < MAXB) sm.ord[tid] = ordg[tid];
  __syncthreads();
  const int r0 = blockIdx.x * QS_ROWS;
  for (int idx = tid; idx < QS_ROWS * kept; idx += 256) {
    const int rr = idx % QS_ROWS, u = idx / QS_ROWS, r = r0 + rr;
    sm.W[u][rr] = r < m ? V[r + (int64_t)sm.ord[u] * m] : 0.f;
  }
  __syncthreads();
  dfl acc[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) acc[q] = dfl{0.f, 0.f};
  for (int u = 0; u < kept; ++u) {
    const float x = sm.W[u][lane];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int s = w + 8 * q;
      if (s < kept && u <= s) acc[q] = df_fma_f(acc[q], x, sm.Ri[u][s]);
    }
  }
  const int r = r0 + lane;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int s = w + 8 * q;
    // FP32 basis and its TF32 split, on the FP32 pipe: q = hi + lo (double-float),
    // Q = rn(q), Qh = Q rounded to the nearest TF32 value, Ql = q - Qh (hi - Qh
    // exact by Sterbenz) rounded to the nearest TF32 value: q - Qh - Ql <= 2^-23 |q|
    const dfl v = s < kept ? acc[q] : dfl{0.f, 0.f};
    const float qf = __fadd_rn(v.hi, v.lo);
    const float h = tf32_rn(qf);
    const float l = tf32_rn(__fadd_rn(v.hi - h, v.lo));
    if (r < m) {
      if (s < kept) Q[r + (int64_t)s * ldq] = qf;
      if (Qh) {
        Qh[r + (int64_t)s * ldh] = h;
        Ql[r + (int64_t)s * ldh] = l;
      }
    }
    sm.Hr[lane][s] = h;
    sm.Lr[lane][s] = l;
  }
  if (Qrh) {  // the same parts by rows (64 per row), for the tensor-core update
    __syncthreads();
    for (int idx = tid; idx < QS_ROWS * MAXB; idx += 256) {
      const int rr = idx / MAXB, s = idx % MAXB, rw = r0 + rr;
      if (rw < m) {
        Qrh[(int64_t)rw * MAXB + s] = sm.Hr[rr][s];
        Qrl[(int64_t)rw * MAXB + s] = sm.Lr[rr][s];
      }
    }
  }
}

// R(I2, I2) = R11, the panel R of a single CholQR pass (upper triangle, slot order).
__global__ void k_write_r11(const State* __restrict__ st, const float2* __restrict__ R11g, double* __restrict__ R,
                            int64_t ldr) {
  const int kept = st->bs, i = st->i;
  for (int idx = threadIdx.x; idx < kept * kept; idx += blockDim.x) {
    const int a = idx / kept, c = idx % kept;
    const float2 v = R11g[a * MAXB + c];
    R[(int64_t)(i + a) * ldr + (i + c)] = c >= a ? (double)v.x + (double)v.y : 0.0;
  }
}

}  // namespace
}  // namespace rbrp
