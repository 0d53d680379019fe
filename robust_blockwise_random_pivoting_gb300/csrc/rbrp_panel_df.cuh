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
constexpr int DF_TROWS = 64;  // panel rows per CTA of the row-solve kernels (one thread per row)

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
           int* __restrict__ perm, double* __restrict__ diags, float2* __restrict__ R11g, int* __restrict__ ordg,
           int* __restrict__ Jg, int* __restrict__ K1g, int* __restrict__ K2g) {
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
  if (tid < MAXB) ordg[tid] = sm.ord[tid];
  block_swap_parallel(sm, i, kept, js, perm, diags, Jg, K1g, K2g, st);
}

// Rows of X R^{-1} (R upper, kept x kept, double-float pairs in global) for 128 rows per CTA,
// one thread per row, in double-float; optionally the Gram partial of the result.
struct RowsDfSmem {
  dfl R[MAXB][MAXB + 1];
  dfl W[DF_TROWS][MAXB + 1];
  dfl inv[MAXB];   // 1 / R(s, s)
  int ord[MAXB];
};

// Forward substitution of each row against R (one thread per row).  The sum over
// the solved entries runs in four independent double-float chains, so the latency
// chain of a row is a quarter as long; the diagonal reciprocals are computed once.
__device__ __forceinline__ void rows_solve_df(RowsDfSmem& sm, int kept) {
  const int r = threadIdx.x;
  if (r < kept) sm.inv[r] = df_recip(sm.R[r][r]);
  __syncthreads();
  if (r < DF_TROWS) {
    for (int s = 0; s < kept; ++s) {
      dfl a0 = sm.W[r][s], a1 = {0.f, 0.f}, a2 = {0.f, 0.f}, a3 = {0.f, 0.f};
      int u = 0;
      for (; u + 4 <= s; u += 4) {
        a0 = df_fms(a0, sm.W[r][u], sm.R[u][s]);
        a1 = df_fms(a1, sm.W[r][u + 1], sm.R[u + 1][s]);
        a2 = df_fms(a2, sm.W[r][u + 2], sm.R[u + 2][s]);
        a3 = df_fms(a3, sm.W[r][u + 3], sm.R[u + 3][s]);
      }
      for (; u < s; ++u) a0 = df_fms(a0, sm.W[r][u], sm.R[u][s]);
      sm.W[r][s] = df_mul(df_add(df_add(a0, a1), df_add(a2, a3)), sm.inv[s]);
    }
  }
  __syncthreads();
}

__device__ __forceinline__ void load_R_df(RowsDfSmem& sm, const float2* __restrict__ Rg, int kept) {
  for (int idx = threadIdx.x; idx < kept * kept; idx += blockDim.x) {
    const float2 v = Rg[(idx / kept) * MAXB + idx % kept];
    sm.R[idx / kept][idx % kept] = dfl{v.x, v.y};
  }
}

// Q_blk = V(:, ord[:kept]) R11^{-1} in double-float, written as the FP32 basis and
// its exact TF32 split (Qh = tf32(Q), Ql = fp32(Q - Qh), zero beyond the kept
// columns).  One CholQR pass suffices here: with ~48-bit arithmetic the loss of
// orthogonality, ~2^-48 cond(V_kept)^2, stays far below the FP32 rounding of
// the stored basis for the conditioning the robust filter admits.
__global__ void __launch_bounds__(DF_TROWS)
k_panel_q_df(const float* __restrict__ V, int m, const State* __restrict__ st, const float2* __restrict__ R11g,
             const int* __restrict__ ordg, float* __restrict__ Q, int64_t ldq, float* __restrict__ Qh,
             float* __restrict__ Ql, int64_t ldh) {
  extern __shared__ __align__(16) unsigned char dyn_smem[];
  RowsDfSmem& sm = *reinterpret_cast<RowsDfSmem*>(dyn_smem);
  const int tid = threadIdx.x;
  const int kept = st->bs;
  if (kept == 0) return;
  load_R_df(sm, R11g, kept);
  if (tid < MAXB) sm.ord[tid] = ordg[tid];
  __syncthreads();
  const int r0 = blockIdx.x * DF_TROWS;
  for (int idx = tid; idx < DF_TROWS * kept; idx += DF_TROWS) {
    const int rr = idx % DF_TROWS, s = idx / DF_TROWS, r = r0 + rr;
    sm.W[rr][s] = {r < m ? V[r + (int64_t)sm.ord[s] * m] : 0.f, 0.f};
  }
  __syncthreads();
  rows_solve_df(sm, kept);
  for (int idx = tid; idx < DF_TROWS * MAXB; idx += DF_TROWS) {
    const int rr = idx % DF_TROWS, s = idx / DF_TROWS, r = r0 + rr;
    if (r < m) {
      // FP32 basis and its exact TF32 split, on the FP32 pipe: q = hi + lo (double-float),
      // Q = rn(q), Qh = tf32(Q), Ql = rn(q - Qh) with hi - Qh exact (Sterbenz)
      const dfl w = s < kept ? sm.W[rr][s] : dfl{0.f, 0.f};
      const float qf = __fadd_rn(w.hi, w.lo);
      if (s < kept) Q[r + (int64_t)s * ldq] = qf;
      if (Qh) {
        const float h = __uint_as_float(__float_as_uint(qf) & 0xFFFFE000u);
        Qh[r + (int64_t)s * ldh] = h;
        Ql[r + (int64_t)s * ldh] = __fadd_rn(w.hi - h, w.lo);
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
