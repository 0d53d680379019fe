// rbrp_panel_df.cuh - panel CPQR / CholQR2 of the FP32 residual form in
// double-float arithmetic.
//
// GB300's FP64 pipe issues ~1/64 of the FP32 pipe's rate, and the panel work
// (Gram matrices, two row solves, two small Cholesky factorisations per block)
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

namespace rbrp {
namespace {

struct dfl {
  float hi, lo;
};

__device__ __forceinline__ dfl df_of(double x) {
  const float h = (float)x;
  return {h, (float)(x - (double)h)};
}
__device__ __forceinline__ double df_dbl(dfl a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ dfl df_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ dfl df_fast(float a, float b) {
  const float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
  dfl s = df_two_sum(a.hi, b.hi);
  s.lo += a.lo + b.lo;
  return df_fast(s.hi, s.lo);
}
__device__ __forceinline__ dfl df_neg(dfl a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ dfl df_mul(dfl a, dfl b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return df_fast(p, e);
}
// s - a * b
__device__ __forceinline__ dfl df_fms(dfl s, dfl a, dfl b) { return df_add(s, df_neg(df_mul(a, b))); }
__device__ __forceinline__ dfl df_recip(dfl b) {
  const float q = 1.0f / b.hi;
  const dfl r = df_add({1.0f, 0.0f}, df_neg(df_mul({q, 0.0f}, b)));  // 1 - q b
  return df_fast(q, q * r.hi);
}
__device__ __forceinline__ dfl df_sqrt(dfl a) {
  if (!(a.hi > 0.0f)) return {0.0f, 0.0f};
  const float s = sqrtf(a.hi);
  const dfl e = df_add(a, df_neg(df_mul({s, 0.0f}, {s, 0.0f})));  // a - s^2
  return df_fast(s, e.hi / (2.0f * s));
}
// exact product of two floats, accumulated
__device__ __forceinline__ void df_acc_prod(dfl& acc, float x, float y) {
  const float p = x * y;
  const float e = fmaf(x, y, -p);
  dfl s = df_two_sum(acc.hi, p);
  s.lo += acc.lo + e;
  acc = df_fast(s.hi, s.lo);
}

constexpr int DF_ROWS = 128;  // panel rows per CTA in the row kernels

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
  for (int q = 0; q < 16; ++q) {
    const int c2 = (tid & 3) + 4 * q;
    if (c2 < c1) continue;
    dfl acc = {0.f, 0.f};
    if (c1 < bss && c2 < bss)
      for (int rr = 0; rr < DF_ROWS; ++rr) df_acc_prod(acc, Vs[rr][c1], Vs[rr][c2]);
    const double g = df_dbl(acc);
    G[c1 * MAXB + c2] = g;
    G[c2 * MAXB + c1] = g;
  }
}

struct PcholDfSmem {
  dfl S[MAXB][MAXB + 1];   // Schur complement, indexed by panel column
  dfl R[MAXB][MAXB + 1];   // R[t][j]: row t of the factor, by panel column j
  int ord[MAXB];           // slot -> panel column
  int alive[MAXB];
  int stop, piv;
  dfl inv;
};

// Pivoted Cholesky of the panel Gram matrix with the robust filter (same rule as
// pivoted_chol_filter), 256 threads, no data movement for the swaps.  CTA 0
// publishes R11 (slot order, FP64), ord, the kept count and does the block swap.
__global__ void __launch_bounds__(256)
k_pchol_df(const double* __restrict__ G, int m, State* st, double tol_loc, const int* __restrict__ js,
           int* __restrict__ perm, double* __restrict__ diags, double* __restrict__ R11g, int* __restrict__ ordg,
           int* __restrict__ Jg, int* __restrict__ K1g, int* __restrict__ K2g) {
  extern __shared__ __align__(16) unsigned char dyn_smem[];
  PcholDfSmem& sm = *reinterpret_cast<PcholDfSmem*>(dyn_smem);
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int nb = st->bs_sampled, i = st->i;
  const int rows = min(nb, m);
  for (int idx = tid; idx < nb * nb; idx += 256) sm.S[idx / nb][idx % nb] = df_of(G[(idx / nb) * MAXB + idx % nb]);
  if (tid < MAXB) {
    sm.ord[tid] = tid;
    sm.alive[tid] = tid < nb;
  }
  __syncthreads();
  // total = trace(G) in double-float
  float tot_hi = 0.f;
  double total = 0.0;
  if (wid == 0) {
    dfl t = {0.f, 0.f};
    for (int s = 0; s < nb; ++s) t = df_add(t, sm.S[s][s]);
    total = df_dbl(t);
    (void)tot_hi;
  }
  int kept = rows;
  for (int t = 0; t < rows; ++t) {
    if (wid == 0) {
      // remaining trace and the first maximal slot (LAPACK dgeqp3 order)
      dfl rem = {0.f, 0.f};
      double best = -1.0;
      int bs = nb;
      for (int s = t + lane; s < nb; s += 32) {
        const dfl d = sm.S[sm.ord[s]][sm.ord[s]];
        rem = df_add(rem, d);
        const double dv = df_dbl(d);
        if (dv > best) { best = dv; bs = s; }
      }
      double remv = df_dbl(rem);
      remv = warp_sum(remv);
      remv = __shfl_sync(0xffffffffu, remv, 0);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_down_sync(0xffffffffu, best, o);
        const int oi = __shfl_down_sync(0xffffffffu, bs, o);
        if (ob > best || (ob == best && oi < bs)) { best = ob; bs = oi; }
      }
      if (lane == 0) {
        const double tt = total;
        const bool stop = !(tt > 0.0) || (remv / tt < tol_loc) || !(best > 0.0);
        sm.stop = stop;
        if (!stop) {
          const int o = sm.ord[t];
          sm.ord[t] = sm.ord[bs];
          sm.ord[bs] = o;
          const int pv = sm.ord[t];
          sm.alive[pv] = 0;
          const dfl r = df_sqrt(sm.S[pv][pv]);
          sm.R[t][pv] = r;
          sm.inv = df_recip(r);
          sm.piv = pv;
        }
      }
    }
    __syncthreads();
    if (sm.stop) { kept = t; break; }
    const int pv = sm.piv;
    const dfl inv = sm.inv;
    for (int j = tid; j < nb; j += 256)
      if (sm.alive[j]) sm.R[t][j] = df_mul(sm.S[pv][j], inv);
    __syncthreads();
    // Schur complement over the alive columns (full square: rows j1, columns j2)
    for (int idx = tid; idx < nb * nb; idx += 256) {
      const int j1 = idx / nb, j2 = idx % nb;
      if (sm.alive[j1] && sm.alive[j2]) sm.S[j1][j2] = df_fms(sm.S[j1][j2], sm.R[t][j1], sm.R[t][j2]);
    }
    __syncthreads();
  }
  // R11 in slot order: R11[a][c] = R[a][ord[c]] for c >= a
  for (int idx = tid; idx < MAXB * MAXB; idx += 256) {
    const int a = idx / MAXB, c = idx % MAXB;
    R11g[idx] = (a < kept && c < kept && c >= a) ? df_dbl(sm.R[a][sm.ord[c]]) : 0.0;
  }
  if (tid < MAXB) ordg[tid] = sm.ord[tid];
  if (tid == 0) {
    int J[MAXB], K1[MAXB], K2[MAXB];
    int nK = 0;
    for (int s = 0; s < kept; ++s) J[s] = js[sm.ord[s]];
    int nk1 = 0;
    for (int p = i; p < i + kept; ++p) {
      bool in = false;
      for (int s = 0; s < kept; ++s) in |= (J[s] == p);
      if (!in) K1[nk1++] = p;
    }
    for (int s = 0; s < kept; ++s)
      if (J[s] < i || J[s] >= i + kept) K2[nK++] = J[s];
    int Tperm[MAXB];
    for (int s = 0; s < kept; ++s) Tperm[s] = perm[J[s]];
    for (int t = 0; t < nK; ++t) {
      perm[K2[t]] = perm[K1[t]];
      diags[K2[t]] = diags[K1[t]];
    }
    for (int s = 0; s < kept; ++s) perm[i + s] = Tperm[s];
    for (int s = 0; s < kept; ++s) Jg[s] = J[s];
    for (int t = 0; t < nK; ++t) { K1g[t] = K1[t]; K2g[t] = K2[t]; }
    st->bs = kept;
    st->nK = nK;
    st->zero_panel = kept == 0;
  }
}

// Rows of X R^{-1} (R upper, kept x kept, FP64 in global) for 128 rows per CTA,
// one thread per row, in double-float; optionally the Gram partial of the result.
struct RowsDfSmem {
  dfl R[MAXB][MAXB + 1];
  dfl W[DF_ROWS][MAXB + 1];
  int ord[MAXB];
};

__device__ __forceinline__ void rows_solve_df(RowsDfSmem& sm, int kept) {
  const int r = threadIdx.x;
  if (r < DF_ROWS) {
    for (int s = 0; s < kept; ++s) {
      dfl x = sm.W[r][s];
      for (int u = 0; u < s; ++u) x = df_fms(x, sm.W[r][u], sm.R[u][s]);
      sm.W[r][s] = df_mul(x, df_recip(sm.R[s][s]));
    }
  }
  __syncthreads();
}

__device__ __forceinline__ void load_R_df(RowsDfSmem& sm, const double* __restrict__ Rg, int kept) {
  for (int idx = threadIdx.x; idx < kept * kept; idx += blockDim.x)
    sm.R[idx / kept][idx % kept] = df_of(Rg[(idx / kept) * MAXB + idx % kept]);
}

// Q1 = V(:, ord[:kept]) R11^{-1} (double-float, stored as float pairs) and Q1^T Q1 partials.
__global__ void __launch_bounds__(DF_ROWS)
k_panel1_df(const float* __restrict__ V, int m, const State* __restrict__ st, const double* __restrict__ R11g,
            const int* __restrict__ ordg, float2* __restrict__ Q1, double* __restrict__ G2part) {
  extern __shared__ __align__(16) unsigned char dyn_smem[];
  RowsDfSmem& sm = *reinterpret_cast<RowsDfSmem*>(dyn_smem);
  const int tid = threadIdx.x;
  const int kept = st->bs;
  if (kept == 0) return;
  load_R_df(sm, R11g, kept);
  if (tid < MAXB) sm.ord[tid] = ordg[tid];
  __syncthreads();
  const int r0 = blockIdx.x * DF_ROWS;
  for (int idx = tid; idx < DF_ROWS * kept; idx += DF_ROWS) {
    const int rr = idx % DF_ROWS, s = idx / DF_ROWS, r = r0 + rr;
    sm.W[rr][s] = {r < m ? V[r + (int64_t)sm.ord[s] * m] : 0.f, 0.f};
  }
  __syncthreads();
  rows_solve_df(sm, kept);
  for (int idx = tid; idx < DF_ROWS * kept; idx += DF_ROWS) {
    const int rr = idx % DF_ROWS, s = idx / DF_ROWS, r = r0 + rr;
    if (r < m) Q1[r + (int64_t)s * m] = make_float2(sm.W[rr][s].hi, sm.W[rr][s].lo);
  }
  // Gram partial (upper triangle, mirrored): thread -> (c1, c2) pairs
  double* G = G2part + (int64_t)blockIdx.x * MAXB * MAXB;
  const int rows_valid = max(0, min(DF_ROWS, m - r0));
  for (int pair = tid; pair < MAXB * MAXB; pair += DF_ROWS) {
    const int c1 = pair / MAXB, c2 = pair % MAXB;
    if (c2 < c1) continue;
    dfl acc = {0.f, 0.f};
    if (c1 < kept && c2 < kept)
      for (int rr = 0; rr < rows_valid; ++rr) acc = df_add(acc, df_mul(sm.W[rr][c1], sm.W[rr][c2]));
    const double g = df_dbl(acc);
    G[c1 * MAXB + c2] = g;
    G[c2 * MAXB + c1] = g;
  }
}

// R2 = chol(Q1^T Q1) (one CTA, double-float) and the panel R = R2 R11 into R(I2, I2).
__global__ void __launch_bounds__(256)
k_chol2_df(const double* __restrict__ G2, const State* __restrict__ st, const double* __restrict__ R11g,
           double* __restrict__ R2g, double* __restrict__ R, int64_t ldr) {
  extern __shared__ __align__(16) unsigned char dyn_smem[];
  PcholDfSmem& sm = *reinterpret_cast<PcholDfSmem*>(dyn_smem);
  const int tid = threadIdx.x;
  const int kept = st->bs, i = st->i;
  if (kept == 0) return;
  for (int idx = tid; idx < kept * kept; idx += 256) sm.S[idx / kept][idx % kept] = df_of(G2[(idx / kept) * MAXB + idx % kept]);
  __syncthreads();
  for (int t = 0; t < kept; ++t) {
    if (tid == 0) {
      const dfl r = df_sqrt(sm.S[t][t]);
      sm.R[t][t] = r;
      sm.inv = df_recip(r);
    }
    __syncthreads();
    const dfl inv = sm.inv;
    for (int s = t + 1 + tid; s < kept; s += 256) sm.R[t][s] = df_mul(sm.S[t][s], inv);
    __syncthreads();
    const int w = kept - t - 1;
    for (int idx = tid; idx < w * w; idx += 256) {
      const int s1 = t + 1 + idx / w, s2 = t + 1 + idx % w;
      if (s2 >= s1) sm.S[s1][s2] = df_fms(sm.S[s1][s2], sm.R[t][s1], sm.R[t][s2]);
    }
    __syncthreads();
  }
  for (int idx = tid; idx < MAXB * MAXB; idx += 256) {
    const int a = idx / MAXB, c = idx % MAXB;
    R2g[idx] = (a < kept && c < kept && c >= a) ? df_dbl(sm.R[a][c]) : 0.0;
  }
  for (int idx = tid; idx < kept * kept; idx += 256) {
    const int a = idx / kept, c = idx % kept;
    dfl v = {0.f, 0.f};
    if (c >= a)
      for (int u = a; u <= c; ++u) v = df_add(v, df_mul(sm.R[a][u], df_of(R11g[u * MAXB + c])));
    R[(int64_t)(i + a) * ldr + (i + c)] = df_dbl(v);
  }
}

// Q_blk = Q1 R2^{-1}: FP32 basis for the residual update and its exact TF32
// split (Qh = tf32(Q), Ql = fp32(Q - Qh), zero beyond the kept columns).
__global__ void __launch_bounds__(DF_ROWS)
k_panel2_df(const float2* __restrict__ Q1, int m, const State* __restrict__ st, const double* __restrict__ R2g,
            float* __restrict__ Q, int64_t ldq, float* __restrict__ Qh, float* __restrict__ Ql, int64_t ldh) {
  extern __shared__ __align__(16) unsigned char dyn_smem[];
  RowsDfSmem& sm = *reinterpret_cast<RowsDfSmem*>(dyn_smem);
  const int tid = threadIdx.x;
  const int kept = st->bs;
  if (kept == 0) return;
  load_R_df(sm, R2g, kept);
  const int r0 = blockIdx.x * DF_ROWS;
  for (int idx = tid; idx < DF_ROWS * kept; idx += DF_ROWS) {
    const int rr = idx % DF_ROWS, s = idx / DF_ROWS, r = r0 + rr;
    const float2 v = r < m ? Q1[r + (int64_t)s * m] : make_float2(0.f, 0.f);
    sm.W[rr][s] = {v.x, v.y};
  }
  __syncthreads();
  rows_solve_df(sm, kept);
  for (int idx = tid; idx < DF_ROWS * MAXB; idx += DF_ROWS) {
    const int rr = idx % DF_ROWS, s = idx / DF_ROWS, r = r0 + rr;
    if (r < m) {
      const double q = s < kept ? df_dbl(sm.W[rr][s]) : 0.0;
      if (s < kept) Q[r + (int64_t)s * ldq] = (float)q;
      if (Qh) {
        const float h = __uint_as_float(__float_as_uint((float)q) & 0xFFFFE000u);
        Qh[r + (int64_t)s * ldh] = h;
        Ql[r + (int64_t)s * ldh] = (float)(q - (double)h);
      }
    }
  }
}

}  // namespace
}  // namespace rbrp
