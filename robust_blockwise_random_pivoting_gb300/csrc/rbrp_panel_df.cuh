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
// s - a * b (one error-free product, one TwoSum)
__device__ __forceinline__ dfl df_fms(dfl s, dfl a, dfl b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  const dfl t = df_two_sum(s.hi, -p);
  return df_fast(t.hi, t.lo + (s.lo - e));
}
// acc + a * b
__device__ __forceinline__ dfl df_fma2(dfl acc, dfl a, dfl b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  const dfl t = df_two_sum(acc.hi, p);
  return df_fast(t.hi, t.lo + (acc.lo + e));
}
__device__ __forceinline__ bool df_gt(dfl a, dfl b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }
__device__ __forceinline__ bool df_eq(dfl a, dfl b) { return a.hi == b.hi && a.lo == b.lo; }
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

struct PcholDfSmem {
  dfl S[MAXB][MAXB + 1];   // Schur complement, indexed by panel column
  dfl R[MAXB][MAXB + 1];   // R[t][j]: row t of the factor, by panel column j
  int ord[MAXB];           // slot -> panel column
  int alive[MAXB];
  int J[MAXB], K1[MAXB], K2[MAXB], inblk[MAXB], Tperm[MAXB];
  double Tdiag[MAXB];
  int stop, piv, nK;
  dfl inv;
};

// Block swap of perm and diags (matlab/RBRP.m:81-99), in parallel: K1 = block
// positions not kept (ascending), K2 = kept positions outside the block (pivot
// order), compacted with warp ballots.  All threads call it after `kept` is known.
__device__ void block_swap_parallel(PcholDfSmem& sm, int i, int kept, const int* __restrict__ js,
                                    int* __restrict__ perm, double* __restrict__ diags, int* __restrict__ Jg,
                                    int* __restrict__ K1g, int* __restrict__ K2g, State* st) {
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  if (tid < MAXB) sm.inblk[tid] = 0;
  __syncthreads();
  if (tid < kept) {
    const int p = js[sm.ord[tid]];
    sm.J[tid] = p;
    Jg[tid] = p;
    if (p >= i && p < i + kept) sm.inblk[p - i] = 1;
    sm.Tperm[tid] = perm[p];
  }
  __syncthreads();
  if (wid < 2) {
    // warp 0: K1 (block positions not kept), warp 1: K2 (kept positions outside the block)
    int count = 0;
    for (int base = 0; base < kept; base += 32) {
      const int t = base + lane;
      bool flag = false;
      int val = 0;
      if (t < kept) {
        if (wid == 0) { flag = !sm.inblk[t]; val = i + t; }
        else { const int p = sm.J[t]; flag = p < i || p >= i + kept; val = p; }
      }
      const unsigned bal = __ballot_sync(0xffffffffu, flag);
      if (flag) {
        const int slot = count + __popc(bal & ((1u << lane) - 1u));
        if (wid == 0) sm.K1[slot] = val; else sm.K2[slot] = val;
      }
      count += __popc(bal);
    }
    if (wid == 1 && lane == 0) sm.nK = count;
  }
  __syncthreads();
  const int nK = sm.nK;
  if (tid < nK) {  // perm(K2) = perm(K1), diags(K2) = diags(K1): K1 inside the block, K2 outside
    const int a = sm.K1[tid], b = sm.K2[tid];
    const int pa = perm[a];
    const double da = diags[a];
    perm[b] = pa;
    diags[b] = da;
    K1g[tid] = a;
    K2g[tid] = b;
  }
  __syncthreads();
  if (tid < kept) perm[i + tid] = sm.Tperm[tid];
  if (tid == 0) {
    st->bs = kept;
    st->nK = nK;
    st->zero_panel = kept == 0;
  }
}

// Pivoted Cholesky of the panel Gram matrix with the robust filter (same rule as
// pivoted_chol_filter), 256 threads, no data movement for the swaps.  Publishes
// R11 (slot order, FP64), ord, the kept count and performs the block swap.
__global__ void __launch_bounds__(256)
k_pchol_df(const double* __restrict__ G, int m, State* st, double tol_loc, const int* __restrict__ js,
           int* __restrict__ perm, double* __restrict__ diags, double* __restrict__ R11g, int* __restrict__ ordg,
           int* __restrict__ Jg, int* __restrict__ K1g, int* __restrict__ K2g) {
  extern __shared__ __align__(16) unsigned char dyn_smem[];
  PcholDfSmem& sm = *reinterpret_cast<PcholDfSmem*>(dyn_smem);
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int nb = st->bs_sampled, i = st->i;
  const int rows = min(nb, m);
  const int ty = tid >> 4, tx = tid & 15;  // 4 x 4 Schur entries per thread: rows ty*4+u, columns tx*4+v
  for (int idx = tid; idx < MAXB * MAXB; idx += 256) {
    const int a = idx / MAXB, c = idx % MAXB;
    sm.S[a][c] = (a < nb && c < nb) ? df_of(G[a * MAXB + c]) : dfl{0.f, 0.f};
  }
  if (tid < MAXB) {
    sm.ord[tid] = tid;
    sm.alive[tid] = tid < nb;
  }
  __syncthreads();
  double total = 0.0;  // trace(G), used by warp 0
  if (wid == 0) {
    dfl t = {0.f, 0.f};
    for (int s2 = 0; s2 < nb; ++s2) t = df_add(t, sm.S[s2][s2]);
    total = df_dbl(t);
  }
  int kept = rows;
  for (int t = 0; t < rows; ++t) {
    if (wid == 0) {
      // remaining trace and the first maximal slot (LAPACK dgeqp3 order)
      dfl rem = {0.f, 0.f}, best = {-1.f, 0.f};
      int bs = nb;
      for (int s2 = t + lane; s2 < nb; s2 += 32) {
        const dfl d = sm.S[sm.ord[s2]][sm.ord[s2]];
        rem = df_add(rem, d);
        if (df_gt(d, best)) { best = d; bs = s2; }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const dfl orem = {__shfl_down_sync(0xffffffffu, rem.hi, o), __shfl_down_sync(0xffffffffu, rem.lo, o)};
        rem = df_add(rem, orem);
        const dfl ob = {__shfl_down_sync(0xffffffffu, best.hi, o), __shfl_down_sync(0xffffffffu, best.lo, o)};
        const int oi = __shfl_down_sync(0xffffffffu, bs, o);
        if (df_gt(ob, best) || (df_eq(ob, best) && oi < bs)) { best = ob; bs = oi; }
      }
      if (lane == 0) {
        const bool stop = !(total > 0.0) || (df_dbl(rem) / total < tol_loc) || !(best.hi > 0.f);
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
    if (tid < nb && sm.alive[tid]) sm.R[t][tid] = df_mul(sm.S[pv][tid], inv);
    __syncthreads();
    dfl ru[4], rv[4];
    bool au[4], av[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int j = ty * 4 + u;
      au[u] = j < nb && sm.alive[j];
      ru[u] = sm.R[t][j];
      const int c = tx * 4 + u;
      av[u] = c < nb && sm.alive[c];
      rv[u] = sm.R[t][c];
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v)
        if (au[u] && av[v]) sm.S[ty * 4 + u][tx * 4 + v] = df_fms(sm.S[ty * 4 + u][tx * 4 + v], ru[u], rv[v]);
    __syncthreads();
  }
  // R11 in slot order: R11[a][c] = R[a][ord[c]] for c >= a
  for (int idx = tid; idx < MAXB * MAXB; idx += 256) {
    const int a = idx / MAXB, c = idx % MAXB;
    R11g[idx] = (a < kept && c < kept && c >= a) ? df_dbl(sm.R[a][sm.ord[c]]) : 0.0;
  }
  if (tid < MAXB) ordg[tid] = sm.ord[tid];
  block_swap_parallel(sm, i, kept, js, perm, diags, Jg, K1g, K2g, st);
}

// Rows of X R^{-1} (R upper, kept x kept, FP64 in global) for 128 rows per CTA,
// one thread per row, in double-float; optionally the Gram partial of the result.
struct RowsDfSmem {
  dfl R[MAXB][MAXB + 1];
  dfl W[DF_TROWS][MAXB + 1];
  int ord[MAXB];
};

__device__ __forceinline__ void rows_solve_df(RowsDfSmem& sm, int kept) {
  const int r = threadIdx.x;
  if (r < DF_TROWS) {
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
__global__ void __launch_bounds__(DF_TROWS)
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
  const int r0 = blockIdx.x * DF_TROWS;
  for (int idx = tid; idx < DF_TROWS * kept; idx += DF_TROWS) {
    const int rr = idx % DF_TROWS, s = idx / DF_TROWS, r = r0 + rr;
    sm.W[rr][s] = {r < m ? V[r + (int64_t)sm.ord[s] * m] : 0.f, 0.f};
  }
  __syncthreads();
  rows_solve_df(sm, kept);
  for (int idx = tid; idx < DF_TROWS * kept; idx += DF_TROWS) {
    const int rr = idx % DF_TROWS, s = idx / DF_TROWS, r = r0 + rr;
    if (r < m) Q1[r + (int64_t)s * m] = make_float2(sm.W[rr][s].hi, sm.W[rr][s].lo);
  }
  // Gram partial: thread -> column c1 = tid, all 64 columns c2 (64 independent chains
  // would not fit; 16 at a time)
  double* G = G2part + (int64_t)blockIdx.x * MAXB * MAXB;
  const int rows_valid = max(0, min(DF_TROWS, m - r0));
  const int c1 = tid;
  for (int q0 = 0; q0 < MAXB; q0 += 16) {
    dfl acc[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) acc[q] = {0.f, 0.f};
    if (c1 < kept) {
      for (int rr = 0; rr < rows_valid; ++rr) {
        const dfl x = sm.W[rr][c1];
#pragma unroll
        for (int q = 0; q < 16; ++q) acc[q] = df_fma2(acc[q], x, sm.W[rr][q0 + q]);
      }
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int c2 = q0 + q;
      G[c1 * MAXB + c2] = (c1 < kept && c2 < kept) ? df_dbl(acc[q]) : 0.0;
    }
  }
}

// Q_blk = V(:, ord[:kept]) R11^{-1} in double-float, written as the FP32 basis and
// its exact TF32 split (Qh = tf32(Q), Ql = fp32(Q - Qh), zero beyond the kept
// columns).  One CholQR pass suffices here: with ~48-bit arithmetic the loss of
// orthogonality, ~2^-48 cond(V_kept)^2, stays far below the FP32 rounding of
// the stored basis for the conditioning the robust filter admits.
__global__ void __launch_bounds__(DF_TROWS)
k_panel_q_df(const float* __restrict__ V, int m, const State* __restrict__ st, const double* __restrict__ R11g,
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

// R(I2, I2) = R11, the panel R of a single CholQR pass (upper triangle, slot order).
__global__ void k_write_r11(const State* __restrict__ st, const double* __restrict__ R11g, double* __restrict__ R,
                            int64_t ldr) {
  const int kept = st->bs, i = st->i;
  for (int idx = threadIdx.x; idx < kept * kept; idx += blockDim.x) {
    const int a = idx / kept, c = idx % kept;
    R[(int64_t)(i + a) * ldr + (i + c)] = c >= a ? R11g[a * MAXB + c] : 0.0;
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
  const int ty = tid >> 4, tx = tid & 15;
  for (int t = 0; t < kept; ++t) {
    if (tid == 0) {
      const dfl r = df_sqrt(sm.S[t][t]);
      sm.R[t][t] = r;
      sm.inv = df_recip(r);
    }
    __syncthreads();
    const dfl inv = sm.inv;
    if (tid > t && tid < kept) sm.R[t][tid] = df_mul(sm.S[t][tid], inv);
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int s1 = ty * 4 + u;
      if (s1 <= t || s1 >= kept) continue;
      const dfl r1 = sm.R[t][s1];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int s2 = tx * 4 + v;
        if (s2 >= s1 && s2 < kept) sm.S[s1][s2] = df_fms(sm.S[s1][s2], r1, sm.R[t][s2]);
      }
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
__global__ void __launch_bounds__(DF_TROWS)
k_panel2_df(const float2* __restrict__ Q1, int m, const State* __restrict__ st, const double* __restrict__ R2g,
            float* __restrict__ Q, int64_t ldq, float* __restrict__ Qh, float* __restrict__ Ql, int64_t ldh) {
  extern __shared__ __align__(16) unsigned char dyn_smem[];
  RowsDfSmem& sm = *reinterpret_cast<RowsDfSmem*>(dyn_smem);
  const int tid = threadIdx.x;
  const int kept = st->bs;
  if (kept == 0) return;
  load_R_df(sm, R2g, kept);
  const int r0 = blockIdx.x * DF_TROWS;
  for (int idx = tid; idx < DF_TROWS * kept; idx += DF_TROWS) {
    const int rr = idx % DF_TROWS, s = idx / DF_TROWS, r = r0 + rr;
    const float2 v = r < m ? Q1[r + (int64_t)s * m] : make_float2(0.f, 0.f);
    sm.W[rr][s] = {v.x, v.y};
  }
  __syncthreads();
  rows_solve_df(sm, kept);
  for (int idx = tid; idx < DF_TROWS * MAXB; idx += DF_TROWS) {
    const int rr = idx % DF_TROWS, s = idx / DF_TROWS, r = r0 + rr;
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
