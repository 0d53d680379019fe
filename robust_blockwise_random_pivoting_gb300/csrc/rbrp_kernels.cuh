// rbrp_kernels.cuh - sm_103a kernels of one adaptive RBRP block step.
//
// Per block (positions [i, i+bs) are filled), in launch order:
//   k_sample      weighted block sampling (np-compat / exponential keys / greedy)
//   k_cgs_coef    C = Q(:, :i)^T A(:, J)            (split-m partials)
//   k_cgs_update  V = A(:, J) - Q(:, :i) C, Gram partials V^T V
//   k_panel1      pivoted Cholesky of V^T V = CPQR pivots + robust filter,
//                 Q1 = V_p R11^{-1}, Gram partials Q1^T Q1, block swap
//   k_swap_R      R(:i, K2) = R(:i, K1), R(:i, I2) = R(:i, J)
//   k_panel2      second CholQR pass: Q_blk = Q1 R2^{-1}, R(I2, I2) = R2 R11
//   k_project     W = Q_blk^T A(:, perm[p]) for the remaining positions p,
//                 R(I2, p) = W, diags(p) -= ||W(:, p)||^2 (clipped at 0);
//                 k_project_skinny for blocks of b <= 8 (column streams)
//   k_finish      residual, stop rule, per-block trace
#pragma once
#include <type_traits>
#include "rbrp_common.cuh"
#include "rbrp_df.cuh"
#include "rbrp_sampler.cuh"

namespace rbrp {
// Internal linkage: this header is compiled into one translation unit per
// element type, and each keeps its own copy of the type-independent kernels.
namespace {

// ===========================================================================
// a1: squared column norms (initial weights) - one HBM pass over A.
// gpu/rbrp.cu:82-99,352-356; python/RBRP.ipynb cell 11 lines 93-94.
// One warp per column, 16-byte vector loads when the column starts are
// 16-byte aligned, four loads in flight per lane.
// ===========================================================================
__device__ __forceinline__ double col_sumsq(const double* __restrict__ col, int m, int lane, bool vec) {
  double s0 = 0.0, s1 = 0.0;
  if (vec) {
    const double2* c2 = reinterpret_cast<const double2*>(col);
    const int m2 = m >> 1;
    int r = lane;
    for (; r + 96 < m2; r += 128) {
      const double2 a = __ldg(c2 + r), b = __ldg(c2 + r + 32), c = __ldg(c2 + r + 64), d = __ldg(c2 + r + 96);
      s0 = fma(a.x, a.x, s0); s1 = fma(a.y, a.y, s1);
      s0 = fma(b.x, b.x, s0); s1 = fma(b.y, b.y, s1);
      s0 = fma(c.x, c.x, s0); s1 = fma(c.y, c.y, s1);
      s0 = fma(d.x, d.x, s0); s1 = fma(d.y, d.y, s1);
    }
    for (; r < m2; r += 32) {
      const double2 a = __ldg(c2 + r);
      s0 = fma(a.x, a.x, s0); s1 = fma(a.y, a.y, s1);
    }
    if ((m & 1) && lane == 0) { const double v = col[m - 1]; s0 = fma(v, v, s0); }
  } else {
    for (int r = lane; r < m; r += 32) { const double v = col[r]; s0 = fma(v, v, s0); }
  }
  return warp_sum(s0 + s1);
}

__device__ __forceinline__ double col_sumsq(const float* __restrict__ col, int m, int lane, bool vec) {
  DF acc{0.f, 0.f};
  if (vec) {
    const float4* c4 = reinterpret_cast<const float4*>(col);
    const int m4 = m >> 2;
    int r = lane;
    for (; r + 96 < m4; r += 128) {
      const float4 a = __ldg(c4 + r), b = __ldg(c4 + r + 32), c = __ldg(c4 + r + 64), d = __ldg(c4 + r + 96);
      df_add_sq(acc, a.x); df_add_sq(acc, a.y); df_add_sq(acc, a.z); df_add_sq(acc, a.w);
      df_add_sq(acc, b.x); df_add_sq(acc, b.y); df_add_sq(acc, b.z); df_add_sq(acc, b.w);
      df_add_sq(acc, c.x); df_add_sq(acc, c.y); df_add_sq(acc, c.z); df_add_sq(acc, c.w);
      df_add_sq(acc, d.x); df_add_sq(acc, d.y); df_add_sq(acc, d.z); df_add_sq(acc, d.w);
    }
    for (; r < m4; r += 32) {
      const float4 a = __ldg(c4 + r);
      df_add_sq(acc, a.x); df_add_sq(acc, a.y); df_add_sq(acc, a.z); df_add_sq(acc, a.w);
    }
    for (int t = (m4 << 2) + lane; t < m; t += 32) df_add_sq(acc, col[t]);
  } else {
    for (int r = lane; r < m; r += 32) df_add_sq(acc, col[r]);
  }
  return warp_sum((double)acc.hi + (double)acc.lo);
}

template <typename T>
__global__ void __launch_bounds__(256) k_colnorm(const T* __restrict__ A, int64_t lda, int m, int n,
                                                 double* __restrict__ diags, int* __restrict__ perm,
                                                 State* st) {
  const int lane = threadIdx.x & 31;
  const int c = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (c >= n) return;
  const bool vec = ((reinterpret_cast<uintptr_t>(A) & 15) == 0) && ((lda * (int64_t)sizeof(T)) % 16 == 0);
  const double s = col_sumsq(A + (int64_t)c * lda, m, lane, vec);
  if (lane == 0) {
    diags[c] = s;
    perm[c] = c;
    if (!isfinite(s)) st->status = ST_ERR_NUMERIC;
  }
}

// Initial totals and loop state.  One CTA.
__global__ void __launch_bounds__(1024) k_init(State* st, const double* __restrict__ diags, int n, int kmax) {
  __shared__ double shd[32];
  __shared__ int shi[32];
  double s = 0.0;
  int c = 0;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    const double d = diags[j];
    s += d;
    c += d > 0.0;
  }
  s = block_sum(s, shd);
  c = block_sum(c, shi);
  if (threadIdx.x == 0) {
    st->i = 0;
    st->bs_sampled = 0;
    st->bs = 0;
    st->nblocks = 0;
    st->zero_panel = 0;
    st->nK = 0;
    st->recomputes = 0;
    st->attempts = 0;
    st->draws = 0ull;
    st->res0 = s;
    st->residual = s;
    st->nnz_rem = c;
    st->done = (c == 0 || kmax <= 0 || st->status != 0) ? 1 : 0;
  }
}

__global__ void __launch_bounds__(SAMPLE_THREADS)
k_sample(State* st, const double* __restrict__ diags, const int* __restrict__ perm, int n, int kmax,
         int b, uint64_t seed, int sampler, double* __restrict__ pbuf,
         unsigned long long* __restrict__ kbuf, int* __restrict__ js, int* __restrict__ cols,
         const int* __restrict__ order_of) {
  sample_block(st, diags, perm, n, kmax, b, seed, sampler, pbuf, kbuf, js, cols, order_of);
}

// ===========================================================================
// a3: block Gram-Schmidt against the current basis (one CGS pass, as
// python/RBRP.ipynb cell 11 line 120 and matlab/RBRP.m:55).
// ===========================================================================
// Cpart[z][a*MAXB + c] = sum over rows of split z of Q(r, a) * A(r, cols[c]).
template <typename T>
__global__ void __launch_bounds__(256)
k_cgs_coef(const T* __restrict__ Q, int64_t ldq, const T* __restrict__ A, int64_t lda,
           const int* __restrict__ cols, const State* __restrict__ st, int m, int rows_per_split,
           int64_t pstride, T* __restrict__ Cpart) {
  __shared__ T Qs[32][33];
  __shared__ T As[32][MAXB + 1];
  __shared__ int cs[MAXB];
  const int tid = threadIdx.x;
  const int i = st->i, bss = st->bs_sampled;
  const int a0 = blockIdx.x * 32;
  const int rb = blockIdx.z * rows_per_split, re = min(m, rb + rows_per_split);
  if (tid < MAXB) cs[tid] = tid < bss ? cols[tid] : -1;
  const int al = tid >> 3, cl = tid & 7;
  const int nq = (bss + 7) >> 3;   // column groups that hold sampled columns (uniform: FP64 work only there)
  T acc[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) acc[q] = T(0);
  for (int r0 = rb; r0 < re; r0 += 32) {
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int idx = tid + 256 * q, kk = idx & 31, aa = idx >> 5;
      const int r = r0 + kk, a = a0 + aa;
      Qs[kk][aa] = (r < re && a < i) ? Q[r + (int64_t)a * ldq] : T(0);
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int idx = tid + 256 * q, kk = idx & 31, cc = idx >> 5;
      const int r = r0 + kk, c = cs[cc];
      As[kk][cc] = (r < re && c >= 0) ? A[r + (int64_t)c * lda] : T(0);
    }
    __syncthreads();
    // column groups as a compile-time count: predicated-off FP64 FMAs would still take issue slots
    auto fmas = [&](auto nqc) {
      constexpr int NQ = decltype(nqc)::value;
#pragma unroll 8
      for (int kk = 0; kk < 32; ++kk) {
        const T qa = Qs[kk][al];
#pragma unroll
        for (int q = 0; q < NQ; ++q) acc[q] = fma(qa, As[kk][cl + 8 * q], acc[q]);
      }
    };
    if (nq <= 1) fmas(std::integral_constant<int, 1>{});
    else if (nq <= 2) fmas(std::integral_constant<int, 2>{});
    else if (nq <= 4) fmas(std::integral_constant<int, 4>{});
    else fmas(std::integral_constant<int, 8>{});
  }
  const int a = a0 + al;
  if (a < i) {
    T* out = Cpart + (int64_t)blockIdx.z * pstride + (int64_t)a * MAXB;
#pragma unroll
    for (int q = 0; q < 8; ++q) out[cl + 8 * q] = acc[q];
  }
}

// Deterministic sum of split partials: out[x] = sum_z part[z*stride + x].
template <typename V>
__global__ void k_reduce_parts(const V* __restrict__ part, int nparts, int64_t stride, int64_t count,
                               V* __restrict__ out) {
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < count;
       x += (int64_t)gridDim.x * blockDim.x) {
    V s = V(0);
    for (int z = 0; z < nparts; ++z) s += part[(int64_t)z * stride + x];
    out[x] = s;
  }
}

// V(r, c) = A(r, cols[c]) - sum_a Q(r, a) C(a, c) for 64 rows; Gram partial of the tile.
template <typename T>
__global__ void __launch_bounds__(256)
k_cgs_update(const T* __restrict__ A, int64_t lda, const int* __restrict__ cols,
             const T* __restrict__ Q, int64_t ldq, const T* __restrict__ C,
             const State* __restrict__ st, int m, double* __restrict__ V, double* __restrict__ Gpart,
             int use_q) {
  // the operand tiles and the V tile are never live together
  constexpr size_t kOps = sizeof(T) * (64 * 33 + 32 * MAXB);
  constexpr size_t kV = sizeof(double) * 64 * (MAXB + 1);
  __shared__ __align__(16) unsigned char raw[kOps > kV ? kOps : kV];
  T(*Qs)[33] = reinterpret_cast<T(*)[33]>(raw);
  T(*Cs)[MAXB] = reinterpret_cast<T(*)[MAXB]>(raw + sizeof(T) * 64 * 33);
  double(*Vs)[MAXB + 1] = reinterpret_cast<double(*)[MAXB + 1]>(raw);
  __shared__ int cs[MAXB];
  const int tid = threadIdx.x;
  const int i = use_q ? st->i : 0, bss = st->bs_sampled;
  const int r0 = blockIdx.x * 64;
  if (tid < MAXB) cs[tid] = tid < bss ? cols[tid] : -1;
  const int ty = tid >> 4, tx = tid & 15;
  const int nv = (bss + 15) >> 4;   // column groups that hold sampled columns (uniform over the CTA)
  T acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = T(0);
  for (int a0 = 0; a0 < i; a0 += 32) {
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int idx = tid + 256 * q, rr = idx & 63, aa = idx >> 6;
      const int r = r0 + rr, a = a0 + aa;
      Qs[rr][aa] = (r < m && a < i) ? Q[r + (int64_t)a * ldq] : T(0);
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int idx = tid + 256 * q, cc = idx & 63, aa = idx >> 6;
      Cs[aa][cc] = (a0 + aa < i) ? C[(int64_t)(a0 + aa) * MAXB + cc] : T(0);
    }
    __syncthreads();
    // column groups as a compile-time count: predicated-off FP64 FMAs would still take issue slots
    auto fmas = [&](auto nvc) {
      constexpr int NV = decltype(nvc)::value;
#pragma unroll 4
      for (int aa = 0; aa < 32; ++aa) {
        T qv[4], cv[NV];
#pragma unroll
        for (int u = 0; u < 4; ++u) qv[u] = Qs[ty * 4 + u][aa];
#pragma unroll
        for (int v = 0; v < NV; ++v) cv[v] = Cs[aa][tx + 16 * v];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int v = 0; v < NV; ++v) acc[u][v] = fma(qv[u], cv[v], acc[u][v]);
      }
    };
    if (nv <= 1) fmas(std::integral_constant<int, 1>{});
    else if (nv <= 2) fmas(std::integral_constant<int, 2>{});
    else if (nv <= 3) fmas(std::integral_constant<int, 3>{});
    else fmas(std::integral_constant<int, 4>{});
  }
  __syncthreads();
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int rr = ty * 4 + u, r = r0 + rr;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int c = tx + 16 * v;
      double val = 0.0;
      if (r < m && c < bss) val = (double)A[r + (int64_t)cs[c] * lda] - (double)acc[u][v];
      Vs[rr][c] = val;
    }
  }
  __syncthreads();
  // store V (column major, ld = m) coalesced along rows
  for (int idx = tid; idx < 64 * MAXB; idx += 256) {
    const int rr = idx & 63, c = idx >> 6, r = r0 + rr;
    if (r < m && c < bss) V[r + (int64_t)c * m] = Vs[rr][c];
  }
  // Gram partial (bss x bss, stored MAXB x MAXB)
  double* G = Gpart + (int64_t)blockIdx.x * MAXB * MAXB;
  const int c1 = tid >> 2;
  for (int q = 0; q < 16; ++q) {
    const int c2 = (tid & 3) + 4 * q;
    double s = 0.0;
    if (c1 < bss && c2 < bss) {
#pragma unroll 8
      for (int rr = 0; rr < 64; ++rr) s = fma(Vs[rr][c1], Vs[rr][c2], s);
    }
    G[c1 * MAXB + c2] = s;
  }
}

// ===========================================================================
// a4 + a5: panel CPQR and robust filter.
// CPQR of the m x bs panel V is computed as pivoted Cholesky of its Gram
// matrix in shared memory: at step t the Schur complement's diagonal holds the
// squared norms of the panel columns orthogonalised against the t pivots, so
// the argmax is the CPQR pivot (LAPACK dgeqp3's greedy rule, swap semantics,
// first index among ties), and its trace is the reverse cumulative sum of the
// squared row norms of R that the robust filter tests
// (python/RBRP.ipynb cell 11 lines 69-73, 122-123):
//   keep t rows <=> trace_t / trace_0 >= tol_loc for every earlier step.
// Q is then V_p R^{-1}, made orthonormal by a second CholQR pass (CholQR2).
// ===========================================================================
struct PanelSmem {
  double S[MAXB][MAXB + 1];   // Gram / Schur complement
  double R[MAXB][MAXB + 1];   // Cholesky factor rows
  double W[64][MAXB + 1];     // row tile of the panel
  int ord[MAXB];
  int stop, piv;
  double total;
};

// Pivoted Cholesky with the robust-filter stop; all threads of the CTA call it.
__device__ int pivoted_chol_filter(PanelSmem& sm, int nb, int rows, double tol_loc) {
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  if (tid < MAXB) sm.ord[tid] = tid;
  if (wid == 0) {
    double d = 0.0;
    for (int s = lane; s < nb; s += 32) d += sm.S[s][s];
    d = warp_sum(d);
    if (lane == 0) sm.total = d;
  }
  __syncthreads();
  int kept = rows;
  for (int t = 0; t < rows; ++t) {
    if (wid == 0) {
      double rem = 0.0, best = -1.0;
      int bi = nb;
      for (int s = t + lane; s < nb; s += 32) {
        const double d = sm.S[s][s];
        rem += d;
        if (d > best) { best = d; bi = s; }
      }
      rem = warp_sum(rem);
      rem = __shfl_sync(0xffffffffu, rem, 0);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_down_sync(0xffffffffu, best, o);
        const int oi = __shfl_down_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (lane == 0) {
        const double total = sm.total;
        const bool stop = !(total > 0.0) || (rem / total < tol_loc) || !(best > 0.0);
        sm.stop = stop;
        sm.piv = bi;
      }
    }
    __syncthreads();
    if (sm.stop) { kept = t; break; }
    const int p = sm.piv;
    if (p != t) {
      for (int j = tid; j < nb; j += blockDim.x) {
        const double x = sm.S[t][j]; sm.S[t][j] = sm.S[p][j]; sm.S[p][j] = x;
      }
      __syncthreads();
      for (int j = tid; j < nb; j += blockDim.x) {
        const double x = sm.S[j][t]; sm.S[j][t] = sm.S[j][p]; sm.S[j][p] = x;
      }
      for (int j = tid; j < t; j += blockDim.x) {
        const double x = sm.R[j][t]; sm.R[j][t] = sm.R[j][p]; sm.R[j][p] = x;
      }
      if (tid == 0) { const int o = sm.ord[t]; sm.ord[t] = sm.ord[p]; sm.ord[p] = o; }
      __syncthreads();
    }
    const double rtt = sqrt(sm.S[t][t]);
    for (int s = t + tid; s < nb; s += blockDim.x) sm.R[t][s] = (s == t) ? rtt : sm.S[t][s] / rtt;
    __syncthreads();
    const int w = nb - t - 1;
    for (int idx = tid; idx < w * w; idx += blockDim.x) {
      const int s1 = t + 1 + idx / w, s2 = t + 1 + idx % w;
      sm.S[s1][s2] -= sm.R[t][s1] * sm.R[t][s2];
    }
    __syncthreads();
  }
  return kept;
}

// Single-warp form of pivoted_chol_filter (only __syncwarp between steps): lane
// l owns columns l and l + 32.  Returns the kept count to all 32 lanes.
__device__ int pivoted_chol_filter_warp(PanelSmem& sm, int nb, int rows, double tol_loc) {
  const int lane = threadIdx.x & 31;
  sm.ord[lane] = lane;
  sm.ord[lane + 32] = lane + 32;
  double d = 0.0;
  for (int s = lane; s < nb; s += 32) d += sm.S[s][s];
  const double total = __shfl_sync(0xffffffffu, warp_sum(d), 0);
  __syncwarp();
  for (int t = 0; t < rows; ++t) {
    double rem = 0.0, best = -1.0;
    int bi = nb;
    for (int s = t + lane; s < nb; s += 32) {
      const double v = sm.S[s][s];
      rem += v;
      if (v > best) { best = v; bi = s; }
    }
    rem = __shfl_sync(0xffffffffu, warp_sum(rem), 0);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_down_sync(0xffffffffu, best, o);
      const int oi = __shfl_down_sync(0xffffffffu, bi, o);
      if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    best = __shfl_sync(0xffffffffu, best, 0);
    const int p = __shfl_sync(0xffffffffu, bi, 0);
    if (!(total > 0.0) || (rem / total < tol_loc) || !(best > 0.0)) return t;
    if (p != t) {
      for (int j = lane; j < nb; j += 32) {
        const double x = sm.S[t][j]; sm.S[t][j] = sm.S[p][j]; sm.S[p][j] = x;
      }
      __syncwarp();
      for (int j = lane; j < nb; j += 32) {
        const double x = sm.S[j][t]; sm.S[j][t] = sm.S[j][p]; sm.S[j][p] = x;
      }
      for (int j = lane; j < t; j += 32) {
        const double x = sm.R[j][t]; sm.R[j][t] = sm.R[j][p]; sm.R[j][p] = x;
      }
      if (lane == 0) { const int o = sm.ord[t]; sm.ord[t] = sm.ord[p]; sm.ord[p] = o; }
      __syncwarp();
    }
    const double rtt = sqrt(sm.S[t][t]);
    for (int s = t + lane; s < nb; s += 32) sm.R[t][s] = (s == t) ? rtt : sm.S[t][s] / rtt;
    __syncwarp();
    for (int s2 = t + 1 + lane; s2 < nb; s2 += 32) {
      const double r2 = sm.R[t][s2];
      for (int s1 = t + 1; s1 < nb; ++s1) sm.S[s1][s2] = fma(-sm.R[t][s1], r2, sm.S[s1][s2]);
    }
    __syncwarp();
  }
  return rows;
}

// Single-warp plain Cholesky of S (n x n) into sm.R (upper).
__device__ void chol_upper_warp(PanelSmem& sm, int nb) {
  const int lane = threadIdx.x & 31;
  for (int t = 0; t < nb; ++t) {
    const double rtt = sqrt(fmax(sm.S[t][t], 0.0));
    for (int s = t + lane; s < nb; s += 32) sm.R[t][s] = (s == t) ? rtt : sm.S[t][s] / rtt;
    __syncwarp();
    for (int s2 = t + 1 + lane; s2 < nb; s2 += 32) {
      const double r2 = sm.R[t][s2];
      for (int s1 = t + 1; s1 <= s2; ++s1) sm.S[s1][s2] = fma(-sm.R[t][s1], r2, sm.S[s1][s2]);
    }
    __syncwarp();
  }
}

// Plain Cholesky of S (n x n) into sm.R (upper); all threads call it.
__device__ void chol_upper(PanelSmem& sm, int nb) {
  const int tid = threadIdx.x;
  for (int t = 0; t < nb; ++t) {
    const double rtt = sqrt(fmax(sm.S[t][t], 0.0));
    for (int s = t + tid; s < nb; s += blockDim.x) sm.R[t][s] = (s == t) ? rtt : sm.S[t][s] / rtt;
    __syncthreads();
    const int w = nb - t - 1;
    for (int idx = tid; idx < w * w; idx += blockDim.x) {
      const int s1 = t + 1 + idx / w, s2 = t + 1 + idx % w;
      sm.S[s1][s2] -= sm.R[t][s1] * sm.R[t][s2];
    }
    __syncthreads();
  }
}

// Forward substitution of the CTA's 64 rows: W(r, :) <- W(r, :) R^{-1} (R upper, kept x kept).
__device__ void rows_trsm(PanelSmem& sm, int kept) {
  const int r = threadIdx.x;
  if (r < 64) {
    for (int s = 0; s < kept; ++s) {
      double x = sm.W[r][s];
      for (int u = 0; u < s; ++u) x = fma(-sm.W[r][u], sm.R[u][s], x);
      sm.W[r][s] = x / sm.R[s][s];
    }
  }
  __syncthreads();
}

// Gram partial of the W tile (kept x kept): upper triangle computed, mirrored.
__device__ void tile_gram(const PanelSmem& sm, int kept, int rows_valid, double* G) {
  const int tid = threadIdx.x, c1 = tid >> 2;
  for (int q = 0; q < 16; ++q) {
    const int c2 = (tid & 3) + 4 * q;
    if (c2 < c1) continue;
    double s = 0.0;
    if (c1 < kept && c2 < kept)
      for (int rr = 0; rr < rows_valid; ++rr) s = fma(sm.W[rr][c1], sm.W[rr][c2], s);
    G[c1 * MAXB + c2] = s;
    G[c2 * MAXB + c1] = s;
  }
}

// k_pchol (one CTA): pivoted Cholesky of the panel Gram matrix with the robust
// filter; publishes the pivots (ord), the kept count, R11 and performs the block
// swap of perm and diags (matlab/RBRP.m:81-99: K1 = block positions not kept,
// ascending; K2 = kept positions outside the block, in pivot order).
__global__ void __launch_bounds__(256)
k_pchol(const double* __restrict__ G, int m, State* st, double tol_loc, const int* __restrict__ js,
        int* __restrict__ perm, double* __restrict__ diags, double* __restrict__ R11g, int* __restrict__ ordg,
        int* __restrict__ Jg, int* __restrict__ K1g, int* __restrict__ K2g) {
  extern __shared__ __align__(16) unsigned char dyn_smem[];
  PanelSmem& sm = *reinterpret_cast<PanelSmem*>(dyn_smem);
  const int tid = threadIdx.x;
  const int nb = st->bs_sampled, i = st->i;
  for (int idx = tid; idx < nb * nb; idx += blockDim.x) sm.S[idx / nb][idx % nb] = G[(idx / nb) * MAXB + idx % nb];
  __syncthreads();
  if (tid < 32) {
    const int kw = pivoted_chol_filter_warp(sm, nb, min(nb, m), tol_loc);
    if (tid == 0) sm.stop = kw;
  }
  __syncthreads();
  const int kept = sm.stop;
  for (int idx = tid; idx < MAXB * MAXB; idx += blockDim.x) {
    const int a = idx / MAXB, c = idx % MAXB;
    R11g[idx] = (a < kept && c < kept && c >= a) ? sm.R[a][c] : 0.0;
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

// Load an upper-triangular kept x kept factor (MAXB stride) into sm.R.
__device__ __forceinline__ void load_factor(PanelSmem& sm, const double* __restrict__ Rg, int kept) {
  for (int idx = threadIdx.x; idx < kept * kept; idx += blockDim.x) sm.R[idx / kept][idx % kept] = Rg[(idx / kept) * MAXB + idx % kept];
}

// Q1 = V(:, ord[:kept]) R11^{-1} for 64 rows per CTA, and the Gram partial of Q1.
__global__ void __launch_bounds__(256)
k_panel1(const double* __restrict__ V, int m, const State* __restrict__ st, const double* __restrict__ R11g,
         const int* __restrict__ ordg, double* __restrict__ Q1, double* __restrict__ G2part) {
  extern __shared__ __align__(16) unsigned char dyn_smem[];
  PanelSmem& sm = *reinterpret_cast<PanelSmem*>(dyn_smem);
  const int tid = threadIdx.x;
  const int kept = st->bs;
  if (kept == 0) return;
  load_factor(sm, R11g, kept);
  const int r0 = blockIdx.x * 64;
  const int rows_valid = max(0, min(64, m - r0));
  for (int idx = tid; idx < 64 * kept; idx += blockDim.x) {
    const int rr = idx & 63, s = idx >> 6, r = r0 + rr;
    sm.W[rr][s] = r < m ? V[r + (int64_t)ordg[s] * m] : 0.0;
  }
  __syncthreads();
  rows_trsm(sm, kept);
  for (int idx = tid; idx < 64 * kept; idx += blockDim.x) {
    const int rr = idx & 63, s = idx >> 6, r = r0 + rr;
    if (r < m) Q1[r + (int64_t)s * m] = sm.W[rr][s];
  }
  tile_gram(sm, kept, rows_valid, G2part + (int64_t)blockIdx.x * MAXB * MAXB);
}

// k_chol2 (one CTA): R2 = chol(Q1^T Q1) and the panel R = R2 R11 into R(I2, I2)
// (matlab/RBRP.m:78); R2 is published for the second row solve.
__global__ void __launch_bounds__(256)
k_chol2(const double* __restrict__ G2, const State* __restrict__ st, const double* __restrict__ R11g,
        double* __restrict__ R2g, double* __restrict__ R, int64_t ldr) {
  extern __shared__ __align__(16) unsigned char dyn_smem[];
  PanelSmem& sm = *reinterpret_cast<PanelSmem*>(dyn_smem);
  const int tid = threadIdx.x;
  const int kept = st->bs, i = st->i;
  if (kept == 0) return;
  for (int idx = tid; idx < kept * kept; idx += blockDim.x) sm.S[idx / kept][idx % kept] = G2[(idx / kept) * MAXB + idx % kept];
  __syncthreads();
  if (tid < 32) chol_upper_warp(sm, kept);
  __syncthreads();
  for (int idx = tid; idx < MAXB * MAXB; idx += blockDim.x) {
    const int a = idx / MAXB, c = idx % MAXB;
    R2g[idx] = (a < kept && c < kept && c >= a) ? sm.R[a][c] : 0.0;
  }
  for (int idx = tid; idx < kept * kept; idx += blockDim.x) {
    const int a = idx / kept, c = idx % kept;
    double v = 0.0;
    if (c >= a)
      for (int u = a; u <= c; ++u) v = fma(sm.R[a][u], R11g[u * MAXB + c], v);
    R[(int64_t)(i + a) * ldr + (i + c)] = v;
  }
}

// Column swap of the rows above the block: R(:i, K2) = R(:i, K1); R(:i, I2) = R(:i, J).
__global__ void k_swap_R(double* __restrict__ R, int64_t ldr, const State* __restrict__ st,
                         const int* __restrict__ Jg, const int* __restrict__ K1g, const int* __restrict__ K2g) {
  const int i = st->i, kept = st->bs, nK = st->nK;
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= i || kept == 0) return;
  double* Rr = R + (int64_t)row * ldr;
  double tmp[MAXB];
  for (int s = 0; s < kept; ++s) tmp[s] = Rr[Jg[s]];
  for (int t = 0; t < nK; ++t) Rr[K2g[t]] = Rr[K1g[t]];
  for (int s = 0; s < kept; ++s) Rr[i + s] = tmp[s];
}

// Second CholQR pass: Q_blk = Q1 R2^{-1}, 64 rows per CTA.
template <typename T>
__global__ void __launch_bounds__(256)
k_panel2(const double* __restrict__ Q1, int m, const State* __restrict__ st, const double* __restrict__ R2g,
         T* __restrict__ Q, int64_t ldq, int q_at_i) {
  extern __shared__ __align__(16) unsigned char dyn_smem[];
  PanelSmem& sm = *reinterpret_cast<PanelSmem*>(dyn_smem);
  const int tid = threadIdx.x;
  const int kept = st->bs, i = st->i;
  if (kept == 0) return;
  load_factor(sm, R2g, kept);
  const int r0 = blockIdx.x * 64;
  for (int idx = tid; idx < 64 * kept; idx += blockDim.x) {
    const int rr = idx & 63, s = idx >> 6, r = r0 + rr;
    sm.W[rr][s] = r < m ? Q1[r + (int64_t)s * m] : 0.0;
  }
  __syncthreads();
  rows_trsm(sm, kept);
  for (int idx = tid; idx < 64 * kept; idx += blockDim.x) {
    const int rr = idx & 63, s = idx >> 6, r = r0 + rr;
    if (r < m) Q[r + (int64_t)((q_at_i ? i : 0) + s) * ldq] = (T)sm.W[rr][s];
  }
}

// ===========================================================================
// a7 + a8: projection of the remaining columns on the new block and the
// residual-norm downdate (python/RBRP.ipynb cell 11 lines 132, 154-158;
// matlab/RBRP.m:103-104,112; the reference applies Householder reflectors to
// the whole trailing matrix instead, gpu/rbrp.cu:297-330, 453-466).
// CTA tile: KB basis vectors (KB >= kept, chosen on the host from b) x PC =
// 4096 / KB positions, K loop over m in chunks of KC rows; every thread holds a
// (KB / TY) x 4 accumulator block.  Each accumulator sums over the rows in
// ascending order, so W is the same for every KB: KB only removes the work on
// basis rows that do not exist (the FP64 pipe is the bound of this kernel).
// ===========================================================================
template <int KB>
struct ProjTile {
  static constexpr int MU = KB < 4 ? KB : 4;     // basis rows per thread
  static constexpr int TY = KB / MU;             // thread rows
  static constexpr int TX = 256 / TY;            // thread columns
  static constexpr int PC = TX * 4;              // positions per CTA
  static constexpr int KC = 4096 / PC < 32 ? 4096 / PC : 32;   // rows per K chunk
};

template <typename T, int KB>
__global__ void __launch_bounds__(256)
k_project(const T* __restrict__ Q, int64_t ldq, const T* __restrict__ A, int64_t lda,
          const int* __restrict__ perm, const State* __restrict__ st, int m, int n,
          double* __restrict__ R, int64_t ldr, double* __restrict__ diags,
          double* __restrict__ part_res, int* __restrict__ part_nnz) {
  using P = ProjTile<KB>;
  constexpr int PC = P::PC, KC = P::KC, TX = P::TX, TY = P::TY, MU = P::MU;
  constexpr size_t kOps = sizeof(T) * (KC * KB + KC * (PC + 1));
  constexpr size_t kW = sizeof(double) * KB * (PC + 1);
  __shared__ __align__(16) unsigned char raw[kOps > kW ? kOps : kW];
  T(*Qs)[KB] = reinterpret_cast<T(*)[KB]>(raw);
  T(*As)[PC + 1] = reinterpret_cast<T(*)[PC + 1]>(raw + sizeof(T) * KC * KB);
  double(*Ws)[PC + 1] = reinterpret_cast<double(*)[PC + 1]>(raw);
  __shared__ int cs[PC];
  __shared__ double snew[PC];
  __shared__ double red_s[PC / 64];
  __shared__ int red_c[PC / 64];
  const int tid = threadIdx.x;
  // kept <= b <= KB by construction (the host picks KB from b); the clamp only keeps smem in bounds
  const int i = st->i, kept = min(st->bs, KB);
  const int pbase = i + st->bs + blockIdx.x * PC;
  if (kept == 0 || pbase >= n) {
    if (tid == 0) { part_res[blockIdx.x] = 0.0; part_nnz[blockIdx.x] = 0; }
    return;
  }
  for (int t = tid; t < PC; t += 256) cs[t] = (pbase + t < n) ? perm[pbase + t] : -1;
  const int ty = tid / TX, tx = tid % TX;
  const int me = (kept + TY - 1) / TY;   // <= MU
  T acc[MU][4];
#pragma unroll
  for (int u = 0; u < MU; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = T(0);
  const T* Qb = Q + (int64_t)i * ldq;
  for (int r0 = 0; r0 < m; r0 += KC) {
    __syncthreads();
    for (int idx = tid; idx < KC * KB; idx += 256) {
      const int kk = idx % KC, aa = idx / KC;
      const int r = r0 + kk;
      Qs[kk][aa] = (r < m && aa < kept) ? Qb[r + (int64_t)aa * ldq] : T(0);
    }
#pragma unroll
    for (int q = 0; q < (KC * PC) / 256; ++q) {
      const int idx = tid + 256 * q, kk = idx % KC, cc = idx / KC;
      const int r = r0 + kk, c = cs[cc];
      As[kk][cc] = (r < m && c >= 0) ? A[r + (int64_t)c * lda] : T(0);
    }
    __syncthreads();
    // basis rows per thread that exist (kept <= TY * me) as a compile-time count:
    // predicated-off FP64 FMAs would still take issue slots on the FP64 pipe
    auto fmas = [&](auto mec) {
      constexpr int ME = decltype(mec)::value;
#pragma unroll 4
      for (int kk = 0; kk < KC; ++kk) {
        T qv[ME], av[4];
#pragma unroll
        for (int u = 0; u < ME; ++u) qv[u] = Qs[kk][ty + TY * u];
#pragma unroll
        for (int v = 0; v < 4; ++v) av[v] = As[kk][tx + TX * v];
#pragma unroll
        for (int u = 0; u < ME; ++u)
#pragma unroll
          for (int v = 0; v < 4; ++v) acc[u][v] = fma(qv[u], av[v], acc[u][v]);
      }
    };
    if (MU == 1 || me <= 1) fmas(std::integral_constant<int, 1>{});
    else if (me <= 2) fmas(std::integral_constant<int, (MU < 2 ? MU : 2)>{});
    else if (me <= 3) fmas(std::integral_constant<int, (MU < 3 ? MU : 3)>{});
    else fmas(std::integral_constant<int, MU>{});
  }
  __syncthreads();
#pragma unroll
  for (int u = 0; u < MU; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) Ws[ty + TY * u][tx + TX * v] = (double)acc[u][v];
  __syncthreads();
  for (int idx = tid; idx < kept * PC; idx += 256) {
    const int a = idx / PC, c = idx % PC;
    if (pbase + c < n) R[(int64_t)(i + a) * ldr + pbase + c] = Ws[a][c];
  }
  for (int t = tid; t < PC; t += 256) {
    const int p = pbase + t;
    double d = 0.0;
    if (p < n) {
      double s = 0.0;
      for (int a = 0; a < kept; ++a) s = fma(Ws[a][t], Ws[a][t], s);
      d = diags[p] - s;
      d = d > 0.0 ? d : (d == d ? 0.0 : d);
      diags[p] = d;
    }
    snew[t] = d;
  }
  __syncthreads();
  // CTA partial of the residual and of the nonzero count, positions in ascending order
  // in chunks of 64 (the sum order of the 64-position tile this kernel generalises)
  if (tid < PC / 64) {
    double sacc = 0.0;
    int c = 0;
    for (int t = tid * 64; t < tid * 64 + 64; ++t) { sacc += snew[t]; c += snew[t] > 0.0; }
    red_s[tid] = sacc;
    red_c[tid] = c;
  }
  __syncthreads();
  if (tid == 0) {
    double sacc = 0.0;
    int c = 0;
    for (int t = 0; t < PC / 64; ++t) { sacc += red_s[t]; c += red_c[t]; }
    part_res[blockIdx.x] = sacc;
    part_nnz[blockIdx.x] = c;
  }
}

// Skinny form of the same projection for b <= 8 (a GEMV shape: greedy b = 1 is
// column-pivoted QR).  Each warp streams CW = 4 whole columns (coalesced over
// rows) against the basis staged in shared memory, MC rows at a time; lanes keep
// strided partial sums that a butterfly combines.  32 positions per CTA.
constexpr int SKINNY_COLS = 32;

template <typename T, int KB>
__global__ void __launch_bounds__(256)
k_project_skinny(const T* __restrict__ Q, int64_t ldq, const T* __restrict__ A, int64_t lda,
                 const int* __restrict__ perm, const State* __restrict__ st, int m, int n,
                 double* __restrict__ R, int64_t ldr, double* __restrict__ diags,
                 double* __restrict__ part_res, int* __restrict__ part_nnz) {
  constexpr int CW = 4, MC = 256, NW = 8;
  static_assert(NW * CW == SKINNY_COLS, "positions per CTA");
  __shared__ T Qs[KB][MC];   // basis chunk, row index fastest: lanes read consecutive rows
  __shared__ double red_s[NW];
  __shared__ int red_c[NW];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // kept <= b <= KB by construction (the host picks KB from b); the clamp only keeps smem in bounds
  const int i = st->i, kept = min(st->bs, KB);
  const int pbase = i + st->bs + blockIdx.x * SKINNY_COLS;
  if (kept == 0 || pbase >= n) {
    if (tid == 0) { part_res[blockIdx.x] = 0.0; part_nnz[blockIdx.x] = 0; }
    return;
  }
  int col[CW];
#pragma unroll
  for (int c = 0; c < CW; ++c) {
    const int p = pbase + warp * CW + c;
    col[c] = p < n ? perm[p] : -1;
  }
  T acc[CW][KB];
#pragma unroll
  for (int c = 0; c < CW; ++c)
#pragma unroll
    for (int a = 0; a < KB; ++a) acc[c][a] = T(0);
  const T* Qb = Q + (int64_t)i * ldq;
  for (int r0 = 0; r0 < m; r0 += MC) {
    __syncthreads();
    for (int idx = tid; idx < KB * MC; idx += 256) {
      const int a = idx / MC, rr = idx % MC, r = r0 + rr;
      Qs[a][rr] = (r < m && a < kept) ? Qb[r + (int64_t)a * ldq] : T(0);
    }
    __syncthreads();
    const int rend = min(MC, m - r0);
#pragma unroll 2
    for (int rr = lane; rr < rend; rr += 32) {
      T av[CW], qv[KB];
#pragma unroll
      for (int c = 0; c < CW; ++c) av[c] = col[c] >= 0 ? A[(r0 + rr) + (int64_t)col[c] * lda] : T(0);
#pragma unroll
      for (int a = 0; a < KB; ++a) qv[a] = Qs[a][rr];
#pragma unroll
      for (int c = 0; c < CW; ++c)
#pragma unroll
        for (int a = 0; a < KB; ++a) acc[c][a] = fma(av[c], qv[a], acc[c][a]);
    }
  }
#pragma unroll
  for (int c = 0; c < CW; ++c)
#pragma unroll
    for (int a = 0; a < KB; ++a)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc[c][a] += __shfl_xor_sync(0xffffffffu, acc[c][a], o);
  double dsum = 0.0;
  int dcnt = 0;
#pragma unroll
  for (int c = 0; c < CW; ++c) {
    const int p = pbase + warp * CW + c;
    if (lane == c && p < n) {
      double s = 0.0;
#pragma unroll
      for (int a = 0; a < KB; ++a) {
        if (a < kept) {
          const double w = (double)acc[c][a];
          R[(int64_t)(i + a) * ldr + p] = w;
          s = fma(w, w, s);
        }
      }
      double d = diags[p] - s;
      d = d > 0.0 ? d : (d == d ? 0.0 : d);
      diags[p] = d;
      dsum = d;
      dcnt = d > 0.0;
    }
  }
#pragma unroll
  for (int o = 1; o < CW; o <<= 1) {
    dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
    dcnt += __shfl_xor_sync(0xffffffffu, dcnt, o);
  }
  if (lane == 0) {
    red_s[warp] = dsum;
    red_c[warp] = dcnt;
  }
  __syncthreads();
  if (tid == 0) {
    double sacc = 0.0;
    int c = 0;
    for (int w = 0; w < NW; ++w) { sacc += red_s[w]; c += red_c[w]; }
    part_res[blockIdx.x] = sacc;
    part_nnz[blockIdx.x] = c;
  }
}

// ===========================================================================
// Residual form (FP32 storage).  The residual A_res = (I - Q Q^T) A is kept
// explicitly, position ordered, and updated after every block - the
// trailing-matrix update of gpu/rbrp.cu:297-330,448 (Householder there,
// Q_blk W here) - so every residual norm is recomputed exactly from the
// residual instead of downdated: a downdate ||a||^2 - ||Q^T a||^2 in FP32
// arithmetic cannot resolve residuals below ~1e-7 of ||a||^2.
// ===========================================================================

// Block swap of the residual's columns: A_res(:, K2) = A_res(:, K1).  Kept
// columns need no copy (their residual was gathered into the panel already).
__global__ void k_swap_cols(float* __restrict__ Ares, int64_t ld, const State* __restrict__ st, int m,
                            const int* __restrict__ K1g, const int* __restrict__ K2g) {
  const int t = blockIdx.y;
  if (t >= st->nK) return;
  const float* src = Ares + (int64_t)K1g[t] * ld;
  float* dst = Ares + (int64_t)K2g[t] * ld;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x) dst[r] = src[r];
}

__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float x) {
  const float t = hi + x;
  const float bb = t - hi;
  lo += (hi - (t - bb)) + (x - bb);
  hi = t;
}

// P1: W = Q_blk^T A_res(:, p) for the remaining positions p, into R(I2, p).
// CTA tile 64 basis vectors x 64 positions, 32-row K stages; each stage's FP32
// partial sums are folded into double-float accumulators (TwoSum), so W is
// accurate to ~1e-8 relative over m = 16384 rows.
__global__ void __launch_bounds__(128)
k_proj_w(const float* __restrict__ Qb, int64_t ldq, const float* __restrict__ Ares, int64_t ld,
         const State* __restrict__ st, int m, int n, double* __restrict__ R, int64_t ldr) {
  __shared__ __align__(16) float Qs[32][MAXB];
  __shared__ __align__(16) float As[32][MAXB + 4];
  const int tid = threadIdx.x;
  const int i = st->i, kept = st->bs;
  const int p0 = i + kept + blockIdx.x * 64;
  if (kept == 0 || p0 >= n) return;
  const int ncol = min(64, n - p0);
  const int ta = tid >> 4, tc = tid & 15;  // rows a = ta*8 + u, columns c = tc*4 + v
  float hi[8][4], lo[8][4];
#pragma unroll
  for (int u = 0; u < 8; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) hi[u][v] = lo[u][v] = 0.f;
  for (int r0 = 0; r0 < m; r0 += 32) {
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int idx = tid + 128 * q, kk = idx & 31, aa = idx >> 5, r = r0 + kk;
      Qs[kk][aa] = (r < m && aa < kept) ? Qb[r + (int64_t)aa * ldq] : 0.f;
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int idx = tid + 128 * q, kk = idx & 31, cc = idx >> 5, r = r0 + kk;
      As[kk][cc] = (r < m && cc < ncol) ? Ares[r + (int64_t)(p0 + cc) * ld] : 0.f;
    }
    __syncthreads();
    float c[8][4];
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) c[u][v] = 0.f;
#pragma unroll 8
    for (int kk = 0; kk < 32; ++kk) {
      const float4 q0 = *reinterpret_cast<const float4*>(&Qs[kk][ta * 8]);
      const float4 q1 = *reinterpret_cast<const float4*>(&Qs[kk][ta * 8 + 4]);
      const float4 a4 = *reinterpret_cast<const float4*>(&As[kk][tc * 4]);
      const float qv[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
      const float av[4] = {a4.x, a4.y, a4.z, a4.w};
#pragma unroll
      for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) c[u][v] = fmaf(qv[u], av[v], c[u][v]);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) two_sum_acc(hi[u][v], lo[u][v], c[u][v]);
  }
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    const int a = ta * 8 + u;
    if (a < kept) {
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int cc = tc * 4 + v;
        if (cc < ncol) R[(int64_t)(i + a) * ldr + p0 + cc] = (double)hi[u][v] + (double)lo[u][v];
      }
    }
  }
}

// P2 on the CUDA cores (the CUDA-core variant; the default is k_resid_update_tc):
// A_res(:, p) -= Q_blk W(:, p) and the partial squared norms of the updated
// columns (double-float sums), for 64 positions x one row range per CTA.  Warp w
// owns 8 columns, lane l four consecutive rows of every 128-row stage (16-byte
// loads and stores, coalesced along the column).  Row ranges of the same columns
// are summed by k_norm_reduce.  W comes from R (written by k_proj_w).
constexpr int P2_COLS = 64;
constexpr int P2_ROWS = 128;
constexpr int P2_MAX_SPLIT = 8;
constexpr int P2_THREADS = 256;
constexpr size_t P2_SMEM = sizeof(float) * (size_t)MAXB * (P2_COLS + 2 * P2_ROWS);   // W + two basis stages

// 16-byte asynchronous copy global -> shared; bytes beyond src_bytes are zero-filled
__device__ __forceinline__ void upd_cp16(float* smem, const float* gmem, int src_bytes) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(gmem), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void upd_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void upd_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

__global__ void __launch_bounds__(P2_THREADS, 2)
k_resid_update(const float* __restrict__ Qb, int64_t ldq, float* __restrict__ Ares, int64_t ld,
               const State* __restrict__ st, int m, int n, int rows_per_split, const double* __restrict__ R,
               int64_t ldr, double* __restrict__ part_norm) {
  extern __shared__ __align__(16) float p2_smem[];
  float* Ws = p2_smem;                       // Ws[a * P2_COLS + c]
  float* Qbuf = p2_smem + MAXB * P2_COLS;    // two stages of Qs[a * P2_ROWS + rr]
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int i = st->i, kept = st->bs;
  const int p0 = i + kept + blockIdx.x * P2_COLS;
  if (kept == 0 || p0 >= n) return;
  const int ncol = min(P2_COLS, n - p0);
  const int rb = blockIdx.y * rows_per_split, re = min(m, rb + rows_per_split);
  for (int idx = tid; idx < kept * P2_COLS; idx += P2_THREADS) {
    const int a = idx / P2_COLS, c = idx % P2_COLS;
    Ws[idx] = c < ncol ? (float)R[(int64_t)(i + a) * ldr + p0 + c] : 0.f;
  }
  DF nrm[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) nrm[c].hi = nrm[c].lo = 0.f;
  // basis stage of rows [r0, r0 + P2_ROWS) into dst by cp.async; rows at or past re read as zero
  auto load_q = [&](int r0, float* dst) {
    for (int idx = tid; idx < kept * (P2_ROWS / 4); idx += P2_THREADS) {
      const int a = idx / (P2_ROWS / 4), j = idx % (P2_ROWS / 4), rq = r0 + 4 * j;
      const int bytes = 4 * max(0, min(4, re - rq));
      upd_cp16(dst + a * P2_ROWS + 4 * j, bytes > 0 ? Qb + rq + (int64_t)a * ldq : Qb, bytes);
    }
    upd_commit();
  };
  load_q(rb, Qbuf);
  int stage = 0;
  for (int r0 = rb; r0 < re; r0 += P2_ROWS, ++stage) {
    const float* Qs = Qbuf + (stage & 1) * MAXB * P2_ROWS;
    // this thread's residual values, fetched before the products so the loads
    // are in flight during the stage's FMA work
    const int r = r0 + 4 * lane;
    const bool vec_ok = r + 3 < re;
    float4 xa[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const int cc = w * 8 + c;
      xa[c] = (vec_ok && cc < ncol) ? *reinterpret_cast<const float4*>(Ares + (int64_t)(p0 + cc) * ld + r)
                                    : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    // the next stage's basis goes into the other buffer, whose last readers passed the
    // barrier that ended the previous stage
    if (r0 + P2_ROWS < re) {
      load_q(r0 + P2_ROWS, Qbuf + ((stage + 1) & 1) * MAXB * P2_ROWS);
      upd_wait<1>();
    } else {
      upd_wait<0>();
    }
    __syncthreads();
    float acc[4][8];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int c = 0; c < 8; ++c) acc[u][c] = 0.f;
#pragma unroll 4
    for (int a = 0; a < kept; ++a) {
      const float4 q4 = reinterpret_cast<const float4*>(Qs + a * P2_ROWS)[lane];
      const float4* w4 = reinterpret_cast<const float4*>(Ws + a * P2_COLS + w * 8);
      const float4 x0 = w4[0], x1 = w4[1];
      const float qv[4] = {q4.x, q4.y, q4.z, q4.w};
      const float wv[8] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int c = 0; c < 8; ++c) acc[u][c] = fmaf(qv[u], wv[c], acc[u][c]);
    }
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const int cc = w * 8 + c;
      if (cc < ncol) {
        float* col = Ares + (int64_t)(p0 + cc) * ld;
        if (vec_ok) {
          float4 x = xa[c];
          x.x -= acc[0][c];
          x.y -= acc[1][c];
          x.z -= acc[2][c];
          x.w -= acc[3][c];
          *reinterpret_cast<float4*>(col + r) = x;
          // FP32 sum of the 4 squares (positive terms, relative error < 3e-7), folded
          // into the double-float norm by TwoSum
          const float q4 = fmaf(x.w, x.w, fmaf(x.z, x.z, fmaf(x.y, x.y, x.x * x.x)));
          const float t = nrm[c].hi + q4;
          const float bb = t - nrm[c].hi;
          nrm[c].lo += (nrm[c].hi - (t - bb)) + (q4 - bb);
          nrm[c].hi = t;
        } else {
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            if (r + u < re) {
              const float x = col[r + u] - acc[u][c];
              col[r + u] = x;
              df_add_sq(nrm[c], x);
            }
          }
        }
      }
    }
    __syncthreads();   // every warp is done with this stage's basis before it is refilled
  }
  // warp sums of the double-float norms on the FP32 pipe; lane 0 converts once per column
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    dfl v = df_two_sum(nrm[c].hi, nrm[c].lo);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      v = df_add(v, {__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)});
    const int cc = w * 8 + c;
    if (lane == 0 && cc < ncol) part_norm[(int64_t)blockIdx.y * n + p0 + cc] = (double)v.hi + (double)v.lo;
  }
}

// diags(p) = sum over row ranges of the partial norms; per-CTA residual sums and
// positive counts for k_finish.
__global__ void __launch_bounds__(256)
k_norm_reduce(const double* __restrict__ part_norm, int nsplit, int n, const State* __restrict__ st,
              double* __restrict__ diags, double* __restrict__ part_res, int* __restrict__ part_nnz) {
  __shared__ double shd[32];
  __shared__ int shi[32];
  const int p = st->i + st->bs + blockIdx.x * 256 + threadIdx.x;
  double d = 0.0;
  if (st->bs > 0 && p < n) {
    for (int z = 0; z < nsplit; ++z) d += part_norm[(int64_t)z * n + p];
    diags[p] = d;
  }
  const double s = block_sum(d, shd);
  const int c = block_sum((int)(d > 0.0), shi);
  if (threadIdx.x == 0) {
    part_res[blockIdx.x] = s;
    part_nnz[blockIdx.x] = c;
  }
}

// ===========================================================================
// a8 + a9 + a12: residual, stopping rule and per-block trace.  One CTA.
// ===========================================================================
__global__ void __launch_bounds__(1024)
k_finish(State* st, const double* __restrict__ part_res, const int* __restrict__ part_nnz, int nparts,
         double* __restrict__ diags, const int* __restrict__ js, int n, int kmax, double tol,
         int* __restrict__ trace_rank, double* __restrict__ trace_err, int* __restrict__ trace_samp) {
  __shared__ double shd[32];
  __shared__ int shi[32];
  __shared__ int s_done, s_zero, s_i, s_bs, s_bss;
  const int tid = threadIdx.x;
  if (tid == 0) {
    s_done = st->done;
    s_zero = st->zero_panel;
    s_i = st->i;
    s_bs = st->bs;
    s_bss = st->bs_sampled;
  }
  __syncthreads();
  if (s_done) return;
  if (tid == 0) st->attempts += 1;
  if (s_zero) {
    // numerically zero panel: drop the sampled columns' weights and go on
    if (tid < s_bss) diags[js[tid]] = 0.0;
    __syncthreads();
    double s = 0.0;
    int c = 0;
    for (int p = s_i + tid; p < n; p += blockDim.x) {
      const double d = diags[p];
      s += d;
      c += d > 0.0;
    }
    s = block_sum(s, shd);
    c = block_sum(c, shi);
    if (tid == 0) {
      st->residual = s;
      st->nnz_rem = c;
      st->zero_panel = 0;
      if (c == 0 || s_bss == 0) st->done = 1;  // nothing left that can be sampled
    }
    return;
  }
  // residual and nonzero count: strided partial sums, then a fixed-order block tree
  double s = 0.0;
  int c = 0;
  for (int z = tid; z < nparts; z += blockDim.x) { s += part_res[z]; c += part_nnz[z]; }
  s = block_sum(s, shd);
  c = block_sum(c, shi);
  if (tid == 0) {
    const int i = s_i + s_bs;
    const int nb = st->nblocks;
    st->i = i;
    st->residual = s;
    st->nnz_rem = c;
    trace_rank[nb] = i;
    trace_err[nb] = st->res0 > 0.0 ? s / st->res0 : 0.0;
    trace_samp[nb] = s_bss;
    st->nblocks = nb + 1;
    if ((tol > 0.0 && s < st->res0 * tol) || c == 0 || i >= kmax || !(s == s)) st->done = 1;
    if (!(s == s) && st->status == 0) st->status = ST_ERR_NUMERIC;  // an earlier status (a timeout) stays
  }
}

}  // namespace
}  // namespace rbrp
