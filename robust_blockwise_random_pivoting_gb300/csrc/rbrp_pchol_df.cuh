// rbrp_pchol_df.cuh - double-float pivoted Cholesky with the robust filter
// and the block swap, for panels of up to BB columns (BB = 16, 32 or 64).
// Used by the one-matrix panel kernel (BB = 64) and the batched kernel.
#pragma once
#include "rbrp_common.cuh"
#include "rbrp_df.cuh"

namespace rbrp {
namespace {

template <int BB>
struct PcholDfSmemT {
  dfl S[BB][BB + 1];  // Schur complement, indexed by panel column
  dfl R[BB][BB + 1];  // R[t][j]: row t of the factor, by panel column j
  int ord[BB];        // slot -> panel column
  int alive[BB];
  int J[BB], K1[BB], K2[BB], inblk[BB], Tperm[BB];
  int stop, piv, nK;
  dfl inv;
};

// Block swap of perm and diags (matlab/RBRP.m:81-99), in parallel: K1 = block
// positions not kept (ascending), K2 = kept positions outside the block (pivot
// order), compacted with warp ballots.  All threads call it after `kept` is known.
template <int BB>
__device__ void block_swap_parallel(PcholDfSmemT<BB>& sm, int i, int kept, const int* __restrict__ js,
                                    int* __restrict__ perm, double* __restrict__ diags, int* __restrict__ Jg,
                                    int* __restrict__ K1g, int* __restrict__ K2g, State* st) {
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  if (tid < BB) sm.inblk[tid] = 0;
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

// Pivoted Cholesky of a panel Gram matrix with the robust filter, in
// double-float, by 256 threads.  On entry sm.S holds the nb x nb Gram matrix
// (zero elsewhere), sm.ord the identity and sm.alive[j] = (j < nb).  Pivots
// follow LAPACK dgeqp3 (the first slot of maximal Schur diagonal); the filter
// (python/RBRP.ipynb cell 11 lines 69-73) stops once the remaining trace falls
// below tol_loc of the total.  Swaps are virtual (ord maps slot -> panel
// column), so sm.R[t][j] holds row t of the factor by panel column j.
// Returns the number of kept pivots.
template <int BB>
__device__ int pchol_filter_df(PcholDfSmemT<BB>& sm, int nb, int rows, double tol_loc) {
  constexpr int U = BB / 16;  // U x U Schur entries per thread: rows ty*U+u, columns tx*U+v
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int ty = tid >> 4, tx = tid & 15;
  // trace(G) and the stop threshold tol_loc * trace as a double-float, used by warp 0:
  // the per-step test rem < thr stays on the FP32 pipe (rem / trace < tol_loc, no FP64 divide)
  bool have_total = false;
  dfl thr = {0.f, 0.f};
  if (wid == 0) {
    dfl t = {0.f, 0.f};
    for (int s2 = 0; s2 < nb; ++s2) t = df_add(t, sm.S[s2][s2]);
    const double total = df_dbl(t);
    have_total = total > 0.0;
    thr = df_of(tol_loc * total);
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
        const bool stop = !have_total || df_gt(thr, rem) || !(best.hi > 0.f);
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
    dfl ru[U], rv[U];
    bool au[U], av[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int j = ty * U + u;
      au[u] = j < nb && sm.alive[j];
      ru[u] = sm.R[t][j];
      const int c = tx * U + u;
      av[u] = c < nb && sm.alive[c];
      rv[u] = sm.R[t][c];
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int v = 0; v < U; ++v)
        if (au[u] && av[v]) sm.S[ty * U + u][tx * U + v] = df_fms(sm.S[ty * U + u][tx * U + v], ru[u], rv[v]);
    __syncthreads();
  }
  return kept;
}

}  // namespace
}  // namespace rbrp
