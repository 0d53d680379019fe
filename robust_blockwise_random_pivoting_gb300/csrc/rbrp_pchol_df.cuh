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
  int slot[BB];       // panel column -> slot (pchol_filter_df_lean)
  int alive[BB];
  int J[BB], K1[BB], K2[BB], inblk[BB], Tperm[BB];
  int stop, piv, nK;
  dfl inv;
  dfl cval[32], crem[32];  // per diagonal owner: best live diagonal and live diagonal sum
  int cslot[32], ccol[32];
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

// The same factorization and filter as pchol_filter_df<64>, by 1024 threads
// (LEAN_THREADS): thread (ty, tx) of a 32 x 32 grid owns the Schur entries of
// rows ty + 32u and columns tx + 32v (u, v < 2), so a warp touches one row pair
// of consecutive entries (no bank conflicts) and each thread's update is four
// independent double-float chains.  Two barriers per step instead of three and
// a 32-way pivot search: the 32 threads that own diagonal entries (ty == tx)
// rank their live diagonals right after updating them, and every thread forms
// its own factor-row values S(pv, j) / r from the pivot row, which no thread
// writes during the update.  Each Schur entry gets the same double-float
// operation on the same inputs and pivots tie to the first slot as before;
// only the remaining-trace sum of the stop test is added in another order.
// Square root and reciprocal start from the correctly rounded FP32 intrinsics.
constexpr int LEAN_THREADS = 1024;

__device__ __forceinline__ dfl df_sqrt_lean(dfl a) {
  if (!(a.hi > 0.0f)) return {0.0f, 0.0f};
  const float sq = __fsqrt_rn(a.hi);
  const dfl e = df_add(a, df_neg(df_mul({sq, 0.0f}, {sq, 0.0f})));  // a - sq^2
  return df_fast(sq, e.hi * (0.5f * __frcp_rn(sq)));
}
__device__ __forceinline__ dfl df_recip_lean(dfl b) {
  const float q = __frcp_rn(b.hi);
  const dfl r = df_add({1.0f, 0.0f}, df_neg(df_mul({q, 0.0f}, b)));  // 1 - q b
  return df_fast(q, q * r.hi);
}

__device__ int pchol_filter_df_lean(PcholDfSmemT<64>& sm, int nb, int rows, double tol_loc) {
  constexpr int BB = 64, U = 2, G = 32;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int ty = wid, tx = lane;
  const bool owner = ty == tx;  // owns the diagonal entries ty + 32u
  bool have_total = false;
  dfl thr = {0.f, 0.f};
  if (tid < BB) sm.slot[tid] = tid;
  auto rank_diag = [&]() {
    dfl best = {-1.f, 0.f}, rem = {0.f, 0.f};
    int bs = BB, bc = -1;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int j = ty + G * u;
      if (j < nb && sm.alive[j]) {
        const dfl d = sm.S[j][j];
        rem = df_add(rem, d);
        const int sj = sm.slot[j];
        if (df_gt(d, best) || (df_eq(d, best) && sj < bs)) { best = d; bs = sj; bc = j; }
      }
    }
    sm.cval[ty] = best;
    sm.crem[ty] = rem;
    sm.cslot[ty] = bs;
    sm.ccol[ty] = bc;
  };
  __syncthreads();
  if (owner) rank_diag();
  __syncthreads();
  if (wid == 0) {
    dfl t = sm.crem[lane];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      t = df_add(t, {__shfl_down_sync(0xffffffffu, t.hi, o), __shfl_down_sync(0xffffffffu, t.lo, o)});
    const double total = __shfl_sync(0xffffffffu, df_dbl(t), 0);
    have_total = total > 0.0;
    thr = df_of(tol_loc * total);
  }
  int kept = rows;
  for (int t = 0; t < rows; ++t) {
    if (wid == 0) {
      dfl best = sm.cval[lane], rem = sm.crem[lane];
      int bs = sm.cslot[lane], bc = sm.ccol[lane];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        rem = df_add(rem, {__shfl_down_sync(0xffffffffu, rem.hi, o), __shfl_down_sync(0xffffffffu, rem.lo, o)});
        const dfl ob = {__shfl_down_sync(0xffffffffu, best.hi, o), __shfl_down_sync(0xffffffffu, best.lo, o)};
        const int os = __shfl_down_sync(0xffffffffu, bs, o), oc = __shfl_down_sync(0xffffffffu, bc, o);
        if (df_gt(ob, best) || (df_eq(ob, best) && os < bs)) { best = ob; bs = os; bc = oc; }
      }
      if (lane == 0) {
        const bool stop = !have_total || df_gt(thr, rem) || !(best.hi > 0.f) || bc < 0;
        sm.stop = stop;
        if (!stop) {
          // LAPACK order: the pivot column moves to slot t, slot t's column to the pivot's slot
          const int o = sm.ord[t];
          sm.ord[t] = bc;
          sm.ord[bs] = o;
          sm.slot[o] = bs;
          sm.slot[bc] = t;
          sm.alive[bc] = 0;
          const dfl r = df_sqrt_lean(sm.S[bc][bc]);
          sm.R[t][bc] = r;
          sm.inv = df_recip_lean(r);
          sm.piv = bc;
        }
      }
    }
    __syncthreads();
    if (sm.stop) { kept = t; break; }
    const int pv = sm.piv;
    const dfl inv = sm.inv;
    dfl ru[U], rv[U];
    bool au[U], av[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int j = ty + G * u, c = tx + G * u;
      au[u] = j < nb && sm.alive[j];
      av[u] = c < nb && sm.alive[c];
      ru[u] = au[u] ? df_mul(sm.S[pv][j], inv) : dfl{0.f, 0.f};
      rv[u] = av[u] ? df_mul(sm.S[pv][c], inv) : dfl{0.f, 0.f};
    }
    if (ty == 0) {
#pragma unroll
      for (int v = 0; v < U; ++v)
        if (av[v]) sm.R[t][tx + G * v] = rv[v];
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int v = 0; v < U; ++v)
        if (au[u] && av[v]) sm.S[ty + G * u][tx + G * v] = df_fms(sm.S[ty + G * u][tx + G * v], ru[u], rv[v]);
    if (owner) rank_diag();
    __syncthreads();
  }
  return kept;
}

}  // namespace
}  // namespace rbrp
