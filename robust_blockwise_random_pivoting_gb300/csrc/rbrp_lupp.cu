// rbrp_lupp.cu - partial-pivoted LU pivots for the RandLUPP_OS comparison ID.
//
// RandLUPP_OS (gpu/randLUPP_OS.cu:48-90) factors Yk = Y(1:k, :)^T (n x k) with
// cusolverDnDgetrf and turns the pivots into a column permutation of Y by
// sequential swaps (pivots_to_permutation, gpu/permute.cu:8-23); the skeleton
// is its first k entries.  Only the pivots are used, so only they are computed:
//
//  * k_lupp_load: tiled transpose of W (k x n) into Wt (n x k, column major), so
//    that a column of the elimination is one coalesced stream; checks finiteness.
//  * k_lupp: one cooperative launch runs all k elimination steps.  Rows of Wt
//    never move: the row swaps of LAPACK are kept as positions (rowAt in global
//    memory, the owned rows' positions in shared memory), which is all the pivot
//    rule needs - the pivot of step j is the live row of largest |Wt(i, j)|, ties
//    to the smallest current position (idamax's first index).  CTA c owns the
//    32-row tiles c, c + grid, ...; their current column, positions and dead
//    flags stay in its shared memory.  Warp w >= 1 updates the columns j+1+w,
//    j+9+w, ...; warp 0 updates column j+1 (prefetched by warp 1 while warp 0
//    reduces the pivot candidates), forms its (|value|, position) keys for the
//    next step, and the columns j+9, j+17, ....  One grid barrier per step,
//    bounded in time; data written by other CTAs is read through L2.
//
// Arithmetic follows dgetf2: l_i = Wt(i, j) * (1 / u_j), Wt(i, c) -= l_i u_c (one
// FMA).  LAPACK's blocked/recursive dgetrf rounds in another order, so pivots
// can differ from it only at near-ties.
#include <climits>

#include "rbrp_internal.h"

namespace rbrp {
namespace {

constexpr int LU_THREADS = 256;
constexpr int LU_WARPS = LU_THREADS / 32;
constexpr int ST_SINGULAR = 1;      // a zero pivot (dgetrf info > 0)
constexpr int ST_NONFINITE = 2;     // Inf/NaN in W
constexpr int ST_TIMEOUT = 3;       // a grid barrier expired
constexpr int ST_BADPIVOT = 4;      // no valid pivot row (cannot happen for 1 <= k <= n)

struct __align__(16) LuKey {  // argmax candidate: larger v wins, then smaller pos
  double v;
  int pos, row;
};
struct GridBar {
  unsigned count, gen;
  int abort, status;
};

__device__ __forceinline__ bool key_better(double av, int ap, double bv, int bp) {
  return av > bv || (av == bv && ap < bp);
}

__device__ __forceinline__ void warp_argmax(double& v, int& pos, int& row) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double ov = __shfl_xor_sync(0xffffffffu, v, o);
    const int op = __shfl_xor_sync(0xffffffffu, pos, o);
    const int orow = __shfl_xor_sync(0xffffffffu, row, o);
    if (key_better(ov, op, v, pos)) v = ov, pos = op, row = orow;
  }
}

// Sense-by-generation grid barrier.  Thread 0 of each CTA arrives; the last
// arrival resets the count and advances the generation.  A wait longer than
// `budget` SM clocks (~2 s by default) sets `abort`; every later barrier then
// returns false at once.  Thread 0 decides the result for its whole CTA, so the
// CTA never splits.
__device__ bool grid_sync(GridBar* b, unsigned nblocks, long long budget) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* vgen = &b->gen;
    volatile int* vabort = &b->abort;
    const unsigned g = *vgen;
    __threadfence();
    if (atomicAdd(&b->count, 1u) == nblocks - 1) {
      atomicExch(&b->count, 0u);
      __threadfence();
      atomicAdd(&b->gen, 1u);
    } else {
      const long long t0 = clock64();
      while (*vgen == g) {
        if (*vabort) break;
        if (clock64() - t0 > budget) {
          atomicExch(&b->abort, 1);
          atomicCAS(&b->status, 0, ST_TIMEOUT);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    s_ok = *vabort == 0;
  }
  __syncthreads();
  return s_ok != 0;
}

// Wt (n x k, ld n) = W^T for W (k x n, ld ldw); flags non-finite entries.
__global__ void k_lupp_load(const double* __restrict__ W, int64_t ldw, int k, int n, double* __restrict__ Wt,
                            GridBar* bar) {
  __shared__ double tile[32][33];
  const int c0 = blockIdx.y * 32, i0 = blockIdx.x * 32;  // c: row of W, i: column of W
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  bool bad = false;
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + r, c = c0 + tx;
    double v = 0.0;
    if (i < n && c < k) {
      v = W[c + (int64_t)i * ldw];
      bad |= !isfinite(v);
    }
    tile[r][tx] = v;
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int c = c0 + r, i = i0 + tx;
    if (i < n && c < k) Wt[i + (int64_t)c * n] = tile[tx][r];
  }
  if (__any_sync(0xffffffffu, bad) && tx == 0) atomicCAS(&bar->status, 0, ST_NONFINITE);
}

// Dynamic shared memory of k_lupp for k columns and tpc tiles per CTA.
__host__ __device__ inline size_t lupp_smem(int k, int tpc) {
  return (size_t)k * sizeof(double) + 3 * (size_t)tpc * 32 * sizeof(double) + (size_t)tpc * 32 * sizeof(int) +
         (size_t)tpc * 32;
}

__global__ void __launch_bounds__(LU_THREADS) k_lupp(double* __restrict__ Wt, int k, int n, int tpc,
                                                     int* __restrict__ rowAt, int* __restrict__ pivrow,
                                                     int* __restrict__ ipiv, LuKey* __restrict__ parts, GridBar* bar,
                                                     int* __restrict__ perm, long long budget) {
  // shared: pivot row u (k) | current column, two steps (2 x tpc x 32) | next column prefetch
  // (tpc x 32) | positions of the owned rows (tpc x 32) | dead flags (tpc x 32)
  extern __shared__ __align__(16) unsigned char lsm[];
  double* u = reinterpret_cast<double*>(lsm);
  double* colv = u + k;
  double* colnx = colv + 2 * tpc * 32;
  int* posl = reinterpret_cast<int*>(colnx + tpc * 32);
  unsigned char* deadl = reinterpret_cast<unsigned char*>(posl + tpc * 32);
  __shared__ int s_p, s_pp, s_rj;
  __shared__ double s_piv;
  const unsigned nblocks = gridDim.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ntiles = (n + 31) / 32;
  if (*(volatile int*)&bar->status == ST_NONFINITE) return;  // load kernel flagged W (uniform over the grid)

  // positions start as the identity; the keys of column 0
  double bv = -1.0;
  int bp = INT_MAX, br = -1;
  if (warp == 0) {
    for (int q = 0; q < tpc; ++q) {
      const int t = blockIdx.x + q * (int)nblocks, i = t * 32 + lane, o = q * 32 + lane;
      const bool in = t < ntiles && i < n;
      posl[o] = i;
      deadl[o] = in ? 0 : 1;
      const double a0 = in ? __ldcg(Wt + i) : 0.0;
      colv[o] = a0;
      if (in) {
        rowAt[i] = i;
        if (key_better(fabs(a0), i, bv, bp)) bv = fabs(a0), bp = i, br = i;
      }
    }
    warp_argmax(bv, bp, br);
    if (lane == 0) parts[blockIdx.x] = LuKey{bv, bp, br};
  }
  if (!grid_sync(bar, nblocks, budget)) return;

  for (int j = 0; j < k; ++j) {
    const LuKey* in = parts + (size_t)(j & 1) * nblocks;
    LuKey* out = parts + (size_t)((j + 1) & 1) * nblocks;
    const double* cur = colv + (j & 1) * tpc * 32;
    double* nxt = colv + ((j + 1) & 1) * tpc * 32;
    if (warp == 0) {  // the pivot: best of the per-CTA candidates (one 16-byte load each)
      double v = -1.0;
      int pos = INT_MAX, row = -1;
      const int rj = lane == 0 ? __ldcg(rowAt + j) : 0;
#pragma unroll 4
      for (unsigned c = lane; c < nblocks; c += 32) {
        const int4 e = __ldcg(reinterpret_cast<const int4*>(in + c));
        const double cv = __hiloint2double(e.y, e.x);
        if (key_better(cv, e.z, v, pos)) v = cv, pos = e.z, row = e.w;
      }
      warp_argmax(v, pos, row);
      if (lane == 0) {
        s_p = row;
        s_pp = pos;
        s_rj = rj;
      }
    } else if (warp == 1 && j + 1 < k) {  // meanwhile: column j+1 of the owned rows (independent of the pivot)
      for (int q = 0; q < tpc; ++q) {
        const int i = (blockIdx.x + q * (int)nblocks) * 32 + lane;
        colnx[q * 32 + lane] = i < n ? __ldcg(Wt + i + (int64_t)(j + 1) * n) : 0.0;
      }
    }
    __syncthreads();
    const int p = s_p, pp = s_pp, rj = s_rj;
    // every step has a live row, so p is valid; the test is uniform over the grid
    if (p < 0 || p >= n || pp < j || pp >= n) {
      if (threadIdx.x == 0) atomicCAS(&bar->status, 0, ST_BADPIVOT);
      return;
    }
    for (int c = j + threadIdx.x; c < k; c += LU_THREADS) u[c - j] = __ldcg(Wt + p + (int64_t)c * n);
    __syncthreads();
    if (threadIdx.x == 0) {
      s_piv = u[0];
      if (u[0] == 0.0) atomicCAS(&bar->status, 0, ST_SINGULAR);
      if (blockIdx.x == 0) {
        pivrow[j] = p;
        if (ipiv) ipiv[j] = pp + 1;
      }
    }
    __syncthreads();
    // dgetf2: no scaling (and so no update) when the pivot is exactly zero
    const double inv = s_piv != 0.0 ? 1.0 / s_piv : 0.0;

    double kv = -1.0;
    int kp = INT_MAX, kr = -1;
    for (int q = 0; q < tpc; ++q) {
      const int o = q * 32 + lane;
      const int i = (blockIdx.x + q * (int)nblocks) * 32 + lane;
      const bool live = !deadl[o] && i != p;
      const double l = live ? cur[o] * inv : 0.0;
      double* a = Wt + i;
      if (warp == 0) {
        if (live && i == rj) {  // LAPACK swaps positions j and pp: the row at j moves to pp
          posl[o] = pp;
          rowAt[pp] = i;
        }
        if (live && j + 1 < k) {  // column j+1: from the prefetch, kept in shared memory for the next step
          double nv = colnx[o];
          if (l != 0.0) {
            nv = fma(-l, u[1], nv);
            a[(int64_t)(j + 1) * n] = nv;
          }
          nxt[o] = nv;
          if (key_better(fabs(nv), posl[o], kv, kp)) kv = fabs(nv), kp = posl[o], kr = i;
        }
        if (i == p) deadl[o] = 1;
      }
      if (live && l != 0.0) {
        // eight columns' loads in flight before their stores: one L2 round trip per eight columns
        int c = j + 1 + (warp == 0 ? LU_WARPS : warp);
        for (; c + 7 * LU_WARPS < k; c += 8 * LU_WARPS) {
          double v[8];
#pragma unroll
          for (int e = 0; e < 8; ++e) v[e] = __ldcg(a + (int64_t)(c + e * LU_WARPS) * n);
#pragma unroll
          for (int e = 0; e < 8; ++e) a[(int64_t)(c + e * LU_WARPS) * n] = fma(-l, u[c + e * LU_WARPS - j], v[e]);
        }
        for (; c < k; c += LU_WARPS) a[(int64_t)c * n] = fma(-l, u[c - j], __ldcg(a + (int64_t)c * n));
      }
    }
    if (warp == 0) {
      warp_argmax(kv, kp, kr);
      if (lane == 0) out[blockIdx.x] = LuKey{kv, kp, kr};
    }
    if (!grid_sync(bar, nblocks, budget)) return;
  }

  // perm[pos] = the original row at position pos after all swaps
  for (int t = blockIdx.x; t < ntiles; t += nblocks) {
    const int pos = t * 32 + lane;
    if (warp == 0 && pos < n) perm[pos] = pos < k ? __ldcg(pivrow + pos) : __ldcg(rowAt + pos);
  }
}

}  // namespace
}  // namespace rbrp

using namespace rbrp;

extern "C" rbrp_status rbrp_lupp_pivots_f64(rbrp_handle h, int k, int n, const double* dW, int64_t ldw, int* dPerm,
                                           int* dIpiv) {
  if (!h) return RBRP_ERR_INVALID_ARG;
  if (k < 1 || n < k || ldw < k || !dW || !dPerm)
    return set_error(h, RBRP_ERR_INVALID_ARG, "need 1 <= k <= n, ldw >= k, W and perm");
  DeviceGuard g(h->device);
  rbrp_status s;
  int sms = 0, per_sm = 0;
  s = cuda_check(h, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device), "SM count");
  if (s != RBRP_OK) return s;
  const int ntiles = (n + 31) / 32;
  // shared memory for the most tiles a CTA can own (one CTA per SM); more CTAs per SM own fewer
  const int tpc_max = (ntiles + sms - 1) / sms;
  const size_t smem = lupp_smem(k, tpc_max);
  if (smem > 200 * 1024)
    return set_error(h, RBRP_ERR_INVALID_ARG, "LU pivots: k and n too large for the shared-memory working set");
  s = cuda_check(h, cudaFuncSetAttribute(k_lupp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                 "cudaFuncSetAttribute(k_lupp)");
  if (s != RBRP_OK) return s;
  s = cuda_check(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lupp, LU_THREADS, smem), "occupancy");
  if (s != RBRP_OK) return s;
  if (per_sm < 1) return set_error(h, RBRP_ERR_INVALID_ARG, "k_lupp does not fit on an SM");
  // all co-resident CTAs: the update's latency is hidden by warps, which matters more than
  // the per-CTA candidate scan and barrier arrival (one CTA per SM measured slower)
  const int grid = std::min(ntiles, per_sm * sms);
  const int tpc = (ntiles + grid - 1) / grid;   // <= tpc_max

  // workspace: Wt | parts (2 x grid) | bar | rowAt | pivrow
  auto up = [](size_t x) { return (x + 255) / 256 * 256; };
  const size_t o_parts = up((size_t)n * k * sizeof(double));
  const size_t o_bar = o_parts + up(2 * (size_t)grid * sizeof(LuKey));
  const size_t o_row = o_bar + up(sizeof(GridBar));
  const size_t o_piv = o_row + up((size_t)n * sizeof(int));
  const size_t bytes = o_piv + up((size_t)k * sizeof(int));
  if (h->lupp_bytes < bytes) {
    if (h->lupp_ws) cudaFree(h->lupp_ws);
    h->lupp_ws = nullptr;
    h->lupp_bytes = 0;
    s = cuda_check(h, cudaMalloc(&h->lupp_ws, bytes), "cudaMalloc(LU workspace)");
    if (s != RBRP_OK) return s;
    h->lupp_bytes = bytes;
  }
  unsigned char* w = static_cast<unsigned char*>(h->lupp_ws);
  double* Wt = reinterpret_cast<double*>(w);
  LuKey* parts = reinterpret_cast<LuKey*>(w + o_parts);
  GridBar* bar = reinterpret_cast<GridBar*>(w + o_bar);
  int* rowAt = reinterpret_cast<int*>(w + o_row);
  int* pivrow = reinterpret_cast<int*>(w + o_piv);

  cudaStream_t st = h->stream;
  s = cuda_check(h, cudaMemsetAsync(bar, 0, sizeof(GridBar), st), "clear barrier");
  if (s != RBRP_OK) return s;
  k_lupp_load<<<dim3(ntiles, (k + 31) / 32), 256, 0, st>>>(dW, ldw, k, n, Wt, bar);
  s = cuda_check(h, cudaGetLastError(), "k_lupp_load");
  if (s != RBRP_OK) return s;
  int tpc_arg = tpc;
  long long budget = h->wait_budget > 0 ? h->wait_budget : kWaitBudgetDefault;
  void* args[] = {&Wt, &k, &n, &tpc_arg, &rowAt, &pivrow, &dIpiv, &parts, &bar, &dPerm, &budget};
  s = cuda_check(h, cudaLaunchCooperativeKernel((const void*)k_lupp, dim3(grid), dim3(LU_THREADS), args, smem, st),
                 "cooperative launch of k_lupp");
  if (s != RBRP_OK) return s;
  GridBar hb;
  s = cuda_check(h, cudaMemcpyAsync(&hb, bar, sizeof(GridBar), cudaMemcpyDeviceToHost, st), "read LU status");
  if (s == RBRP_OK) s = cuda_check(h, cudaStreamSynchronize(st), "LU pivots");
  if (s != RBRP_OK) return s;
  if (hb.status == ST_NONFINITE) return set_error(h, RBRP_ERR_NUMERIC, "non-finite entries in W");
  if (hb.status == ST_TIMEOUT || hb.abort)
    return set_error(h, RBRP_ERR_DEVICE_TIMEOUT, "a grid barrier of the LU timed out; the kernel aborted cleanly");
  if (hb.status == ST_BADPIVOT) return set_error(h, RBRP_ERR_NUMERIC, "LU pivot search found no live row");
  if (hb.status == ST_SINGULAR) return set_error(h, RBRP_ERR_NUMERIC, "zero pivot: W has rank below k");
  return RBRP_OK;
}
