// rbrp_capi.cu - C ABI, workspace management, interpolation-matrix solve
// (a10) and ID-error kernel (a11) of the GB300 RBRP library.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "rbrp_internal.h"
#include "../../include/rbrp_gb300_testing.h"

namespace rbrp {

// ===========================================================================
// a10: T = R11^{-1} R12 (matlab/driver.m:86; gpu/interp.cu:45-105 solves the
// same triangular system after re-factoring a sketch; gpu/id_cpqr.cu:133-136).
// R is the RBRP factor (row major, ld = n, indexed by position): R11 =
// R[:k, :k] upper triangular, R12 = R[:k, k:].  T is k x (n-k), column major.
// ===========================================================================
__global__ void k_gather_T(const double* __restrict__ R, int64_t ldr, int k, int ncols, double* __restrict__ T) {
  __shared__ double tile[32][33];
  const int c0 = blockIdx.x * 32, a0 = blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int q = 0; q < 32; q += 8) {
    const int a = a0 + ty + q, c = c0 + tx;
    tile[ty + q][tx] = (a < k && c < ncols) ? R[(int64_t)a * ldr + k + c] : 0.0;
  }
  __syncthreads();
  for (int q = 0; q < 32; q += 8) {
    const int c = c0 + ty + q, a = a0 + tx;
    if (a < k && c < ncols) T[a + (int64_t)c * k] = tile[tx][ty + q];
  }
}

struct TrsmSmem {
  double Rs[64][65];
  double Xs[64][33];
  double Acc[64][33];
};

// Block back substitution, 32 right-hand sides per CTA, 64-row diagonal blocks
// from the bottom; the update of a row block by the solved blocks below it is a
// 64 x 64 x 32 product per step.
__global__ void __launch_bounds__(256) k_trsm_T(const double* __restrict__ R, int64_t ldr, int k, int ncols,
                                                double* __restrict__ T) {
  extern __shared__ __align__(16) unsigned char dyn_smem[];
  TrsmSmem& sm = *reinterpret_cast<TrsmSmem*>(dyn_smem);
  const int tid = threadIdx.x;
  const int c0 = blockIdx.x * 32;
  const int nc = min(32, ncols - c0);
  const int nbk = (k + 63) / 64;
  const int x = tid >> 2;  // output row of this thread in the 64 x 32 tile
  for (int bi = nbk - 1; bi >= 0; --bi) {
    const int b0 = bi * 64, bl = min(64, k - b0);
    for (int idx = tid; idx < 64 * 32; idx += 256) {
      const int xr = idx & 63, c = idx >> 6;
      sm.Acc[xr][c] = (xr < bl && c < nc) ? T[(b0 + xr) + (int64_t)(c0 + c) * k] : 0.0;
    }
    double acc[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) acc[q] = 0.0;
    for (int bj = bi + 1; bj < nbk; ++bj) {
      const int cr = bj * 64, cl = min(64, k - cr);
      __syncthreads();
      for (int idx = tid; idx < 64 * 64; idx += 256) {
        const int y = idx & 63, xr = idx >> 6;
        sm.Rs[xr][y] = (xr < bl && y < cl) ? R[(int64_t)(b0 + xr) * ldr + cr + y] : 0.0;
      }
      for (int idx = tid; idx < 64 * 32; idx += 256) {
        const int y = idx & 63, c = idx >> 6;
        sm.Xs[y][c] = (y < cl && c < nc) ? T[(cr + y) + (int64_t)(c0 + c) * k] : 0.0;
      }
      __syncthreads();
#pragma unroll 4
      for (int y = 0; y < 64; ++y) {
        const double r = sm.Rs[x][y];
#pragma unroll
        for (int q = 0; q < 8; ++q) acc[q] = fma(r, sm.Xs[y][(tid & 3) + 4 * q], acc[q]);
      }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 8; ++q) sm.Acc[x][(tid & 3) + 4 * q] -= acc[q];
    for (int idx = tid; idx < 64 * 64; idx += 256) {
      const int y = idx & 63, xr = idx >> 6;
      sm.Rs[xr][y] = (xr < bl && y < bl && y >= xr) ? R[(int64_t)(b0 + xr) * ldr + b0 + y] : 0.0;
    }
    __syncthreads();
    if (tid < nc) {
      for (int xr = bl - 1; xr >= 0; --xr) {
        double v = sm.Acc[xr][tid];
        for (int y = xr + 1; y < bl; ++y) v = fma(-sm.Rs[xr][y], sm.Acc[y][tid], v);
        sm.Acc[xr][tid] = v / sm.Rs[xr][xr];
      }
    }
    __syncthreads();
    for (int idx = tid; idx < 64 * 32; idx += 256) {
      const int xr = idx & 63, c = idx >> 6;
      if (xr < bl && c < nc) T[(b0 + xr) + (int64_t)(c0 + c) * k] = sm.Acc[xr][c];
    }
    __syncthreads();
  }
}

// Double-float form of the same solve.  GB300's FP64 pipe issues ~1/64 of its
// FP32 pipe's rate, so the whole solve runs in double-float arithmetic on the
// FP32 pipe: R11 and the right-hand sides are split once into float pairs
// (hi + lo, ~48 significant bits) by k_split_df, the block updates use
// error-free products (FMA split) and TwoSum, the 64 x 64 diagonal blocks are
// solved in double-float too, and T is joined back to FP64 once at the end.
__global__ void k_split_df(const double* __restrict__ R, int64_t ldr, int k, int ncols,
                           float2* __restrict__ R11df, float2* __restrict__ Tdf) {
  const int64_t total11 = (int64_t)k * k, totalT = (int64_t)k * ncols;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total11 + totalT;
       idx += (int64_t)gridDim.x * blockDim.x) {
    double x;
    float2* dst;
    if (idx < total11) {  // R11 row major (ld k), upper triangle
      const int a = (int)(idx / k), c = (int)(idx % k);
      x = c >= a ? R[(int64_t)a * ldr + c] : 0.0;
      dst = R11df + idx;
    } else {              // T column major (ld k), from R12 row major
      const int64_t t = idx - total11;
      const int c = (int)(t / k), a = (int)(t % k);
      x = R[(int64_t)a * ldr + k + c];
      dst = Tdf + t;
    }
    const float hi = (float)x;
    *dst = make_float2(hi, (float)(x - (double)hi));
  }
}

__global__ void k_join_df(const float2* __restrict__ Tdf, int64_t count, double* __restrict__ T) {
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < count; idx += (int64_t)gridDim.x * blockDim.x) {
    const float2 v = Tdf[idx];
    T[idx] = (double)v.x + (double)v.y;
  }
}

__device__ __forceinline__ float2 df2_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return make_float2(s, (a - (s - bb)) + (b - bb));
}
__device__ __forceinline__ float2 df2_fast(float a, float b) {
  const float s = a + b;
  return make_float2(s, b - (s - a));
}
// (sh, sl) += a * b in double-float: the exact product a.x b.x = p + e (FMA split)
// and the cross terms go into the low part by FMAs, the high parts are added by
// TwoSum with its error into the low part (12 FP32 operations).
__device__ __forceinline__ void df_mac(float& sh, float& sl, float2 a, float2 b) {
  const float p = a.x * b.x;
  const float e = fmaf(a.x, b.x, -p);
  sl = fmaf(a.y, b.x, fmaf(a.x, b.y, sl + e));
  const float t = sh + p;
  const float bb = t - sh;
  sl += (sh - (t - bb)) + (p - bb);
  sh = t;
}
__device__ __forceinline__ float2 df2_add(float2 a, float2 b) {
  float2 s = df2_two_sum(a.x, b.x);
  s.y += a.y + b.y;
  return df2_fast(s.x, s.y);
}
__device__ __forceinline__ float2 df2_mul(float2 a, float2 b) {
  const float p = a.x * b.x;
  float e = fmaf(a.x, b.x, -p);
  e = fmaf(a.x, b.y, e);
  e = fmaf(a.y, b.x, e);
  return df2_fast(p, e);
}
__device__ __forceinline__ float2 df2_recip(float2 b) {
  const float q = 1.0f / b.x;
  const float2 r = df2_add(make_float2(1.0f, 0.0f), df2_mul(make_float2(-q, 0.0f), b));
  return df2_fast(q, q * r.x);
}

// The double-float solve is right-looking: block row b (64 rows from the bottom
// up) is solved for all columns at once, then its product with R11(0:b0, b) is
// subtracted from every earlier row.  Each step has work over rows and columns,
// so the whole GPU stays busy however few columns T has.  (A left-looking form,
// one CTA per 32 columns for the whole solve, had as many CTAs as column tiles:
// 120 for the adjoint's 3822 columns; it took 8.5 ms at 8192 x 8192, k = 2033,
// against 7.6, and the same 16.2 ms at 16384.)
//
// k_trsm_rl_diag: X_b = R11(b, b)^{-1} B_b, one warp per column, lane l holding
// rows l and l + 32 of the block; back substitution with the solved value
// broadcast by shuffles, in double-float.
__global__ void __launch_bounds__(256) k_trsm_rl_diag(const float2* __restrict__ R11, int k, int ncols, int b0, int bl,
                                                      float2* __restrict__ T) {
  __shared__ float2 Rd[64][65];
  __shared__ float2 inv[64];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  for (int idx = tid; idx < 64 * 64; idx += 256) {
    const int xr = idx >> 6, y = idx & 63;
    Rd[xr][y] = (xr < bl && y < bl && y >= xr) ? R11[(int64_t)(b0 + xr) * k + b0 + y] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  if (tid < bl) inv[tid] = df2_recip(Rd[tid][tid]);
  __syncthreads();
  const int c = blockIdx.x * 8 + w;
  if (c >= ncols) return;
  float2* col = T + b0 + (int64_t)c * k;
  float2 v0 = lane < bl ? col[lane] : make_float2(0.f, 0.f);
  float2 v1 = lane + 32 < bl ? col[lane + 32] : make_float2(0.f, 0.f);
  for (int r = bl - 1; r >= 0; --r) {
    // the owner of row r finishes it; every lane then removes its rows' share
    const float2 mine = r < 32 ? v0 : v1;
    const float2 xr = df2_mul(mine, inv[r]);
    const float2 x = make_float2(__shfl_sync(0xffffffffu, xr.x, r & 31), __shfl_sync(0xffffffffu, xr.y, r & 31));
    if (lane == (r & 31)) {
      if (r < 32) v0 = x; else v1 = x;
    }
    if (lane < r) df_mac(v0.x, v0.y, make_float2(-Rd[lane][r].x, -Rd[lane][r].y), x);
    if (lane + 32 < r) df_mac(v1.x, v1.y, make_float2(-Rd[lane + 32][r].x, -Rd[lane + 32][r].y), x);
    // keep the low parts small, as the left-looking solve does after each block
    if (lane < r) v0 = df2_fast(v0.x, v0.y);
    if (lane + 32 < r) v1 = df2_fast(v1.x, v1.y);
  }
  if (lane < bl) col[lane] = v0;
  if (lane + 32 < bl) col[lane + 32] = v1;
}

// k_trsm_rl_update: B(rows of tile, cols of tile) -= R11(rows, b) X_b for the
// 64 x 64 tile (blockIdx.x: rows below b0, blockIdx.y: columns), in double-float:
// each thread two rows (x, x + 32) and 8 columns, so every shared load of X feeds
// two products; each product exact (FMA split) and summed by TwoSum.
struct TrsmRlSmem {
  float2 Rs[64][65];
  float2 Xs[64][65];
};
__global__ void __launch_bounds__(256) k_trsm_rl_update(const float2* __restrict__ R11, int k, int ncols, int b0,
                                                        int bl, float2* __restrict__ T) {
  extern __shared__ __align__(16) unsigned char dyn_smem[];
  TrsmRlSmem& sm = *reinterpret_cast<TrsmRlSmem*>(dyn_smem);
  const int tid = threadIdx.x;
  const int r0 = blockIdx.x * 64, c0 = blockIdx.y * 64;
  const int nc = min(64, ncols - c0);
  for (int idx = tid; idx < 64 * 64; idx += 256) {
    const int xr = idx >> 6, y = idx & 63;
    const float2 v = y < bl ? R11[(int64_t)(r0 + xr) * k + b0 + y] : make_float2(0.f, 0.f);
    sm.Rs[xr][y] = make_float2(-v.x, -v.y);
  }
  for (int idx = tid; idx < 64 * 64; idx += 256) {
    const int y = idx & 63, c = idx >> 6;
    sm.Xs[y][c] = (y < bl && c < nc) ? T[(b0 + y) + (int64_t)(c0 + c) * k] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  const int x = tid >> 3, cq = tid & 7;  // rows x and x + 32, columns cq + 8 q
  float sh[2][8], sl[2][8];
#pragma unroll
  for (int h = 0; h < 2; ++h)
#pragma unroll
    for (int q = 0; q < 8; ++q) sh[h][q] = sl[h][q] = 0.f;
#pragma unroll 2
  for (int y = 0; y < 64; ++y) {
    const float2 ra = sm.Rs[x][y], rb = sm.Rs[x + 32][y];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const float2 xv = sm.Xs[y][cq + 8 * q];
      df_mac(sh[0][q], sl[0][q], ra, xv);
      df_mac(sh[1][q], sl[1][q], rb, xv);
    }
  }
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int row = r0 + x + 32 * h;  // r0 + 63 < b0: every row of the tile exists
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int c = cq + 8 * q;
      if (c < nc) {
        float2* t = T + row + (int64_t)(c0 + c) * k;
        *t = df2_add(*t, make_float2(sh[h][q], sl[h][q]));
      }
    }
  }
}

// ===========================================================================
// a11: ||A(:, rd) - A(:, S) T||_F^2 in FP64 (python/RBRP.ipynb cell 7 lines
// 40-53; gpu/id_cpqr.cu:145-170).  Validation only: one FP64 GEMM.
// ===========================================================================
template <typename T>
__global__ void __launch_bounds__(256)
k_id_error(const T* __restrict__ A, int64_t lda, const int* __restrict__ perm, const double* __restrict__ Tm,
           int k, int m, int n, double* __restrict__ part) {
  __shared__ double As[64][33];
  __shared__ double Ts[32][33];
  __shared__ double red[32];
  const int tid = threadIdx.x;
  const int r0 = blockIdx.y * 64, c0 = blockIdx.x * 32;
  const int ncols = n - k;
  const int x = tid >> 2;
  double acc[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) acc[q] = 0.0;
  for (int a0 = 0; a0 < k; a0 += 32) {
    __syncthreads();
    for (int idx = tid; idx < 64 * 32; idx += 256) {
      const int xr = idx & 63, y = idx >> 6;
      const int r = r0 + xr, a = a0 + y;
      As[xr][y] = (r < m && a < k) ? (double)A[r + (int64_t)perm[a] * lda] : 0.0;
    }
    for (int idx = tid; idx < 32 * 32; idx += 256) {
      const int y = idx & 31, c = idx >> 5;
      Ts[y][c] = (a0 + y < k && c0 + c < ncols) ? Tm[(a0 + y) + (int64_t)(c0 + c) * k] : 0.0;
    }
    __syncthreads();
#pragma unroll 4
    for (int y = 0; y < 32; ++y) {
      const double av = As[x][y];
#pragma unroll
      for (int q = 0; q < 8; ++q) acc[q] = fma(av, Ts[y][(tid & 3) + 4 * q], acc[q]);
    }
  }
  double s = 0.0;
  const int r = r0 + x;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int c = c0 + (tid & 3) + 4 * q;
    if (r < m && c < ncols) {
      const double e = (double)A[r + (int64_t)perm[k + c] * lda] - acc[q];
      s = fma(e, e, s);
    }
  }
  s = block_sum(s, red);
  if (tid == 0) part[(int64_t)blockIdx.y * gridDim.x + blockIdx.x] = s;
}

// ---------------------------------------------------------------------------
int splits_for(int i, int m) {
  const int tiles = (i + 31) / 32;
  int s = 304 / tiles;  // about two CTAs per SM
  s = s < 1 ? 1 : s;
  const int cap = m / 128 > 1 ? m / 128 : 1;
  return s > cap ? cap : s;
}

Layout make_layout(int m, int n, int kmax, size_t elem, bool residual) {
  Layout L;
  L.m = m;
  L.n = n;
  L.kmax = kmax;
  L.ntiles = (m + 63) / 64;
  L.nproj = (n + 31) / 32;   // partials of the projection: 32 positions per CTA at the finest
  L.cpart_rows = residual ? 1 : (kmax > 304 * 32 ? kmax : 304 * 32);
  L.elem = elem;
  L.residual = residual;
  L.ld_res = residual ? ((int64_t)m + 31) / 32 * 32 : 0;  // 128-byte aligned columns
  return L;
}

rbrp_status set_error(rbrp_handle h, rbrp_status s, const std::string& msg) {
  if (h) h->last_error = msg;
  return s;
}

rbrp_status cuda_check(rbrp_handle h, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return RBRP_OK;
  std::string msg = std::string(what) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return set_error(h, RBRP_ERR_ALLOC, msg);
  return set_error(h, RBRP_ERR_CUDA, msg);
}

static size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

rbrp_status ensure_workspace(rbrp_handle h, const Layout& L) {
  const size_t m = L.m, n = L.n, kmax = L.kmax, el = L.elem;
  const size_t M2 = (size_t)MAXB * MAXB;
  struct Item {
    void** ptr;
    size_t bytes;
  } items[] = {
      {(void**)&h->st, sizeof(State)},
      {(void**)&h->diags, n * 8},
      {(void**)&h->perm, n * 4},
      {(void**)&h->pbuf, 2 * n * 8},
      {(void**)&h->kbuf, n * 8},
      {(void**)&h->Q, (L.residual ? (size_t)L.ld_res * MAXB : m * kmax) * el},
      {(void**)&h->part_norm, L.residual ? (size_t)P2_MAX_SPLIT_WS * n * 8 : 0},
      {(void**)&h->Wpart, L.residual ? (size_t)P1_MAX_SPLIT * MAXB * n * 8 : 0},
      {(void**)&h->Ares, L.residual ? (size_t)L.ld_res * n * sizeof(float) : 0},
      {(void**)&h->Qh, L.residual ? (size_t)L.ld_res * MAXB * sizeof(float) : 0},
      {(void**)&h->Ql, L.residual ? (size_t)L.ld_res * MAXB * sizeof(float) : 0},
      {(void**)&h->Qrh, L.residual ? m * MAXB * sizeof(float) : 0},
      {(void**)&h->Qrl, L.residual ? m * MAXB * sizeof(float) : 0},
      {(void**)&h->Wth, L.residual ? n * MAXB * sizeof(float) : 0},
      {(void**)&h->Wtl, L.residual ? n * MAXB * sizeof(float) : 0},
      {(void**)&h->R, kmax * n * 8},
      {(void**)&h->V, m * MAXB * 8},
      {(void**)&h->Q1, m * MAXB * 8},
      {(void**)&h->Cpart, (size_t)L.cpart_rows * MAXB * el},
      {(void**)&h->C, (L.residual ? 1 : kmax) * MAXB * el},
      {(void**)&h->Gpart, (size_t)L.ntiles * M2 * 8},
      {(void**)&h->G, M2 * 8},
      {(void**)&h->G2part, (size_t)L.ntiles * M2 * 8},
      {(void**)&h->G2, M2 * 8},
      {(void**)&h->R11, M2 * 8},
      {(void**)&h->R2, M2 * 8},
      {(void**)&h->ord, MAXB * 4},
      {(void**)&h->js, MAXB * 4},
      {(void**)&h->cols, MAXB * 4},
      {(void**)&h->J, MAXB * 4},
      {(void**)&h->K1, MAXB * 4},
      {(void**)&h->K2, MAXB * 4},
      {(void**)&h->part_res, (size_t)L.nproj * 8},
      {(void**)&h->part_nnz, (size_t)L.nproj * 4},
      {(void**)&h->trace_rank, kmax * 4},
      {(void**)&h->trace_err, kmax * 8},
      {(void**)&h->trace_samp, kmax * 4},
      {(void**)&h->err_part, (size_t)L.ntiles * ((n + 31) / 32) * 8},
  };
  size_t total = 0;
  for (auto& it : items) total += align_up(it.bytes);
  if (total > h->ws_bytes) {
    if (h->ws) cudaFree(h->ws);
    h->ws = nullptr;
    h->ws_bytes = 0;
    rbrp_status s = cuda_check(h, cudaMalloc(&h->ws, total), "workspace cudaMalloc");
    if (s != RBRP_OK) return s;
    h->ws_bytes = total;
  }
  h->ld_res = L.ld_res;
  char* base = static_cast<char*>(h->ws);
  size_t off = 0;
  for (auto& it : items) {
    *it.ptr = base + off;
    off += align_up(it.bytes);
  }
  if (!h->hst) {
    rbrp_status s = cuda_check(h, cudaMallocHost((void**)&h->hst, sizeof(State)), "cudaMallocHost(state)");
    if (s != RBRP_OK) return s;
  }
  return RBRP_OK;
}

static PFN_cuTensorMapEncodeTiled_v12000 tmap_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    else
      cudaGetLastError();
  }
  return fn;
}

rbrp_status make_tmap_f32(rbrp_handle h, void* map, const float* base, uint64_t inner, uint64_t outer,
                          uint64_t ld_elems, uint32_t box_inner, uint32_t box_outer) {
  auto fn = tmap_encoder();
  if (!fn) return set_error(h, RBRP_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
  cuuint64_t dims[2] = {inner, outer};
  cuuint64_t strides[1] = {ld_elems * sizeof(float)};
  cuuint32_t box[2] = {box_inner, box_outer};
  cuuint32_t es[2] = {1, 1};
  CUresult r = fn(static_cast<CUtensorMap*>(map), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims,
                  strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(h, RBRP_ERR_CUDA, "cuTensorMapEncodeTiled failed");
  return RBRP_OK;
}

rbrp_status solve_T(rbrp_handle h, int k, int n) {
  const size_t bytes = (size_t)k * (size_t)(n - k) * sizeof(double);
  if (bytes > h->T_bytes) {
    if (h->T) cudaFree(h->T);
    h->T = nullptr;
    h->T_bytes = 0;
    rbrp_status s = cuda_check(h, cudaMalloc((void**)&h->T, bytes), "cudaMalloc(T)");
    if (s != RBRP_OK) return s;
    h->T_bytes = bytes;
  }
  const int ncols = n - k;
  rbrp_status s;
  if (h->tsolve_fp64) {
    dim3 g1((ncols + 31) / 32, (k + 31) / 32), b1(32, 8);
    k_gather_T<<<g1, b1, 0, h->stream>>>(h->R, n, k, ncols, h->T);
    s = cuda_check(h, cudaFuncSetAttribute(k_trsm_T, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)sizeof(TrsmSmem)), "cudaFuncSetAttribute(k_trsm_T)");
    if (s != RBRP_OK) return s;
    k_trsm_T<<<(ncols + 31) / 32, 256, sizeof(TrsmSmem), h->stream>>>(h->R, n, k, ncols, h->T);
  } else {
    // double-float operands: R11 (k x k) and the right-hand sides (k x ncols), ~16 bytes per T entry
    const size_t need = ((size_t)k * k + (size_t)k * ncols) * sizeof(float2);
    if (need > h->df_bytes) {
      if (h->df_buf) cudaFree(h->df_buf);
      h->df_buf = nullptr;
      h->df_bytes = 0;
      s = cuda_check(h, cudaMalloc(&h->df_buf, need), "cudaMalloc(T solve operands)");
      if (s != RBRP_OK) return s;
      h->df_bytes = need;
    }
    float2* R11df = static_cast<float2*>(h->df_buf);
    float2* Tdf = R11df + (size_t)k * k;
    k_split_df<<<1216, 256, 0, h->stream>>>(h->R, n, k, ncols, R11df, Tdf);
    s = cuda_check(h, cudaFuncSetAttribute(k_trsm_rl_update, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)sizeof(TrsmRlSmem)), "cudaFuncSetAttribute(k_trsm_rl_update)");
    if (s != RBRP_OK) return s;
    const int nbk = (k + 63) / 64;
    for (int bi = nbk - 1; bi >= 0; --bi) {
      const int b0 = bi * 64, bl = std::min(64, k - b0);
      k_trsm_rl_diag<<<(ncols + 7) / 8, 256, 0, h->stream>>>(R11df, k, ncols, b0, bl, Tdf);
      if (b0 > 0)
        k_trsm_rl_update<<<dim3(b0 / 64, (ncols + 63) / 64), 256, sizeof(TrsmRlSmem), h->stream>>>(R11df, k, ncols,
                                                                                                   b0, bl, Tdf);
    }
    k_join_df<<<1216, 256, 0, h->stream>>>(Tdf, (int64_t)k * ncols, h->T);
  }
  return cuda_check(h, cudaGetLastError(), "T solve launch");
}

template <typename T>
rbrp_status id_error(rbrp_handle h, int m, int n, const T* dA, int64_t lda, double* err) {
  const int k = h->k;
  if (k >= n || k == 0) {
    *err = k == 0 ? 1.0 : 0.0;
    return RBRP_OK;
  }
  const int ncols = n - k;
  dim3 g((ncols + 31) / 32, (m + 63) / 64);
  k_id_error<T><<<g, 256, 0, h->stream>>>(dA, lda, h->perm, h->T, k, m, n, h->err_part);
  const size_t np = (size_t)g.x * g.y;
  std::vector<double> part(np);
  rbrp_status s = cuda_check(h, cudaMemcpyAsync(part.data(), h->err_part, np * 8, cudaMemcpyDeviceToHost, h->stream),
                             "ID error copy");
  if (s != RBRP_OK) return s;
  s = cuda_check(h, cudaStreamSynchronize(h->stream), "ID error kernel");
  if (s != RBRP_OK) return s;
  double acc = 0.0;
  for (double v : part) acc += v;
  *err = h->res.res0 > 0.0 ? acc / h->res.res0 : 0.0;
  return RBRP_OK;
}

template rbrp_status id_error<double>(rbrp_handle, int, int, const double*, int64_t, double*);
template rbrp_status id_error<float>(rbrp_handle, int, int, const float*, int64_t, double*);

int prof_begin(rbrp_handle h) {
  if (!h->profiling) return -1;
  while ((int)h->prof_events.size() <= h->prof_next) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) {
      cudaGetLastError();
      return -1;
    }
    h->prof_events.push_back(e);
  }
  cudaEventRecord(h->prof_events[h->prof_next], h->stream);
  return h->prof_next++;
}

void prof_end(rbrp_handle h, int phase, int ev0, double bytes, double flops, int launches) {
  if (ev0 < 0) return;
  const int ev1 = prof_begin(h);
  if (ev1 < 0) return;
  h->marks.push_back({phase, ev0, ev1, bytes, flops, launches});
}

void prof_collect(rbrp_handle h) {
  for (const auto& mk : h->marks) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->prof_events[mk.ev0], h->prof_events[mk.ev1]);
    h->stats.ms[mk.phase] += ms;
    h->stats.bytes[mk.phase] += mk.bytes;
    h->stats.flops[mk.phase] += mk.flops;
    h->stats.launches[mk.phase] += mk.launches;
  }
  h->marks.clear();
  h->prof_next = 0;
}

static rbrp_status check_device_ptr(rbrp_handle h, const void* p, const char* name) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return set_error(h, RBRP_ERR_INVALID_ARG, std::string(name) + " is not a CUDA pointer");
  }
  if (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)
    return set_error(h, RBRP_ERR_INVALID_ARG, std::string(name) + " is not a device pointer");
  if (at.type == cudaMemoryTypeDevice && at.device != h->device)
    return set_error(h, RBRP_ERR_INVALID_ARG, std::string(name) + " lives on another device");
  return RBRP_OK;
}

static rbrp_status validate(rbrp_handle h, int m, int n, const void* dA, int64_t lda, const rbrp_params* p,
                            size_t elem) {
  if (!h) return RBRP_ERR_INVALID_ARG;
  if (!p) return set_error(h, RBRP_ERR_INVALID_ARG, "params is NULL");
  if (m < 1 || n < 1) return set_error(h, RBRP_ERR_INVALID_ARG, "m and n must be >= 1");
  if (lda < m) return set_error(h, RBRP_ERR_INVALID_ARG, "lda < m");
  if (!dA) return set_error(h, RBRP_ERR_INVALID_ARG, "A is NULL");
  if (reinterpret_cast<uintptr_t>(dA) % elem) return set_error(h, RBRP_ERR_INVALID_ARG, "A is misaligned");
  if (p->b < 1 || p->b > MAXB) return set_error(h, RBRP_ERR_INVALID_ARG, "block size b must be in [1, 64]");
  if (!std::isfinite(p->tol) || !std::isfinite(p->tol_loc))
    return set_error(h, RBRP_ERR_INVALID_ARG, "tol and tol_loc must be finite");
  if (p->sampler < 0 || p->sampler > 2) return set_error(h, RBRP_ERR_INVALID_ARG, "unknown sampler");
  if ((int64_t)m * (int64_t)n > ((int64_t)1 << 31) * 16)
    return set_error(h, RBRP_ERR_INVALID_ARG, "matrix too large");
  return check_device_ptr(h, dA, "A");
}

template <typename T>
rbrp_status host_run(rbrp_handle h, int m, int n, const T* hA, int64_t lda, const rbrp_params* p,
                            int* hPerm, double* hT, int64_t ldt, int64_t t_cap, rbrp_result* out) {
  if (!h || !hA || !p) return RBRP_ERR_INVALID_ARG;
  if (m < 1 || n < 1 || lda < m) return set_error(h, RBRP_ERR_INVALID_ARG, "bad shape");
  DeviceGuard g(h->device);
  const size_t bytes = (size_t)lda * (size_t)n * sizeof(T);
  if (bytes > h->hostA_bytes) {
    if (h->hostA_dev) cudaFree(h->hostA_dev);
    h->hostA_dev = nullptr;
    h->hostA_bytes = 0;
    rbrp_status s = cuda_check(h, cudaMalloc(&h->hostA_dev, bytes), "cudaMalloc(A copy)");
    if (s != RBRP_OK) return s;
    h->hostA_bytes = bytes;
  }
  rbrp_status s = cuda_check(h, cudaMemcpyAsync(h->hostA_dev, hA, bytes, cudaMemcpyHostToDevice, h->stream), "copy A in");
  if (s != RBRP_OK) return s;
  s = run_rbrp<T>(h, m, n, static_cast<const T*>(h->hostA_dev), lda, *p, nullptr, out);
  if (s != RBRP_OK) return s;
  if (hPerm) {
    s = cuda_check(h, cudaMemcpyAsync(hPerm, h->perm, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, h->stream),
                   "copy perm out");
    if (s != RBRP_OK) return s;
  }
  const int k = h->k, nc = n - k;
  if (hT && k > 0 && nc > 0 && p->compute_T) {
    if (ldt < k || t_cap < ldt * (int64_t)nc) return set_error(h, RBRP_ERR_CAPACITY, "host T buffer too small");
    s = cuda_check(h, cudaMemcpy2DAsync(hT, ldt * sizeof(double), h->T, (size_t)k * sizeof(double),
                                        (size_t)k * sizeof(double), nc, cudaMemcpyDeviceToHost, h->stream),
                   "copy T out");
    if (s != RBRP_OK) return s;
  }
  return cuda_check(h, cudaStreamSynchronize(h->stream), "host-buffer run");
}

// Algorithmic flops of a finished run: per block t, 2 m n_t b_t (projection)
// + 4 m k_t b^_t (one CGS pass) + 4 m b^_t^2 (panel QR), plus k^2 (n - k) (T).
double run_flops(const rbrp_handle h, bool with_T) {
  double f = 0.0;
  int prev = 0;
  for (size_t t = 0; t < h->h_ranks.size(); ++t) {
    const double kt = prev, bt = h->h_ranks[t] - prev, bh = h->h_samp[t];
    const double nt = (double)h->n - h->h_ranks[t];
    f += 2.0 * h->m * nt * bt + 4.0 * h->m * kt * bh + 4.0 * h->m * bh * bh;
    prev = h->h_ranks[t];
  }
  if (with_T) f += (double)h->k * h->k * (double)(h->n - h->k);
  return f;
}

}  // namespace rbrp

using namespace rbrp;

namespace rbrp {
// Fixed-skeleton ID: the adaptive loop with the sampler replaced by "the next
// b columns of S" and a filter that keeps every nonzero pivot, so the run ends
// with S (reordered by the panel pivots) in perm[:k] and T = R11^{-1} R12 =
// A(:, S)^+ A(:, rd).
template <typename T>
rbrp_status fixed_id(rbrp_handle h, int m, int n, const T* dA, int64_t lda, const int* dS, int k, int b,
                            int* dPerm, rbrp_result* out) {
  rbrp_params p;
  rbrp_params_default(&p);
  p.b = b;
  p.tol = 0.0;
  p.kmax = k;
  p.tol_loc = 1e-300;  // keep every pivot with a positive Schur diagonal
  p.compute_T = 1;
  rbrp_status s = validate(h, m, n, dA, lda, &p, sizeof(T));
  if (s != RBRP_OK) return s;
  if (!dS || k < 1 || k > std::min(m, n)) return set_error(h, RBRP_ERR_INVALID_ARG, "need 1 <= k <= min(m, n) and S");
  if (dPerm && (s = check_device_ptr(h, dPerm, "perm")) != RBRP_OK) return s;
  if ((s = check_device_ptr(h, dS, "S")) != RBRP_OK) return s;
  DeviceGuard g(h->device);
  std::vector<int> S(k), order(n, -1);
  s = cuda_check(h, cudaMemcpy(S.data(), dS, sizeof(int) * (size_t)k, cudaMemcpyDeviceToHost), "copy S");
  if (s != RBRP_OK) return s;
  for (int t = 0; t < k; ++t) {
    if (S[t] < 0 || S[t] >= n) return set_error(h, RBRP_ERR_INVALID_ARG, "skeleton index out of range");
    if (order[S[t]] >= 0) return set_error(h, RBRP_ERR_INVALID_ARG, "repeated skeleton index");
    order[S[t]] = t;
  }
  if (h->given_cap < (size_t)n) {
    if (h->given_order) cudaFree(h->given_order);
    h->given_order = nullptr;
    h->given_cap = 0;
    s = cuda_check(h, cudaMalloc((void**)&h->given_order, sizeof(int) * (size_t)n), "cudaMalloc(skeleton order)");
    if (s != RBRP_OK) return s;
    h->given_cap = n;
  }
  s = cuda_check(h, cudaMemcpyAsync(h->given_order, order.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice,
                                    h->stream), "copy skeleton order");
  if (s != RBRP_OK) return s;
  p.sampler = SAMPLER_GIVEN;
  // the handle's projection variant (tcgen05 by default): on the 8192^2 Gaussian-kernel
  // adjoint workload the loss and dL/dA agree with FP64 as closely as with the CUDA-core one
  s = run_rbrp<T>(h, m, n, dA, lda, p, dPerm, out);
  // the host vector is released on return: finish the copy before that
  const rbrp_status s2 = cuda_check(h, cudaStreamSynchronize(h->stream), "fixed-skeleton run");
  return s != RBRP_OK ? s : s2;
}

}  // namespace rbrp


extern "C" {

void rbrp_params_default(rbrp_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->tol = 1e-12;
  p->b = 64;
  p->kmax = 0;
  p->seed = 0;
  p->sampler = RBRP_SAMPLER_NP;
  p->precision = RBRP_PREC_F64;
  p->tol_loc = 0.0;
  p->compute_T = 1;
  p->recompute = 1;
}

int rbrp_abi_version(void) { return RBRP_GB300_ABI_VERSION; }

const char* rbrp_status_string(rbrp_status s) {
  switch (s) {
    case RBRP_OK: return "ok";
    case RBRP_ERR_INVALID_ARG: return "invalid argument";
    case RBRP_ERR_CUDA: return "CUDA error";
    case RBRP_ERR_ALLOC: return "allocation failed";
    case RBRP_ERR_NOT_COMPUTED: return "no result computed";
    case RBRP_ERR_NUMERIC: return "numerical failure";
    case RBRP_ERR_CAPACITY: return "buffer too small";
    case RBRP_ERR_DEVICE_TIMEOUT: return "device wait timed out";
  }
  return "unknown status";
}

const char* rbrp_last_error(rbrp_handle h) { return h ? h->last_error.c_str() : "null handle"; }

rbrp_status rbrp_create(rbrp_handle* out, int device) {
  if (!out) return RBRP_ERR_INVALID_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return RBRP_ERR_CUDA;
  }
  if (device < 0 || device >= ndev) return RBRP_ERR_INVALID_ARG;
  rbrp_handle h = new (std::nothrow) rbrp_handle_st();
  if (!h) return RBRP_ERR_ALLOC;
  h->device = device;
  DeviceGuard g(device);
  if (!g.ok || cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      cudaEventCreate(&h->ev_start) != cudaSuccess || cudaEventCreate(&h->ev_loop) != cudaSuccess ||
      cudaEventCreate(&h->ev_end) != cudaSuccess) {
    cudaGetLastError();
    delete h;
    return RBRP_ERR_CUDA;
  }
  *out = h;
  return RBRP_OK;
}

rbrp_status rbrp_destroy(rbrp_handle h) {
  if (!h) return RBRP_ERR_INVALID_ARG;
  {
    DeviceGuard g(h->device);
    if (h->ws) cudaFree(h->ws);
    if (h->T) cudaFree(h->T);
    if (h->df_buf) cudaFree(h->df_buf);
    if (h->hostA_dev) cudaFree(h->hostA_dev);
    if (h->given_order) cudaFree(h->given_order);
    if (h->adj_ws) cudaFree(h->adj_ws);
    if (h->sketch_ws) cudaFree(h->sketch_ws);
    if (h->lupp_ws) cudaFree(h->lupp_ws);
    if (h->md_ws) cudaFree(h->md_ws);
    if (h->md_aux) cudaFree(h->md_aux);
    if (h->hst) cudaFreeHost(h->hst);
    for (auto e : h->block_events) cudaEventDestroy(e);
    for (auto e : h->prof_events) cudaEventDestroy(e);
    if (h->ev_start) cudaEventDestroy(h->ev_start);
    if (h->ev_loop) cudaEventDestroy(h->ev_loop);
    if (h->ev_end) cudaEventDestroy(h->ev_end);
    batch_release(h);
  }
  delete h;
  return RBRP_OK;
}

rbrp_status rbrp_set_stream(rbrp_handle h, void* stream) {
  if (!h) return RBRP_ERR_INVALID_ARG;
  h->stream = static_cast<cudaStream_t>(stream);
  return RBRP_OK;
}

rbrp_status rbrp_id_f64(rbrp_handle h, int m, int n, const double* dA, int64_t lda, const rbrp_params* p,
                        int* dPerm, rbrp_result* out) {
  rbrp_status s = validate(h, m, n, dA, lda, p, sizeof(double));
  if (s != RBRP_OK) return s;
  if (dPerm && (s = check_device_ptr(h, dPerm, "perm")) != RBRP_OK) return s;
  DeviceGuard g(h->device);
  return run_rbrp<double>(h, m, n, dA, lda, *p, dPerm, out);
}

rbrp_status rbrp_id_f32(rbrp_handle h, int m, int n, const float* dA, int64_t lda, const rbrp_params* p,
                        int* dPerm, rbrp_result* out) {
  rbrp_status s = validate(h, m, n, dA, lda, p, sizeof(float));
  if (s != RBRP_OK) return s;
  if (dPerm && (s = check_device_ptr(h, dPerm, "perm")) != RBRP_OK) return s;
  DeviceGuard g(h->device);
  return run_rbrp<float>(h, m, n, dA, lda, *p, dPerm, out);
}

rbrp_status rbrp_fixed_id_f32(rbrp_handle h, int m, int n, const float* dA, int64_t lda, const int* dS, int k, int b,
                              int* dPerm, rbrp_result* out) {
  return fixed_id<float>(h, m, n, dA, lda, dS, k, b, dPerm, out);
}

rbrp_status rbrp_fixed_id_f64(rbrp_handle h, int m, int n, const double* dA, int64_t lda, const int* dS, int k,
                              int b, int* dPerm, rbrp_result* out) {
  return fixed_id<double>(h, m, n, dA, lda, dS, k, b, dPerm, out);
}

rbrp_status rbrp_copy_T(rbrp_handle h, double* dT, int64_t ldt) {
  if (!h) return RBRP_ERR_INVALID_ARG;
  if (!h->have_result) return set_error(h, RBRP_ERR_NOT_COMPUTED, "no successful run");
  const int k = h->k, nc = h->n - h->k;
  if (k == 0 || nc == 0) return RBRP_OK;
  if (!h->T) return set_error(h, RBRP_ERR_NOT_COMPUTED, "T was not computed (compute_T = 0)");
  if (!dT || ldt < k) return set_error(h, RBRP_ERR_INVALID_ARG, "dT is NULL or ldt < k");
  DeviceGuard g(h->device);
  return cuda_check(h, cudaMemcpy2DAsync(dT, ldt * sizeof(double), h->T, (size_t)k * sizeof(double),
                                         (size_t)k * sizeof(double), nc, cudaMemcpyDeviceToDevice, h->stream),
                    "copy T");
}

namespace rbrp {
namespace {
// L(perm[p], a) = R(a, p) for p >= a, else 0 (R: k x n row major by position, ld n).
__global__ void k_copy_L(const double* __restrict__ R, const int* __restrict__ perm, int n, int k,
                         double* __restrict__ L, int64_t ldl) {
  const int64_t total = (int64_t)n * k;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int a = (int)(idx / n), p = (int)(idx % n);
    L[(int64_t)perm[p] + (int64_t)a * ldl] = p >= a ? R[(int64_t)a * n + p] : 0.0;
  }
}
}  // namespace
}  // namespace rbrp

rbrp_status rbrp_copy_L(rbrp_handle h, double* dL, int64_t ldl) {
  if (!h) return RBRP_ERR_INVALID_ARG;
  if (!h->have_result) return set_error(h, RBRP_ERR_NOT_COMPUTED, "no successful run");
  const int k = h->k, n = h->n;
  if (k == 0 || n == 0) return RBRP_OK;
  if (!dL || ldl < n) return set_error(h, RBRP_ERR_INVALID_ARG, "dL is NULL or ldl < n");
  DeviceGuard g(h->device);
  const int64_t total = (int64_t)n * k;
  const int blocks = (int)std::min<int64_t>(4 * 1216, (total + 255) / 256);
  k_copy_L<<<blocks, 256, 0, h->stream>>>(h->R, h->perm, n, k, dL, ldl);
  return cuda_check(h, cudaGetLastError(), "copy L");
}

rbrp_status rbrp_T_device(rbrp_handle h, const double** dT, int* ld) {
  if (!h || !dT || !ld) return RBRP_ERR_INVALID_ARG;
  if (!h->have_result) return set_error(h, RBRP_ERR_NOT_COMPUTED, "no successful run");
  *dT = h->T;
  *ld = h->k;
  return RBRP_OK;
}

rbrp_status rbrp_get_trace(rbrp_handle h, int* ranks, double* errors, double* t_ms, int cap, int* nblocks) {
  if (!h || !nblocks) return RBRP_ERR_INVALID_ARG;
  if (!h->have_result) return set_error(h, RBRP_ERR_NOT_COMPUTED, "no successful run");
  const int nb = (int)h->h_ranks.size();
  *nblocks = nb;
  if (cap < nb && (ranks || errors || t_ms)) return set_error(h, RBRP_ERR_CAPACITY, "trace capacity too small");
  for (int t = 0; t < nb; ++t) {
    if (ranks) ranks[t] = h->h_ranks[t];
    if (errors) errors[t] = h->h_err[t];
    if (t_ms) t_ms[t] = h->h_tms[t];
  }
  return RBRP_OK;
}

rbrp_status rbrp_id_error_f64(rbrp_handle h, int m, int n, const double* dA, int64_t lda, double* err) {
  if (!h || !err || !dA) return RBRP_ERR_INVALID_ARG;
  if (!h->have_result) return set_error(h, RBRP_ERR_NOT_COMPUTED, "no successful run");
  if (m != h->m || n != h->n || lda < m) return set_error(h, RBRP_ERR_INVALID_ARG, "shape differs from the last run");
  if (h->k > 0 && h->k < n && !h->T) return set_error(h, RBRP_ERR_NOT_COMPUTED, "T was not computed");
  DeviceGuard g(h->device);
  return id_error<double>(h, m, n, dA, lda, err);
}

rbrp_status rbrp_id_error_f32(rbrp_handle h, int m, int n, const float* dA, int64_t lda, double* err) {
  if (!h || !err || !dA) return RBRP_ERR_INVALID_ARG;
  if (!h->have_result) return set_error(h, RBRP_ERR_NOT_COMPUTED, "no successful run");
  if (m != h->m || n != h->n || lda < m) return set_error(h, RBRP_ERR_INVALID_ARG, "shape differs from the last run");
  if (h->k > 0 && h->k < n && !h->T) return set_error(h, RBRP_ERR_NOT_COMPUTED, "T was not computed");
  DeviceGuard g(h->device);
  return id_error<float>(h, m, n, dA, lda, err);
}

rbrp_status rbrp_id_f64_host(rbrp_handle h, int m, int n, const double* hA, int64_t lda, const rbrp_params* p,
                             int* hPerm, double* hT, int64_t ldt, int64_t t_cap, rbrp_result* out) {
  return host_run<double>(h, m, n, hA, lda, p, hPerm, hT, ldt, t_cap, out);
}

rbrp_status rbrp_id_f32_host(rbrp_handle h, int m, int n, const float* hA, int64_t lda, const rbrp_params* p,
                             int* hPerm, double* hT, int64_t ldt, int64_t t_cap, rbrp_result* out) {
  return host_run<float>(h, m, n, hA, lda, p, hPerm, hT, ldt, t_cap, out);
}

rbrp_status rbrp_set_profiling(rbrp_handle h, int on) {
  if (!h) return RBRP_ERR_INVALID_ARG;
  h->profiling = on != 0;
  return RBRP_OK;
}

rbrp_status rbrp_get_phase_stats(rbrp_handle h, rbrp_phase_stats* out) {
  if (!h || !out) return RBRP_ERR_INVALID_ARG;
  *out = h->stats;
  return RBRP_OK;
}

rbrp_status rbrp_reset_phase_stats(rbrp_handle h) {
  if (!h) return RBRP_ERR_INVALID_ARG;
  std::memset(&h->stats, 0, sizeof(h->stats));
  return RBRP_OK;
}

rbrp_status rbrp_set_variant(rbrp_handle h, int variant) {
  if (!h || variant < 0 || variant > 1) return RBRP_ERR_INVALID_ARG;
  h->variant = variant;
  return RBRP_OK;
}

rbrp_status rbrp_set_wait_budget(rbrp_handle h, long long cycles) {
  if (!h || cycles < 0) return RBRP_ERR_INVALID_ARG;
  h->wait_budget = cycles;
  return RBRP_OK;
}

rbrp_status rbrp_set_tsolve_fp64(rbrp_handle h, int on) {
  if (!h) return RBRP_ERR_INVALID_ARG;
  h->tsolve_fp64 = on != 0;
  return RBRP_OK;
}

rbrp_status rbrp_RBRP(int m, int n, double* dA, int blk, int* ranks, double* error, double* t_ranks, int cap,
                      int* nblocks, double* t_rbrp, double* flops) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return RBRP_ERR_CUDA;
  rbrp_handle h = nullptr;
  rbrp_status s = rbrp_create(&h, dev);
  if (s != RBRP_OK) return s;
  rbrp_params p;
  rbrp_params_default(&p);
  p.b = blk;
  p.tol = 0.0;  // the reference loop runs to min(m, n) (gpu/rbrp.cu:361,367)
  p.compute_T = 0;
  rbrp_result r;
  s = rbrp_id_f64(h, m, n, dA, m, &p, nullptr, &r);
  if (s == RBRP_OK) {
    int nb = 0;
    s = rbrp_get_trace(h, ranks, error, t_ranks, cap, &nb);
    if (nblocks) *nblocks = nb;
    if (t_ranks)
      for (int t = 0; t < nb && t < cap; ++t) t_ranks[t] *= 1e-3;
    if (t_rbrp) *t_rbrp = r.ms_total * 1e-3;
    if (flops) *flops = run_flops(h, false);
  }
  rbrp_destroy(h);
  return s;
}

rbrp_status rbrp_RandAdapRBRP(const double* dA, int m, int n, int** sk, int** rd, double** T, int* rank,
                              double* flops, double tol, int blk) {
  if (!sk || !rd || !T || !rank) return RBRP_ERR_INVALID_ARG;
  *sk = nullptr;
  *rd = nullptr;
  *T = nullptr;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return RBRP_ERR_CUDA;
  rbrp_handle h = nullptr;
  rbrp_status s = rbrp_create(&h, dev);
  if (s != RBRP_OK) return s;
  rbrp_params p;
  rbrp_params_default(&p);
  p.b = blk;
  p.tol = tol;
  rbrp_result r;
  s = rbrp_id_f64(h, m, n, dA, m, &p, nullptr, &r);
  if (s == RBRP_OK) {
    const int k = r.k, nc = n - k;
    *rank = k;
    if (cudaMalloc((void**)sk, sizeof(int) * (size_t)(k > 0 ? k : 1)) != cudaSuccess ||
        cudaMalloc((void**)rd, sizeof(int) * (size_t)(nc > 0 ? nc : 1)) != cudaSuccess ||
        cudaMalloc((void**)T, sizeof(double) * (size_t)(k > 0 && nc > 0 ? (size_t)k * nc : 1)) != cudaSuccess) {
      cudaGetLastError();
      if (*sk) cudaFree(*sk);
      if (*rd) cudaFree(*rd);
      if (*T) cudaFree(*T);
      *sk = nullptr;
      *rd = nullptr;
      *T = nullptr;
      s = RBRP_ERR_ALLOC;
    } else {
      cudaMemcpy(*sk, h->perm, sizeof(int) * (size_t)k, cudaMemcpyDeviceToDevice);
      cudaMemcpy(*rd, h->perm + k, sizeof(int) * (size_t)nc, cudaMemcpyDeviceToDevice);
      if (k > 0 && nc > 0) cudaMemcpy(*T, h->T, sizeof(double) * (size_t)k * nc, cudaMemcpyDeviceToDevice);
      if (flops) *flops = run_flops(h, true);
      if (cudaDeviceSynchronize() != cudaSuccess) s = RBRP_ERR_CUDA;
    }
  }
  rbrp_destroy(h);
  return s;
}

rbrp_status rbrp_free(void* dptr) {
  if (!dptr) return RBRP_OK;
  return cudaFree(dptr) == cudaSuccess ? RBRP_OK : RBRP_ERR_CUDA;
}

}  // extern "C"
