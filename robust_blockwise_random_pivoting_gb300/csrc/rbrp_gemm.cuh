// rbrp_gemm.cuh - 128 x 128-tile FP32 GEMM building block (CUDA cores) with
// pluggable operand loaders, shared by the adjoint and sketch kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace rbrp {
namespace {

constexpr int GT = 256;        // threads of a GEMM CTA
constexpr int GTILE = 128;     // output tile edge
constexpr int GK = 16;         // contraction chunk

// 128 x 128 FP32 GEMM tile: acc[8][8] += X(r0:r0+128, :) Y(:, c0:c0+128), the
// contraction in chunks of 16 staged through double-buffered shared memory.
// Thread (ty, tx) = (tid / 16, tid % 16) owns rows ty*4 + {0..3} and
// 64 + ty*4 + {0..3}, columns tx*4 + {0..3} and 64 + tx*4 + {0..3}.
struct GemmSmem {
  __align__(16) float X[2][GK][GTILE + 4];  // X[kk][row]
  __align__(16) float Y[2][GK][GTILE + 4];  // Y[kk][col]
};

// Loaders return one staged element for (chunk-relative kk, tile-relative index).
struct LoadC {  // X = C: C[r][t] = A[r + perm[t] lda]
  const float* A;
  int64_t lda;
  const int* perm;
  int m, K;
  __device__ __forceinline__ float x(int r, int t) const {
    return (r < m && t < K) ? A[r + (int64_t)perm[t] * lda] : 0.f;
  }
};
struct LoadE {  // X = E (m x nc, column major, ld m)
  const float* E;
  int m, K;
  __device__ __forceinline__ float x(int r, int c) const { return (r < m && c < K) ? E[r + (int64_t)c * m] : 0.f; }
};
struct LoadColMajorX {  // X (M x K, column major, ld)
  const float* X;
  int64_t ld;
  int M, K;
  __device__ __forceinline__ float x(int r, int kk) const {
    return (r < M && kk < K) ? X[r + (int64_t)kk * ld] : 0.f;
  }
};
struct LoadColMajorY {  // Y (K x N, column major, ld): stage with YKF = true
  const float* Y;
  int64_t ld;
  int K, N;
  __device__ __forceinline__ float y(int kk, int c) const {
    return (kk < K && c < N) ? Y[kk + (int64_t)c * ld] : 0.f;
  }
};
struct LoadRowMajor {  // Y[kk][col] from a row-major K x N matrix
  const float* Y;
  int K, N;
  __device__ __forceinline__ float y(int kk, int c) const {
    return (kk < K && c < N) ? Y[(int64_t)kk * N + c] : 0.f;
  }
};

// YKF: the Y operand is staged with the contraction index fastest across
// threads (for a column-major Y whose contraction runs down its columns);
// otherwise the tile index is fastest for both operands.
template <class LX, class LY, bool YKF = false>
__device__ __forceinline__ void gemm_tile(GemmSmem& sm, const LX& lx, const LY& ly, int K, int r0, int c0,
                                          float (&acc)[8][8]) {
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  // staging: 16 x 128 values per operand, 8 per thread
  const int s_i = tid & 127, s_k = tid >> 7;    // tile index fastest: index, first kk (step 2)
  const int y_k = tid & 15, y_i = tid >> 4;     // contraction fastest: kk, first index (step 16)
  float xr[8], yr[8];
  auto load = [&](int k0) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int kk = s_k + 2 * q;
      xr[q] = lx.x(r0 + s_i, k0 + kk);
      yr[q] = YKF ? ly.y(k0 + y_k, c0 + y_i + 16 * q) : ly.y(k0 + kk, c0 + s_i);
    }
  };
  auto store = [&](int buf) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int kk = s_k + 2 * q;
      sm.X[buf][kk][s_i] = xr[q];
      if (YKF)
        sm.Y[buf][y_k][y_i + 16 * q] = yr[q];
      else
        sm.Y[buf][kk][s_i] = yr[q];
    }
  };
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
  const int nchunk = (K + GK - 1) / GK;
  load(0);
  store(0);
  __syncthreads();
  for (int ch = 0; ch < nchunk; ++ch) {
    const int buf = ch & 1;
    if (ch + 1 < nchunk) load((ch + 1) * GK);
#pragma unroll
    for (int kk = 0; kk < GK; ++kk) {
      const float4 a0 = *reinterpret_cast<const float4*>(&sm.X[buf][kk][ty * 4]);
      const float4 a1 = *reinterpret_cast<const float4*>(&sm.X[buf][kk][64 + ty * 4]);
      const float4 b0 = *reinterpret_cast<const float4*>(&sm.Y[buf][kk][tx * 4]);
      const float4 b1 = *reinterpret_cast<const float4*>(&sm.Y[buf][kk][64 + tx * 4]);
      const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
    }
    if (ch + 1 < nchunk) store(buf ^ 1);
    __syncthreads();
  }
}

__device__ __forceinline__ int tile_row(int ty, int i) { return (i < 4 ? 0 : 64) + ty * 4 + (i & 3); }
__device__ __forceinline__ int tile_col(int tx, int j) { return (j < 4 ? 0 : 64) + tx * 4 + (j & 3); }


}  // namespace
}  // namespace rbrp
