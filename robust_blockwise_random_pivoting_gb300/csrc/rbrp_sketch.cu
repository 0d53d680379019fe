// rbrp_sketch.cu - Gaussian sketch Y = G A for the sketch-based comparison IDs.
//
// The reference's oversampled randomized IDs (gpu/randCPQR_OS.cu:20-111,
// gpu/randLUPP_OS.cu:14-119) draw G (l x m, entries N(0, 1/m)) and form
// Y = G A with cuBLAS (gpu/gemm.cu:9-15, gpu/random.cu).  Here G comes from
// Philox4x64-10 (key {seed, 0}, counter {e / 8, 0x534B, 0, 0} for entries
// e .. e+7 of G in column-major order) through the Box-Muller transform, and
// the product is the 128 x 128-tiled FP32 CUDA-core GEMM of rbrp_gemm.cuh.
#include "rbrp_internal.h"
#include "rbrp_gemm.cuh"

namespace rbrp {
namespace {

constexpr uint64_t SKETCH_TAG = 0x534Bull;

// G[e] = scale * N(0, 1) for e < count, eight entries per thread and Philox call:
// each 64-bit word gives one Box-Muller pair from two 24-bit uniforms in (0, 1].
__global__ void k_gauss_fill(float* __restrict__ G, int64_t count, uint64_t seed, float scale) {
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g * 8 < count;
       g += (int64_t)gridDim.x * blockDim.x) {
    uint64_t c[4] = {(uint64_t)g, SKETCH_TAG, 0ull, 0ull};
    philox4x64_10(c, seed, 0ull);
#pragma unroll
    for (int w = 0; w < 4; ++w) {
      const float u1 = (float)((c[w] >> 40) + 1ull) * 0x1.0p-24f;           // (0, 1]
      const float u2 = (float)((c[w] >> 16) & 0xFFFFFFull) * 0x1.0p-24f;    // [0, 1)
      const float rad = sqrtf(-2.0f * logf(u1));
      float sn, cs;
      sincospif(2.0f * u2, &sn, &cs);
      const int64_t e = g * 8 + 2 * w;
      if (e < count) G[e] = scale * rad * cs;
      if (e + 1 < count) G[e + 1] = scale * rad * sn;
    }
  }
}

// Y (l x n, ld ldy) = G (l x m, ld l) A (m x n, ld lda), one 128 x 128 tile per CTA.
__global__ void __launch_bounds__(GT) k_sketch_gemm(const float* __restrict__ G, int l, int m, const float* __restrict__ A,
                                                    int64_t lda, int n, float* __restrict__ Y, int64_t ldy) {
  __shared__ GemmSmem sm;
  const int r0 = blockIdx.x * GTILE, c0 = blockIdx.y * GTILE;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  float acc[8][8];
  gemm_tile<LoadColMajorX, LoadColMajorY, true>(sm, LoadColMajorX{G, l, l, m}, LoadColMajorY{A, lda, m, n}, m, r0,
                                                c0, acc);
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int c = c0 + tile_col(tx, j);
    if (c >= n) continue;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int r = r0 + tile_row(ty, i);
      if (r < l) Y[r + (int64_t)c * ldy] = acc[i][j];
    }
  }
}

}  // namespace
}  // namespace rbrp

using namespace rbrp;

extern "C" rbrp_status rbrp_sketch_gaussian_f32(rbrp_handle h, int l, int m, int n, const float* dA, int64_t lda,
                                                uint64_t seed, float scale, float* dY, int64_t ldy) {
  if (!h) return RBRP_ERR_INVALID_ARG;
  if (l < 1 || m < 1 || n < 1 || lda < m || ldy < l || !dA || !dY)
    return set_error(h, RBRP_ERR_INVALID_ARG, "bad sketch shape or pointer");
  DeviceGuard g(h->device);
  const size_t bytes = (size_t)l * (size_t)m * sizeof(float);
  if (h->sketch_bytes < bytes) {
    if (h->sketch_ws) cudaFree(h->sketch_ws);
    h->sketch_ws = nullptr;
    h->sketch_bytes = 0;
    rbrp_status s = cuda_check(h, cudaMalloc(&h->sketch_ws, bytes), "cudaMalloc(sketch matrix)");
    if (s != RBRP_OK) return s;
    h->sketch_bytes = bytes;
  }
  float* G = static_cast<float*>(h->sketch_ws);
  const int64_t count = (int64_t)l * m;
  const int64_t groups = (count + 7) / 8;
  const int blocks = (int)std::min<int64_t>(4864, (groups + 255) / 256);
  k_gauss_fill<<<blocks, 256, 0, h->stream>>>(G, count, seed, scale);
  k_sketch_gemm<<<dim3((l + GTILE - 1) / GTILE, (n + GTILE - 1) / GTILE), GT, 0, h->stream>>>(G, l, m, dA, lda, n, dY,
                                                                                             ldy);
  return cuda_check(h, cudaGetLastError(), "sketch kernels");
}
