// rbrp_sketch.cu - Gaussian sketch Y = G A for the sketch-based comparison IDs.
//
// The reference's oversampled randomized IDs (gpu/randCPQR_OS.cu:20-111,
// gpu/randLUPP_OS.cu:14-119) draw G (l x m, entries N(0, 1/m)) and form
// Y = G A with cuBLAS (gpu/gemm.cu:9-15, gpu/random.cu).  Here G comes from
// Philox4x64-10 (key {seed, 0}, counter {e / 8, 0x534B, 0, 0} for entries
// e .. e+7 of G in column-major order) through the Box-Muller transform.  The
// product runs on the tensor cores through the general tcgen05 3xTF32 GEMM of
// rbrp_gemm_tc.cuh: A is the TMA-fed operand (128 of its columns per CTA, split
// into TF32 hi + lo parts in shared memory), G^T the pre-split one (k_gt_split
// writes its hi and lo parts, K-major), and the epilogue stores the 128 x 64
// tile of Y.  An A whose leading dimension or base is not 16-byte aligned cannot
// be described by a tensor map; it takes the 128 x 128-tiled FP32 CUDA-core
// GEMM of rbrp_gemm.cuh.
#include "rbrp_internal.h"
#include "rbrp_gemm.cuh"
#include "rbrp_gemm_tc.cuh"

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

// Gt (m x l, ld mp) hi and lo TF32 parts of G^T (tf32_split), through a 32 x 32
// shared tile so both sides are coalesced.
__global__ void k_gt_split(const float* __restrict__ G, int l, int m, int64_t mp, float* __restrict__ Gth,
                           float* __restrict__ Gtl) {
  __shared__ float tile[32][33];
  const int r0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 256 threads: 8 rows of 32
  for (int y = ty; y < 32; y += 8) {
    const int r = r0 + tx, kc = k0 + y;
    tile[y][tx] = (r < l && kc < m) ? G[r + (int64_t)kc * l] : 0.f;
  }
  __syncthreads();
  for (int y = ty; y < 32; y += 8) {
    const int kc = k0 + tx, r = r0 + y;
    if (r < l && kc < m) {
      float hi, lo;
      tf32_split(tile[tx][y], hi, lo);
      Gth[kc + (int64_t)r * mp] = hi;
      Gtl[kc + (int64_t)r * mp] = lo;
    }
  }
}

// Y(r, c) for the tile's sketch rows r = r0 .. r0 + 31 of column c of A.
struct EpiY {
  float* Y;
  int64_t ldy;
  int l, n;
  bool vec;  // Y and ldy 16-byte aligned: float4 stores
  __device__ void operator()(int c, int r0, const float (&hi)[32], const float (&lo)[32], int) const {
    if (c >= n || r0 >= l) return;
    float* y = Y + r0 + (int64_t)c * ldy;
    if (vec && r0 + 32 <= l) {
#pragma unroll
      for (int j = 0; j < 32; j += 4)
        *reinterpret_cast<float4*>(y + j) =
            make_float4(hi[j] + lo[j], hi[j + 1] + lo[j + 1], hi[j + 2] + lo[j + 2], hi[j + 3] + lo[j + 3]);
    } else {
#pragma unroll
      for (int j = 0; j < 32; ++j)
        if (r0 + j < l) y[j] = hi[j] + lo[j];
    }
  }
  __device__ void finish(bool) const {}
};

}  // namespace
}  // namespace rbrp

using namespace rbrp;

extern "C" rbrp_status rbrp_sketch_gaussian_f32(rbrp_handle h, int l, int m, int n, const float* dA, int64_t lda,
                                                uint64_t seed, float scale, float* dY, int64_t ldy) {
  if (!h) return RBRP_ERR_INVALID_ARG;
  if (l < 1 || m < 1 || n < 1 || lda < m || ldy < l || !dA || !dY)
    return set_error(h, RBRP_ERR_INVALID_ARG, "bad sketch shape or pointer");
  DeviceGuard g(h->device);
  // the tensor-core GEMM needs a tensor map of A: 16-byte aligned base and leading dimension
  const bool tc_ok = (lda % 4) == 0 && (reinterpret_cast<uintptr_t>(dA) & 15) == 0;
  const int64_t mp = ((int64_t)m + 3) / 4 * 4;
  const size_t gbytes = ((size_t)l * (size_t)m * sizeof(float) + 255) & ~(size_t)255;
  const size_t tbytes = ((size_t)l * (size_t)mp * sizeof(float) + 255) & ~(size_t)255;
  const size_t bytes = gbytes + (tc_ok ? 2 * tbytes + 256 : 0);
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
  if (!tc_ok) {
    k_sketch_gemm<<<dim3((l + GTILE - 1) / GTILE, (n + GTILE - 1) / GTILE), GT, 0, h->stream>>>(G, l, m, dA, lda, n,
                                                                                               dY, ldy);
    return cuda_check(h, cudaGetLastError(), "sketch kernels");
  }
  char* base = static_cast<char*>(h->sketch_ws) + gbytes;
  float* Gth = reinterpret_cast<float*>(base);
  float* Gtl = reinterpret_cast<float*>(base + tbytes);
  int* dstatus = reinterpret_cast<int*>(base + 2 * tbytes);
  if (!h->smem_attr_sketch_tc) {
    rbrp_status s = cuda_check(h, cudaFuncSetAttribute(tc::k_gemm_tc<EpiY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       (int)tc::GEMM_SMEM), "cudaFuncSetAttribute(k_gemm_tc<Y>)");
    if (s != RBRP_OK) return s;
    h->smem_attr_sketch_tc = true;
  }
  CUtensorMap tmA, tmGh, tmGl;
  rbrp_status s = make_tmap_f32(h, &tmA, dA, m, n, lda, tc::BK, tc::BM);
  if (s == RBRP_OK) s = make_tmap_f32(h, &tmGh, Gth, m, l, mp, tc::BK, tc::BN);
  if (s == RBRP_OK) s = make_tmap_f32(h, &tmGl, Gtl, m, l, mp, tc::BK, tc::BN);
  if (s == RBRP_OK) s = cuda_check(h, cudaMemsetAsync(dstatus, 0, sizeof(int), h->stream), "clear status");
  if (s != RBRP_OK) return s;
  k_gt_split<<<dim3((l + 31) / 32, (m + 31) / 32), 256, 0, h->stream>>>(G, l, m, mp, Gth, Gtl);
  const bool vec = (ldy % 4) == 0 && (reinterpret_cast<uintptr_t>(dY) & 15) == 0;
  EpiY epi{dY, ldy, l, n, vec};
  const long long budget = h->wait_budget > 0 ? h->wait_budget : kWaitBudgetDefault;
  tc::k_gemm_tc<EpiY><<<dim3((n + tc::BM - 1) / tc::BM, (l + tc::BN - 1) / tc::BN), tc::NTHREADS, tc::GEMM_SMEM,
                        h->stream>>>(tmA, tmGh, tmGl, n, l, m, budget, dstatus, epi);
  s = cuda_check(h, cudaGetLastError(), "sketch kernels");
  if (s != RBRP_OK) return s;
  int hs = 0;
  s = cuda_check(h, cudaMemcpyAsync(&hs, dstatus, sizeof(int), cudaMemcpyDeviceToHost, h->stream), "sketch status");
  if (s == RBRP_OK) s = cuda_check(h, cudaStreamSynchronize(h->stream), "sketch kernels");
  if (s != RBRP_OK) return s;
  if (hs == tc::ST_ERR_TIMEOUT)
    return set_error(h, RBRP_ERR_DEVICE_TIMEOUT, "a device-side wait of the sketch GEMM timed out; it aborted cleanly");
  return RBRP_OK;
}
