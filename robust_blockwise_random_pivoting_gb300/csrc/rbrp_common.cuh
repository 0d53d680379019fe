// rbrp_common.cuh - device-side definitions shared by the RBRP kernels.
//
// Layout in HBM (one problem; all arrays owned by the handle's workspace):
//   A      m x n, column major, caller owned, never moved (columns reached
//          through perm; the reference copies and physically swaps columns,
//          gpu/rbrp.cu:337-338, 247-267).
//   perm   n int32: position -> original column.
//   diags  n FP64, indexed by POSITION (matlab/RBRP.m:99 swaps them like perm).
//   Q      m x kmax, column major (ld = m), element type of A.
//   R      kmax x n FP64, ROW major (ld = n), indexed by position; rows of block
//          t hold Q_t^T A(:, perm[p]) for the positions p remaining at block t
//          and the panel R on the diagonal block (matlab/RBRP.m:78,103).
//   V, Q1  m x MAXB FP64 panel buffers (column major, ld = m).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace rbrp {

constexpr int MAXB = 64;          // largest block size b supported by the panel kernels
constexpr int SAMPLER_NP = 0;
constexpr int SAMPLER_ES = 1;
constexpr int SAMPLER_GREEDY = 2;
constexpr int SAMPLER_GIVEN = 3;  // fixed skeleton: the next columns of a given list, in list order
constexpr int ST_ERR_NUMERIC = 5; // mirrors RBRP_ERR_NUMERIC

// Loop state, resident in device memory; every per-block kernel reads it, so the
// host needs no data from the device to enqueue a block.
struct State {
  int i;            // rank so far = first position of the current block
  int bs_sampled;   // columns sampled in this block
  int bs;           // columns kept by the robust filter in this block
  int done;         // 1 once the loop has stopped
  int nnz_rem;      // positions >= i with positive residual weight
  int nblocks;      // blocks completed (each kept >= 1 column)
  int status;       // 0 or ST_ERR_NUMERIC
  int zero_panel;   // the filter kept nothing in this block
  int nK;           // |K1| = |K2| of the block swap
  int recomputes;
  int attempts;     // block attempts (also counts zero panels): exponential-key stream index
  unsigned long long draws;  // uniforms consumed from the np-compat stream
  double res0;      // ||A||_F^2
  double residual;  // sum of diags over remaining positions
};

// ---------------------------------------------------------------------------
// Philox4x64-10 (Salmon et al., SC'11).  np-compat stream: uniform t is word
// t%4 of philox(ctr = {1 + t/4, 0, 0, 0}, key = {seed, 0}), >> 11, * 2^-53,
// which is numpy's Philox(key=seed) next_double.
// ---------------------------------------------------------------------------
constexpr uint64_t PHILOX_M0 = 0xD2E7470EE14C6C93ull;
constexpr uint64_t PHILOX_M1 = 0xCA5A826395121157ull;
constexpr uint64_t PHILOX_W0 = 0x9E3779B97F4A7C15ull;
constexpr uint64_t PHILOX_W1 = 0xBB67AE8584CAA73Bull;
constexpr uint64_t ES_TAG = 0x4553ull;

__device__ __forceinline__ void philox4x64_10(uint64_t c[4], uint64_t k0, uint64_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) { k0 += PHILOX_W0; k1 += PHILOX_W1; }
    const uint64_t lo0 = PHILOX_M0 * c[0], hi0 = __umul64hi(PHILOX_M0, c[0]);
    const uint64_t lo1 = PHILOX_M1 * c[2], hi1 = __umul64hi(PHILOX_M1, c[2]);
    const uint64_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
  }
}

__device__ __forceinline__ double u64_to_unit(uint64_t x) {
  return (double)(x >> 11) * 0x1.0p-53;
}

__device__ __forceinline__ double np_uniform(uint64_t seed, uint64_t t) {
  uint64_t c[4] = {1ull + (t >> 2), 0ull, 0ull, 0ull};
  philox4x64_10(c, seed, 0ull);
  return u64_to_unit(c[t & 3]);
}

// exponential-key stream: original column col of block blk
__device__ __forceinline__ double es_uniform(uint64_t seed, uint64_t blk, uint64_t col) {
  uint64_t c[4] = {1ull + (col >> 2), blk + 1ull, ES_TAG, 0ull};
  philox4x64_10(c, seed, 0ull);
  return u64_to_unit(c[col & 3]);
}

// ---------------------------------------------------------------------------
// reductions (fixed order, so results are run-to-run deterministic)
// ---------------------------------------------------------------------------
template <typename V>
__device__ __forceinline__ V warp_sum(V v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum; every thread gets the result.  sh: >= 32 elements.
template <typename V>
__device__ V block_sum(V v, V* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  if (wid == 0) {
    V x = lane < nw ? sh[lane] : V(0);
    x = warp_sum(x);
    if (lane == 0) sh[0] = x;
  }
  __syncthreads();
  V r = sh[0];
  __syncthreads();
  return r;
}

// Block-wide exclusive prefix sum of one value per thread; *total gets the sum.
template <typename V>
__device__ V block_exclusive_scan(V v, V* sh, V* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  V x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    V y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  __syncthreads();
  if (lane == 31) sh[wid] = x;
  __syncthreads();
  if (wid == 0) {
    V w = lane < nw ? sh[lane] : V(0);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      V y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    sh[lane] = w;  // inclusive scan of warp totals
  }
  __syncthreads();
  V off = wid ? sh[wid - 1] : V(0);
  if (total) *total = sh[nw - 1];
  __syncthreads();
  V excl = __shfl_up_sync(0xffffffffu, x, 1);  // exclusive prefix within the warp
  if (lane == 0) excl = V(0);
  (void)v;
  return off + excl;
}

// FP32 double-float accumulator (Knuth TwoSum + exact products by FMA): sums
// squares of FP32 data to ~FP64 accuracy on the FP32 pipe, which on GB300 is
// far wider than the FP64 pipe.
struct DF {
  float hi, lo;
};
__device__ __forceinline__ void df_add_sq(DF& s, float x) {
  const float p = x * x;
  const float pe = fmaf(x, x, -p);
  const float t = s.hi + p;
  const float bb = t - s.hi;
  const float e = (s.hi - (t - bb)) + (p - bb);
  s.hi = t;
  s.lo += e + pe;
}

// x rounded to the nearest TF32 value (ties away from zero) for finite x below
// 2^127: adding half a TF32 ulp to the bit pattern carries into the kept bits
// exactly when the dropped part is at least half an ulp.
__device__ __forceinline__ float tf32_rn(float x) {
  return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}
// The operand split of the tensor cores' 3xTF32 / 4xTF32 products: hi =
// tf32_rn(x) and lo = tf32_rn(x - hi) (x - hi is exact), both TF32 values, so the
// tensor core reads them without loss and |x - hi - lo| <= 2^-23 |x|: a product
// of split operands is good to about an FP32 product's error.
__device__ __forceinline__ void tf32_split(float x, float& hi, float& lo) {
  hi = tf32_rn(x);
  lo = tf32_rn(x - hi);
}

}  // namespace rbrp
