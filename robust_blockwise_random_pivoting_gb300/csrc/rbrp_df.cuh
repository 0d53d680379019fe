// rbrp_df.cuh - double-float arithmetic on the FP32 pipe.
//
// A double-float is a pair of floats (hi + lo, ~48 significant bits).  Sums use
// Knuth's TwoSum, products the FMA-based exact product (error-free
// transformations), so FP64-class panel arithmetic runs on the FP32 pipe,
// which on GB300 issues ~64x the FP64 pipe's rate.
#pragma once
#include <cuda_runtime.h>

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
// acc + x * b for an FP32 x (an exact residual entry) and a double-float b
__device__ __forceinline__ dfl df_fma_f(dfl acc, float x, dfl b) {
  const float p = x * b.hi;
  float e = fmaf(x, b.hi, -p);
  e = fmaf(x, b.lo, e);
  const dfl t = df_two_sum(acc.hi, p);
  return df_fast(t.hi, t.lo + (acc.lo + e));
}
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

}  // namespace
}  // namespace rbrp
