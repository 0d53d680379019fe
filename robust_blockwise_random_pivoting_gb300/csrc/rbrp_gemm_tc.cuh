// rbrp_gemm_tc.cuh - a general tcgen05 / TMEM / TMA 3xTF32 GEMM with a
// pluggable epilogue (sm_103a), on the pipeline of the residual projection
// (rbrp_tc.cuh): D(p, c) = sum_k X(k, p) Y(k, c) for a tile of 128 values of p
// (the MMA M dimension, TMEM lanes, one CTA along gridDim.x) and 64 values of
// c (the MMA N dimension, one CTA along gridDim.y), reduced over all of k in
// stages of 32 (MMA K).
//
// Both operands are K-major FP32 in global memory: X (K x M, column major, ld
// a multiple of 4) and the hi and lo TF32 parts of Y (K x N each, same layout).
//
//   warp 0   TMA producer: the raw X tiles (128 x 32, 128-byte swizzled) into a
//            10-stage ring.
//   warp 1   MMA issuer: X hi Y hi into a large accumulator, X hi Y lo and
//            X lo Y hi into a small one (3xTF32: the FP32 product to ~2^-22); X is
//            read from tensor memory, Y from shared memory.
//   warps 2-5 split each X tile by tf32_split into tensor memory (one row per
//            thread), with two operand slots; the first split thread loads the
//            slot's Y hi / lo tiles (64 x 32).
//   warps 6-13 drain the large accumulator after every RBRP_GEMM_DRAIN stages
//            and the small one every CHUNK stages into double-float registers, then call the
//            epilogue: thread (lane quarter q, column half ch) holds
//            D(p0 + 32 q + lane, c0 + 32 ch + j) for j < 32.
//
// The tensor core rounds its FP32 accumulator once per MMA with a bias; draining
// every RBRP_GEMM_DRAIN stages keeps the rounding from growing with K: the sum
// stays FP32-accurate however long K is.  Every
// wait is bounded by `budget` clock64 cycles; on expiry the CTA sets an abort
// flag and *status, waits (default budget) for its own TMA copies and for the
// MMAs it issued, frees TMEM and returns without running the epilogue.
#pragma once
#include "rbrp_tc.cuh"

// Stages accumulated in the large accumulator between two drains (1, 2 or 4; CHUNK
// is a multiple): more MMAs per drain halve the drain work at twice the rounding
// growth between drains.  2 (8 MMAs per drain): the adjoint's E GEMM at 8192^2,
// k = 4370 took 3.86 ms with 1 and ~3.4 ms with 2, its gradients unchanged against
// FP64 within the tests' bounds.
#ifndef RBRP_GEMM_DRAIN
#define RBRP_GEMM_DRAIN 2
#endif

namespace rbrp {
namespace tc {
namespace {

constexpr int GEMM_DRAIN = RBRP_GEMM_DRAIN;
static_assert(GEMM_DRAIN >= 1 && CHUNK % GEMM_DRAIN == 0, "drain interval");

// Shared memory of k_gemm_tc: raw X tiles in a TMA ring, and per operand slot the
// Y hi / lo tiles; the split warps write X's hi / lo parts into tensor memory (A slots
// after the accumulators), so the MMAs read only Y from shared memory (as k_proj_w_tc).
constexpr int GRAW = 10;
struct __align__(1024) GemmSmem {
  uint8_t raw[GRAW][A_BYTES];
  uint8_t ys[2][2 * B_BYTES];                            // per operand slot: Y hi, Y lo
  unsigned long long rfull[GRAW], rempty[GRAW];
  unsigned long long ofree[2], osplit[2], oy[2];
  unsigned long long bigf[NBIG], bige[NBIG];
  unsigned long long smlf[2], smle[2];
  unsigned long long mmadone;
  uint32_t tmem_base;
  int abort;
};
constexpr size_t GEMM_SMEM = sizeof(GemmSmem) + 1024;

template <typename Epi>
__global__ void __launch_bounds__(NTHREADS, 1)
k_gemm_tc(const __grid_constant__ CUtensorMap tmX, const __grid_constant__ CUtensorMap tmYh,
          const __grid_constant__ CUtensorMap tmYl, int M, int N, int K, long long budget, int* status, Epi epi) {
  extern __shared__ uint8_t gt_raw[];
  GemmSmem& sm = *reinterpret_cast<GemmSmem*>((reinterpret_cast<uintptr_t>(gt_raw) + 1023) & ~(uintptr_t)1023);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int p0 = blockIdx.x * BM, c0 = blockIdx.y * BN;
  const int nk = (K + BK - 1) / BK;
  if (p0 >= M || c0 >= N || nk <= 0) return;
  volatile int* abort = &sm.abort;

  if (threadIdx.x == 0) {
    for (int s = 0; s < GRAW; ++s) {
      mbar_init(&sm.rfull[s], 1);
      mbar_init(&sm.rempty[s], NSPLIT);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&sm.ofree[b], 1);
      mbar_init(&sm.osplit[b], NSPLIT);
      mbar_init(&sm.oy[b], 1);
    }
    for (int b = 0; b < NBIG; ++b) {
      mbar_init(&sm.bigf[b], 1);
      mbar_init(&sm.bige[b], NDRAIN);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&sm.smlf[b], 1);
      mbar_init(&sm.smle[b], NDRAIN);
    }
    mbar_init(&sm.mmadone, 1);
    sm.abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sm.tmem_base)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = sm.tmem_base;
  int issued = 0, yissued = 0;

  if (warp == 0) {
    if (lane == 0) {
      for (int s = 0; s < nk; ++s) {
        const int rs = s % GRAW;
        if (s >= GRAW && !mbar_wait(&sm.rempty[rs], (uint32_t)((s / GRAW) & 1) ^ 1, abort, budget)) break;
        mbar_expect_tx(&sm.rfull[rs], A_BYTES);
        tma_load_2d(sm.raw[rs], &tmX, &sm.rfull[rs], s * BK, p0);
        issued = s + 1;
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      for (int s = 0; s < nk; ++s) {
        const int os = s & 1;
        const uint32_t ouse = (uint32_t)(s >> 1);
        const int g = s / GEMM_DRAIN;                 // drain group of the large accumulator
        const int b = g % NBIG;
        const bool gfirst = (s % GEMM_DRAIN) == 0, glast = (s % GEMM_DRAIN) == GEMM_DRAIN - 1 || s == nk - 1;
        const int chunk = s / CHUNK, sb = chunk & 1;
        const bool first = (s % CHUNK) == 0;
        if (gfirst && g >= NBIG && !mbar_wait(&sm.bige[b], (uint32_t)(g / NBIG - 1) & 1, abort, budget)) break;
        if (first && chunk >= 2 && !mbar_wait(&sm.smle[sb], (uint32_t)((chunk >> 1) - 1) & 1, abort, budget)) break;
        if (!mbar_wait(&sm.osplit[os], ouse & 1, abort, budget)) break;
        if (!mbar_wait(&sm.oy[os], ouse & 1, abort, budget)) break;
        tc_fence_after();
        const uint32_t txh = tbase + TA_COL + (uint32_t)(os * 2 * BK);   // X hi: 32 columns, then X lo
        const uint64_t dyh = sw128_desc(smem_u32(sm.ys[os]));
        const uint64_t dyl = sw128_desc(smem_u32(sm.ys[os] + B_BYTES));
        const uint32_t dbig = tbase + (uint32_t)(b * BN);
        const uint32_t dsml = tbase + (uint32_t)(NBIG * BN + sb * BN);
#pragma unroll
        for (int k = 0; k < BK / 8; ++k) {
          mma_tf32_ta(dbig, txh + 8 * k, dyh + 2 * k, (gfirst && k == 0) ? 0u : 1u);
          mma_tf32_ta(dsml, txh + 8 * k, dyl + 2 * k, (first && k == 0) ? 0u : 1u);
          mma_tf32_ta(dsml, txh + BK + 8 * k, dyh + 2 * k, 1u);
        }
        mma_commit(&sm.ofree[os]);
        if (glast) mma_commit(&sm.bigf[b]);
        if ((s % CHUNK) == CHUNK - 1 || s == nk - 1) mma_commit(&sm.smlf[sb]);
      }
    }
  } else if (warp < 2 + NSPLIT / 32) {
    // split warps: one X row (a 128-byte swizzled row of the raw tile) per thread into
    // TMEM lane 32 (warp % 4) + lane; the first split thread requests the Y tiles
    const int et = threadIdx.x - 64;
    const int row = 32 * (warp & 3) + lane;
    const uint32_t lane_off = (uint32_t)(32 * (warp & 3)) << 16;
    for (int s = 0; s < nk; ++s) {
      const int rs = s % GRAW, os = s & 1;
      if (s >= 2 && !mbar_wait(&sm.ofree[os], (uint32_t)((s >> 1) - 1) & 1, abort, budget)) break;
      if (et == 0) {
        mbar_expect_tx(&sm.oy[os], 2 * B_BYTES);
        tma_load_2d(sm.ys[os], &tmYh, &sm.oy[os], s * BK, c0);
        tma_load_2d(sm.ys[os] + B_BYTES, &tmYl, &sm.oy[os], s * BK, c0);
        yissued = s + 1;
      }
      if (!mbar_wait(&sm.rfull[rs], (uint32_t)(s / GRAW) & 1, abort, budget)) break;
      tc_fence_after();
      const uint8_t* rrow = sm.raw[rs] + row * 128;
      float hi[32], lo[32];
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const float4 v = *reinterpret_cast<const float4*>(rrow + ((c ^ (row & 7)) << 4));
        tf32_split(v.x, hi[4 * c], lo[4 * c]);
        tf32_split(v.y, hi[4 * c + 1], lo[4 * c + 1]);
        tf32_split(v.z, hi[4 * c + 2], lo[4 * c + 2]);
        tf32_split(v.w, hi[4 * c + 3], lo[4 * c + 3]);
      }
      const uint32_t ta = tbase + lane_off + TA_COL + (uint32_t)(os * 2 * BK);
      tmem_st32(ta, hi);
      tmem_st32(ta + BK, lo);
      asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
      tc_fence_before();
      mbar_arrive(&sm.rempty[rs]);
      mbar_arrive(&sm.osplit[os]);
    }
  } else {
    const int dw = warp - 2 - NSPLIT / 32;  // 0..7
    const int q = warp & 3;                  // TMEM lane quarter of this warp
    const int ch = dw >> 2;                  // column half of the accumulators
    const uint32_t lane_off = ((uint32_t)(32 * q) << 16) + (uint32_t)(32 * ch);
    float hi[32], lo[32];
#pragma unroll
    for (int a = 0; a < 32; ++a) hi[a] = lo[a] = 0.f;
    bool ok = true;
    const int ngroups = (nk + GEMM_DRAIN - 1) / GEMM_DRAIN;
    for (int g = 0; g < ngroups; ++g) {
      const int b = g % NBIG;
      const int d = min(nk - 1, g * GEMM_DRAIN + GEMM_DRAIN - 1);  // last stage of the group
      if (!mbar_wait(&sm.bigf[b], (uint32_t)(g / NBIG) & 1, abort, budget)) { ok = false; break; }
      tc_fence_after();
      drain32(tbase + lane_off + (uint32_t)(b * BN), hi, lo);
      tc_fence_before();
      mbar_arrive(&sm.bige[b]);
      if ((d % CHUNK) == CHUNK - 1 || d == nk - 1) {
        const int chunk = d / CHUNK, sb = chunk & 1;
        if (!mbar_wait(&sm.smlf[sb], (uint32_t)(chunk >> 1) & 1, abort, budget)) { ok = false; break; }
        tc_fence_after();
        drain32(tbase + lane_off + (uint32_t)(NBIG * BN + sb * BN), hi, lo);
        tc_fence_before();
        mbar_arrive(&sm.smle[sb]);
      }
    }
    if (ok && !*abort) epi(p0 + 32 * q + lane, c0 + 32 * ch, hi, lo, dw);
  }
  __syncthreads();
  if (*abort) {
    // as k_proj_w_tc: the CTA's own TMA copies and issued MMAs finish before TMEM is freed
    int dummy = 0;
    volatile int* never = &dummy;
    if (threadIdx.x == 0) atomicExch(status, ST_ERR_TIMEOUT);
    if (warp == 0 && lane == 0) {
      for (int s = issued - GRAW > 0 ? issued - GRAW : 0; s < issued; ++s)
        mbar_wait(&sm.rfull[s % GRAW], (uint32_t)(s / GRAW) & 1, never);
    }
    if (threadIdx.x == 64) {
      for (int s = yissued - 2 > 0 ? yissued - 2 : 0; s < yissued; ++s)
        mbar_wait(&sm.oy[s & 1], (uint32_t)(s >> 1) & 1, never);
    }
    if (warp == 1 && lane == 0) {
      mma_commit(&sm.mmadone);
      mbar_wait(&sm.mmadone, 0u, never);
    }
    __syncthreads();
  }
  epi.finish(*abort == 0);
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(TMEM_COLS) : "memory");
  }
}

}  // namespace
}  // namespace tc
}  // namespace rbrp
