// rbrp_update_tc.cuh - tcgen05 / TMEM / TMA residual update of the residual form (sm_103a).
//
// P2: A_res(r, p) -= sum_a Q_blk(r, a) W(a, p) for a tile of 64 trailing
// positions p (the MMA N dimension) and the rows of one row range in chunks of
// 128 (MMA M, TMEM lanes), with K = the kept basis vectors (<= 64, one or two
// 32-wide halves).  Both operands come pre-split into TF32 hi / lo parts (hi +
// lo = the FP32 value), K-major: the basis by rows from k_panel_q_df and W^T
// from k_upd_w_prep (which also sums the projection's row-split partials and
// writes R(I2, p)).  The CUDA-core form of the same step is k_resid_update.
//
//   warp 0   TMA: the W^T tile once (hi and lo, up to 32 KB), then the basis rows
//            of every chunk (hi and lo, up to 64 KB) into a 2-stage ring.
//   warp 1   MMA issuer: per chunk and K half, Q_hi W_hi into that half's large
//            accumulator and Q_hi W_lo + Q_lo W_hi + Q_lo W_lo into the small one;
//            3 x 64 TMEM columns per chunk, double buffered.
//   warps 2-9 the update: TMEM lane = row, so a thread owns one row of the chunk
//            and 32 of the tile's positions, and every load and store instruction
//            of a warp covers 128 contiguous bytes of one column.  The thread loads
//            its 32 residual entries (the next chunk's are in flight meanwhile),
//            subtracts the three accumulators (tcgen05.ld), stores the result, and
//            a reduce-scatter over the warp's 32 rows leaves each lane the chunk's
//            sum of squares of one position, folded into its double-float partial.
//
// Accuracy: both operands are split by tf32_split (hi and lo rounded to the
// nearest TF32 values, the pair within 2^-23 of the value) and all four products
// are taken - the kernel is bound by memory, not by the MMAs - so each product is
// good to ~2^-22, about an FP32 product's error.  Each large accumulator takes the
// 4 MMAs of one K half (exact TF32 products), so its rounding - once per MMA,
// biased - stays at the level of an FP32 FMA chain over the same terms; the small
// products are 2^-11 smaller.  Norm partials: pairwise FP32 sums of 32 squares
// (positive terms) folded into double-float per chunk; the four row quarters of
// a position are added in a fixed order, one partial per row range and
// position, summed by k_norm_reduce.
//
// Every wait is bounded as in rbrp_tc.cuh; on a timeout the CTA sets an abort
// flag and st->status, waits (bounded) for its own TMA copies and MMAs, frees
// TMEM and returns.
#pragma once
#include "rbrp_df.cuh"
#include "rbrp_tc.cuh"

namespace rbrp {
namespace tc {
namespace {

constexpr int U_ROWS = BM;                  // rows per chunk (MMA M = 128)
constexpr int U_POS = BN;                   // positions per CTA (MMA N = 64)
constexpr int U_STAGES = 2;
constexpr int U_NUPD = 256;                 // 8 update warps
constexpr int U_THREADS = 64 + U_NUPD;
constexpr int U_ACC = 3 * U_POS;            // TMEM columns per chunk: large (K half 0), large (half 1), small

struct __align__(1024) UpdSmem {
  uint8_t wt[2][2][B_BYTES];                // [K half][hi, lo]: W^T, 64 positions x 32
  uint8_t qs[U_STAGES][2][2][A_BYTES];      // [stage][K half][hi, lo]: basis rows, 128 x 32
  unsigned long long wfull, qfull[U_STAGES], qempty[U_STAGES], accf[2], acce[2], mmadone;
  float2 nrm[4][U_POS];                     // norm partials by row quarter and tile position
  uint32_t tmem_base;
  int abort;
};
constexpr size_t U_SMEM = sizeof(UpdSmem) + 1024;  // + alignment slack of the dynamic window

// Sum over the warp's 32 lanes of 32 values per lane, scattered: afterwards lane l
// holds the sum of value l (rounds at offsets 16, 8, 4, 2, 1 halve the values a
// lane holds; a fixed pairwise order).
__device__ __forceinline__ float warp_reduce_scatter32(float (&v)[32]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    const bool upper = (lane & o) != 0;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      if (k < o) {
        const float send = upper ? v[k] : v[k + o];
        const float keep = upper ? v[k + o] : v[k];
        v[k] = keep + __shfl_xor_sync(0xffffffffu, send, o);
      }
    }
  }
  return v[0];
}

__global__ void __launch_bounds__(U_THREADS, 1)
k_resid_update_tc(const __grid_constant__ CUtensorMap tmWh, const __grid_constant__ CUtensorMap tmWl,
                  const __grid_constant__ CUtensorMap tmQh, const __grid_constant__ CUtensorMap tmQl, State* st,
                  float* __restrict__ Ares, int64_t ld, int m, int n, int rows_per_split,
                  double* __restrict__ part_norm, long long budget) {
  extern __shared__ uint8_t u_raw[];
  UpdSmem& sm = *reinterpret_cast<UpdSmem*>((reinterpret_cast<uintptr_t>(u_raw) + 1023) & ~(uintptr_t)1023);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = st->i, kept = st->bs;
  const int p0 = i + kept + blockIdx.x * U_POS;
  if (kept == 0 || p0 >= n) return;
  const int rb = blockIdx.y * rows_per_split, re = min(m, rb + rows_per_split);
  if (rb >= re) return;
  const int nch = (re - rb + U_ROWS - 1) / U_ROWS;
  const int nkc = kept > BK ? 2 : 1;
  volatile int* abort = &sm.abort;

  if (threadIdx.x == 0) {
    mbar_init(&sm.wfull, 1);
    for (int s = 0; s < U_STAGES; ++s) {
      mbar_init(&sm.qfull[s], 1);
      mbar_init(&sm.qempty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&sm.accf[b], 1);
      mbar_init(&sm.acce[b], U_NUPD);
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
  int issued = 0;  // producer: chunks whose basis loads were issued
  DF nrm;
  nrm.hi = nrm.lo = 0.f;

  if (warp == 0) {
    if (lane == 0) {
      mbar_expect_tx(&sm.wfull, (uint32_t)(nkc * 2 * B_BYTES));
      for (int kc = 0; kc < nkc; ++kc) {
        tma_load_2d(sm.wt[kc][0], &tmWh, &sm.wfull, kc * BK, p0);
        tma_load_2d(sm.wt[kc][1], &tmWl, &sm.wfull, kc * BK, p0);
      }
      for (int c = 0; c < nch; ++c) {
        const int slot = c % U_STAGES;
        const uint32_t use = (uint32_t)(c / U_STAGES);
        if (c >= U_STAGES && !mbar_wait(&sm.qempty[slot], (use & 1) ^ 1, abort, budget)) break;
        mbar_expect_tx(&sm.qfull[slot], (uint32_t)(nkc * 2 * A_BYTES));
        for (int kc = 0; kc < nkc; ++kc) {
          tma_load_2d(sm.qs[slot][kc][0], &tmQh, &sm.qfull[slot], kc * BK, rb + c * U_ROWS);
          tma_load_2d(sm.qs[slot][kc][1], &tmQl, &sm.qfull[slot], kc * BK, rb + c * U_ROWS);
        }
        issued = c + 1;
      }
    }
  } else if (warp == 1) {
    if (lane == 0 && mbar_wait(&sm.wfull, 0u, abort, budget)) {
      for (int c = 0; c < nch; ++c) {
        const int slot = c % U_STAGES, buf = c & 1;
        const uint32_t use = (uint32_t)(c / U_STAGES);
        if (c >= 2 && !mbar_wait(&sm.acce[buf], (uint32_t)((c >> 1) - 1) & 1, abort, budget)) break;
        if (!mbar_wait(&sm.qfull[slot], use & 1, abort, budget)) break;
        tc_fence_after();
        const uint32_t dacc = tbase + (uint32_t)(buf * U_ACC);
        for (int kc = 0; kc < nkc; ++kc) {
          const uint64_t dqh = sw128_desc(smem_u32(sm.qs[slot][kc][0]));
          const uint64_t dql = sw128_desc(smem_u32(sm.qs[slot][kc][1]));
          const uint64_t dwh = sw128_desc(smem_u32(sm.wt[kc][0]));
          const uint64_t dwl = sw128_desc(smem_u32(sm.wt[kc][1]));
#pragma unroll
          for (int k = 0; k < BK / 8; ++k) {
            mma_tf32(dacc + (uint32_t)(kc * U_POS), dqh + 2 * k, dwh + 2 * k, k == 0 ? 0u : 1u);
            mma_tf32(dacc + (uint32_t)(2 * U_POS), dqh + 2 * k, dwl + 2 * k, (kc == 0 && k == 0) ? 0u : 1u);
            mma_tf32(dacc + (uint32_t)(2 * U_POS), dql + 2 * k, dwh + 2 * k, 1u);
            mma_tf32(dacc + (uint32_t)(2 * U_POS), dql + 2 * k, dwl + 2 * k, 1u);
          }
        }
        mma_commit(&sm.qempty[slot]);
        mma_commit(&sm.accf[buf]);
      }
    }
  } else {
    const int q = warp & 3;               // TMEM lane quarter: rows 32q .. 32q + 31 of each chunk
    const int ch = (warp - 2) >> 2;       // position half of the tile
    const int pb = p0 + 32 * ch;          // this thread's positions pb .. pb + 31
    const int np = max(0, min(32, n - pb));
    float* __restrict__ base = Ares + (int64_t)pb * ld;
    const uint32_t toff = ((uint32_t)(32 * q) << 16) + (uint32_t)(32 * ch);
    // a running pointer down the positions keeps one 64-bit address live, not 32
    auto load = [&](float (&x)[32], int r) {
      const float* pj = base + r;
      const bool rv = r < re;
#pragma unroll
      for (int j = 0; j < 32; ++j, pj += ld) x[j] = (j < np && rv) ? *pj : 0.f;
    };
    bool ok = true;
    auto step = [&](float (&x)[32], float (&xf)[32], int c) {
      if (!ok || c >= nch) return;
      const int r = rb + c * U_ROWS + 32 * q + lane;
      if (c + 1 < nch) load(xf, r + U_ROWS);
      const int buf = c & 1;
      if (!mbar_wait(&sm.accf[buf], (uint32_t)(c >> 1) & 1, abort, budget)) {
        ok = false;
        return;
      }
      tc_fence_after();
      const uint32_t ta = tbase + toff + (uint32_t)(buf * U_ACC);
#pragma unroll
      for (int hf = 0; hf < 2; ++hf) {  // 16 columns at a time keeps the register count down
        float v[16];
        tmem_ld16(ta + 16 * hf, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) x[16 * hf + j] -= v[j];
        if (nkc > 1) {
          tmem_ld16(ta + U_POS + 16 * hf, v);
#pragma unroll
          for (int j = 0; j < 16; ++j) x[16 * hf + j] -= v[j];
        }
        tmem_ld16(ta + 2 * U_POS + 16 * hf, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) x[16 * hf + j] -= v[j];
      }
      tc_fence_before();
      mbar_arrive(&sm.acce[buf]);
      const bool rv = r < re;
      float* pj = base + r;
#pragma unroll
      for (int j = 0; j < 32; ++j, pj += ld) {
        if (j < np && rv) *pj = x[j];
        x[j] = (j < np && rv) ? x[j] * x[j] : 0.f;  // x is spent: its squares
      }
      df_acc(nrm.hi, nrm.lo, warp_reduce_scatter32(x));
    };
    float x0[32], x1[32];
    load(x0, rb + 32 * q + lane);
    for (int c = 0; c < nch && ok; c += 2) {
      step(x0, x1, c);
      step(x1, x0, c + 1);
    }
    sm.nrm[q][32 * ch + lane] = make_float2(nrm.hi, nrm.lo);
  }
  __syncthreads();
  if (!*abort && threadIdx.x < U_POS) {
    // the four row quarters of each position, in a fixed order
    const int t = threadIdx.x, p = p0 + t;
    dfl a = {sm.nrm[0][t].x, sm.nrm[0][t].y};
#pragma unroll
    for (int qq = 1; qq < 4; ++qq) a = df_add(a, dfl{sm.nrm[qq][t].x, sm.nrm[qq][t].y});
    if (p < n) part_norm[(int64_t)blockIdx.y * n + p] = (double)a.hi + (double)a.lo;
  }
  if (*abort) {
    // as k_proj_w_tc: the CTA's own TMA copies and issued MMAs finish before TMEM is freed
    int dummy = 0;
    volatile int* never = &dummy;
    if (threadIdx.x == 0) atomicExch(&st->status, ST_ERR_TIMEOUT);
    if (warp == 0 && lane == 0) {
      mbar_wait(&sm.wfull, 0u, never);
      for (int c = issued - U_STAGES > 0 ? issued - U_STAGES : 0; c < issued; ++c)
        mbar_wait(&sm.qfull[c % U_STAGES], (uint32_t)(c / U_STAGES) & 1, never);
    }
    if (warp == 1 && lane == 0) {
      mma_commit(&sm.mmadone);
      mbar_wait(&sm.mmadone, 0u, never);
    }
    __syncthreads();
  }
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(TMEM_COLS) : "memory");
  }
}

// W^T for k_resid_update_tc, 32 trailing positions per CTA: W(a, p) = the
// double-float sum of the projection's row-split partials in split order (as
// k_resid_update sums them), R(i + a, p) = W in FP64, and the TF32 hi / lo parts
// of rn(W) (tf32_split) into Wth / Wtl (position-major, 64 per position, zero
// for a >= kept).
__global__ void __launch_bounds__(256)
k_upd_w_prep(const State* __restrict__ st, int n, const float2* __restrict__ Wpart, int wsplit,
             double* __restrict__ R, int64_t ldr, float* __restrict__ Wth, float* __restrict__ Wtl) {
  __shared__ float tile[32][MAXB + 1];
  const int i = st->i, kept = st->bs;
  const int pb = i + kept + blockIdx.x * 32;
  if (kept == 0 || pb >= n) return;
  const int tid = threadIdx.x;
  for (int idx = tid; idx < 32 * MAXB; idx += 256) {
    const int pp = idx & 31, a = idx >> 5, p = pb + pp;
    float w = 0.f;
    if (a < kept && p < n) {
      dfl v = {0.f, 0.f};
      for (int z = 0; z < wsplit; ++z) {
        const float2 t = Wpart[((int64_t)z * MAXB + a) * n + p];
        v = df_add(v, {t.x, t.y});
      }
      R[(int64_t)(i + a) * ldr + p] = (double)v.hi + (double)v.lo;
      w = v.hi;
    }
    tile[pp][a] = w;
  }
  __syncthreads();
  for (int idx = tid; idx < 32 * MAXB; idx += 256) {
    const int a = idx & (MAXB - 1), pp = idx / MAXB, p = pb + pp;
    if (p < n) {
      float h, l;
      tf32_split(tile[pp][a], h, l);
      Wth[(int64_t)p * MAXB + a] = h;
      Wtl[(int64_t)p * MAXB + a] = l;
    }
  }
}

}  // namespace
}  // namespace tc
}  // namespace rbrp
