// rbrp_tc.cuh - tcgen05 / TMEM / TMA projection kernel of the residual form (sm_103a).
//
// P1: W(p, a) = sum_r A_res(r, p) Q_blk(r, a) for a tile of 128 residual
// columns p (the MMA M dimension, TMEM lanes) and the <= 64 basis vectors a of
// the block (MMA N), reduced over the m rows (MMA K) in stages of 32 rows.
//
//   warp 0   TMA producer: raw A_res tiles (128 columns x 32 rows, FP32,
//            128-byte swizzled) into a 10-stage ring, completion on an mbarrier
//            with a transaction count.
//   warp 1   MMA issuer: tcgen05.mma kind::tf32 with A read from tensor memory and
//            Q from shared memory; per K step the large product Ahi Qhi goes to
//            one TMEM accumulator and the two small ones (Ahi Qlo, Alo Qhi) to
//            another.
//   warps 2-5 split each raw tile (one column per thread) by tf32_split and store
//            the hi / lo parts into one of two A slots in tensor memory; the first
//            of them loads that stage's Q hi / lo tiles (64 x 32 each, one TMA box
//            over the adjacent hi and lo arrays) into the slot's shared memory.
//   warps 6-13 drain the large accumulator after every stage and the small one
//            every 512 rows with tcgen05.ld into double-float registers; two
//            warps share each TMEM lane quarter, one per half of the 64 columns.
//
// Why the drains: the tensor core rounds its FP32 accumulator once per MMA and
// the rounding is biased, so the error grows linearly with the number of MMAs
// between drains; 4 MMAs per drain keep W accurate to ~2e-7, which the
// residual form needs (the part of A_res left along Q_blk by an error in W is
// never removed by later blocks).  The large accumulator has four buffers, the
// small one two.
//
// Every wait is bounded (about 2 s of clock64 time); on a timeout the CTA sets
// an abort flag, raises st->status, waits (bounded) for its own TMA copies and
// MMAs, frees its TMEM and returns.
#pragma once
#include <cuda.h>

#include "rbrp_common.cuh"

namespace rbrp {
namespace tc {
namespace {  // internal linkage: included by each element-type translation unit

constexpr int BM = 128;                  // residual columns per CTA (MMA M)
constexpr int BN = 64;                   // basis vectors (MMA N)
constexpr int BK = 32;                   // rows per stage = one 128-byte swizzle row of FP32
constexpr int CHUNK = 16;                // stages per drain of the small-product accumulator
constexpr int A_BYTES = BM * BK * 4;     // 16 KB
constexpr int B_BYTES = BN * BK * 4;     // 8 KB
constexpr int NSPLIT = 128;              // 4 split warps
constexpr int NDRAIN = 256;              // 8 drain warps
constexpr int NTHREADS = 64 + NSPLIT + NDRAIN;  // TMA warp, MMA warp, split warps, drain warps
constexpr int NBIG = 4;                   // large-product accumulators in the TMEM ring
constexpr int TMEM_COLS = 512;            // large x4 + small x2 = 384 columns, + two A slots of 64
constexpr int ST_ERR_TIMEOUT = 7;

// tcgen05 instruction descriptor: D = F32 (bits 4-5 = 1), A = B = TF32 (bits 7-9,
// 10-12 = 2), both K-major (bits 15, 16 = 0), N >> 3 in bits 17-22, M >> 4 in
// bits 24-28.
constexpr uint32_t IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) |
                           ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for the phase of parity `parity`: false once `budget` SM clocks
// have passed (setting *abort) or another warp has set *abort.
__device__ __forceinline__ bool mbar_wait(unsigned long long* b, uint32_t parity, volatile int* abort,
                                          long long budget = kWaitBudgetDefault) {
  if (mbar_try_wait(b, parity)) return true;
  const long long t0 = clock64();
  for (;;) {
    if (mbar_try_wait(b, parity)) return true;
    if (*abort) return false;
    if (clock64() - t0 > budget) {
      *abort = 1;
      return false;
    }
  }
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, unsigned long long* bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor, K-major operand, 128-byte swizzle: start
// address >> 4 (bits 0-13), leading byte offset (unused for this layout, 16 B),
// stride byte offset 1024 B = 8 rows of 128 B (bits 32-45), descriptor version 1
// (bits 46-47), layout SWIZZLE_128B = 2 (bits 61-63).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(IDESC), "r"(accumulate)
      : "memory");
}

// The same MMA with A (M x 8 TF32, row = TMEM lane, the 8 K values in consecutive
// 32-bit columns) read from tensor memory at a_tmem instead of shared memory.
__device__ __forceinline__ void mma_tf32_ta(uint32_t d_tmem, uint32_t a_tmem, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
      "r"(a_tmem), "l"(bdesc), "r"(IDESC), "r"(accumulate)
      : "memory");
}

// 32 registers into 32 consecutive TMEM columns of this warp's 32 lanes (completion
// is awaited by the caller with tcgen05.wait::st).
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const float (&v)[32]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], "
      "{%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, "
      "%17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, %32};" ::"r"(taddr),
      "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7]), "f"(v[8]), "f"(v[9]),
      "f"(v[10]), "f"(v[11]), "f"(v[12]), "f"(v[13]), "f"(v[14]), "f"(v[15]), "f"(v[16]), "f"(v[17]), "f"(v[18]),
      "f"(v[19]), "f"(v[20]), "f"(v[21]), "f"(v[22]), "f"(v[23]), "f"(v[24]), "f"(v[25]), "f"(v[26]), "f"(v[27]),
      "f"(v[28]), "f"(v[29]), "f"(v[30]), "f"(v[31])
      : "memory");
}

__device__ __forceinline__ void mma_commit(unsigned long long* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void df_acc(float& hi, float& lo, float x) {
  const float t = hi + x;
  const float bb = t - hi;
  lo += (hi - (t - bb)) + (x - bb);
  hi = t;
}

// 16 consecutive TMEM columns of this warp's 32 lanes into registers.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ void drain32(uint32_t taddr, float (&hi)[32], float (&lo)[32]) {
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    float v[16];
    tmem_ld16(taddr + (uint32_t)(16 * h), v);
#pragma unroll
    for (int j = 0; j < 16; ++j) df_acc(hi[16 * h + j], lo[16 * h + j], v[j]);
  }
}

// Shared memory of k_proj_w_tc.  The TMA ring holds raw A tiles only (16 KB a
// stage: 160 KB of A in flight per SM).  The split warps write each tile's hi /
// lo parts straight into tensor memory (the MMAs read A from there), so shared
// memory carries only the raw tiles and, per operand slot, that stage's Q hi / lo.
// An MMA whose A comes from shared memory re-reads its 4 KB per instruction at
// about 128 bytes per clock (a probe: 51 clocks per M128 N64 K8 TF32 MMA); from
// tensor memory only the 2 KB Q operand is read.
constexpr int RAW = 10;                                  // raw A stages in flight
constexpr uint32_t TA_COL = NBIG * BN + 2 * BN;          // TMEM columns of the A slots (after the accumulators)
static_assert(TA_COL + 2 * 2 * BK <= TMEM_COLS, "TMEM budget: accumulators + two A slots of hi, lo");
struct __align__(1024) ProjSmem {
  uint8_t raw[RAW][A_BYTES];
  uint8_t qs[2][2 * B_BYTES];                            // per operand slot: Q hi, Q lo
  unsigned long long rfull[RAW], rempty[RAW];            // raw ring: TMA done / split done
  unsigned long long ofree[2], osplit[2], oq[2];         // operand slots: MMAs done / A in TMEM / Q landed
  unsigned long long bigf[NBIG], bige[NBIG];             // large accumulators: full (MMA done) / empty (drained)
  unsigned long long smlf[2], smle[2];                   // small accumulator
  unsigned long long mmadone;                            // abort path: every MMA this CTA issued has completed
  uint32_t tmem_base;
  int abort;
};
constexpr size_t PROJ_SMEM = sizeof(ProjSmem) + 1024;    // + alignment slack of the dynamic window

__global__ void __launch_bounds__(NTHREADS, 1)
k_proj_w_tc(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmQ, State* st, int m,
            int n, int stages_per_split,
            float2* __restrict__ Wpart, long long budget) {
  extern __shared__ uint8_t p1_raw[];
  ProjSmem& sm = *reinterpret_cast<ProjSmem*>((reinterpret_cast<uintptr_t>(p1_raw) + 1023) & ~(uintptr_t)1023);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = st->i, kept = st->bs;
  const int p0 = i + kept + blockIdx.x * BM;
  if (kept == 0 || p0 >= n) return;
  // this CTA's row range: stages [s0, s0 + nk) of 32 rows (CTAs along y split the rows;
  // their partial W are summed, in split order, by the update)
  const int s0 = blockIdx.y * stages_per_split;
  const int nk = min(stages_per_split, (m + BK - 1) / BK - s0);
  if (nk <= 0) return;
  volatile int* abort = &sm.abort;

  if (threadIdx.x == 0) {
    for (int s = 0; s < RAW; ++s) {
      mbar_init(&sm.rfull[s], 1);
      mbar_init(&sm.rempty[s], NSPLIT);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&sm.ofree[b], 1);
      mbar_init(&sm.osplit[b], NSPLIT);
      mbar_init(&sm.oq[b], 1);
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
  int issued = 0;   // producer: stages whose A loads were issued
  int qissued = 0;  // first split thread: stages whose Q loads were issued

  if (warp == 0) {
    if (lane == 0) {
      for (int s = 0; s < nk; ++s) {
        const int rs = s % RAW;
        if (s >= RAW && !mbar_wait(&sm.rempty[rs], (uint32_t)((s / RAW) & 1) ^ 1, abort, budget)) break;
        mbar_expect_tx(&sm.rfull[rs], A_BYTES);
        tma_load_2d(sm.raw[rs], &tmA, &sm.rfull[rs], (s0 + s) * BK, p0);
        issued = s + 1;
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      for (int s = 0; s < nk; ++s) {
        const int os = s & 1;
        const uint32_t ouse = (uint32_t)(s >> 1);
        const int b = s % NBIG;                      // large accumulator of this stage
        const int chunk = s / CHUNK, sb = chunk & 1;  // small accumulator of this chunk
        const bool first = (s % CHUNK) == 0;
        if (s >= NBIG && !mbar_wait(&sm.bige[b], (uint32_t)(s / NBIG - 1) & 1, abort, budget)) break;
        if (first && chunk >= 2 && !mbar_wait(&sm.smle[sb], (uint32_t)((chunk >> 1) - 1) & 1, abort, budget)) break;
        if (!mbar_wait(&sm.osplit[os], ouse & 1, abort, budget)) break;
        if (!mbar_wait(&sm.oq[os], ouse & 1, abort, budget)) break;
        tc_fence_after();
        const uint32_t tah = tbase + TA_COL + (uint32_t)(os * 2 * BK);   // A hi: 32 columns, then A lo
        const uint64_t dqh = sw128_desc(smem_u32(sm.qs[os]));
        const uint64_t dql = sw128_desc(smem_u32(sm.qs[os] + B_BYTES));
        const uint32_t dbig = tbase + (uint32_t)(b * BN);
        const uint32_t dsml = tbase + (uint32_t)(NBIG * BN + sb * BN);
#pragma unroll
        for (int k = 0; k < BK / 8; ++k) {  // K = 8 TF32: 8 TMEM columns of A, 32 bytes of Q
          mma_tf32_ta(dbig, tah + 8 * k, dqh + 2 * k, k == 0 ? 0u : 1u);
          mma_tf32_ta(dsml, tah + 8 * k, dql + 2 * k, (first && k == 0) ? 0u : 1u);
          mma_tf32_ta(dsml, tah + BK + 8 * k, dqh + 2 * k, 1u);
        }
        mma_commit(&sm.ofree[os]);
        mma_commit(&sm.bigf[b]);
        if ((s % CHUNK) == CHUNK - 1 || s == nk - 1) mma_commit(&sm.smlf[sb]);
      }
    }
  } else if (warp < 2 + NSPLIT / 32) {
    // split warps: TMEM lane quarter warp % 4; a thread takes one position (a 128-byte
    // row of the swizzled raw tile: 16-byte chunk c of row r sits at chunk c ^ (r % 8)),
    // splits its 32 values and stores hi / lo into the A slot of stage s; the first split
    // thread requests that stage's Q tiles once the slot is free
    const int et = threadIdx.x - 64;  // 0..NSPLIT-1
    const int row = 32 * (warp & 3) + lane;
    const uint32_t lane_off = (uint32_t)(32 * (warp & 3)) << 16;
    for (int s = 0; s < nk; ++s) {
      const int rs = s % RAW, os = s & 1;
      if (s >= 2 && !mbar_wait(&sm.ofree[os], (uint32_t)((s >> 1) - 1) & 1, abort, budget)) break;
      if (et == 0) {
        mbar_expect_tx(&sm.oq[os], 2 * B_BYTES);   // Q hi (64 rows) then Q lo: one box of 128
        tma_load_2d(sm.qs[os], &tmQ, &sm.oq[os], (s0 + s) * BK, 0);
        qissued = s + 1;
      }
      if (!mbar_wait(&sm.rfull[rs], (uint32_t)(s / RAW) & 1, abort, budget)) break;
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
    // drain warps
    const int dw = warp - 2 - NSPLIT / 32;  // 0..7
    const int q = warp & 3;                  // TMEM lane quarter of this warp
    const int ch = dw >> 2;                  // column half of the accumulators this warp drains
    const uint32_t lane_off = ((uint32_t)(32 * q) << 16) + (uint32_t)(32 * ch);
    float hi[32], lo[32];
#pragma unroll
    for (int a = 0; a < 32; ++a) hi[a] = lo[a] = 0.f;
    bool ok = true;
    for (int d = 0; d < nk; ++d) {
      const int b = d % NBIG;
      if (!mbar_wait(&sm.bigf[b], (uint32_t)(d / NBIG) & 1, abort, budget)) { ok = false; break; }
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
    const int p = p0 + 32 * q + lane;
    if (ok && !*abort && p < n) {
      float2* wz = Wpart + (int64_t)blockIdx.y * BN * n;
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int a = 32 * ch + j;
        if (a < kept) {  // double-float (normalised), summed over the row splits by the update
          const float s = hi[j] + lo[j];
          wz[(int64_t)a * n + p] = make_float2(s, lo[j] - (s - hi[j]));
        }
      }
    }
  }
  __syncthreads();
  if (*abort) {
    // Before tensor memory is freed and the CTA exits, everything this CTA started
    // asynchronously must have finished: its TMA copies (their barriers) and the MMAs
    // the MMA thread issued (one last commit, from that thread, arrives on mmadone once
    // all of them have completed).  Both always complete; these waits use the default
    // budget whatever budget the main loop had.
    int dummy = 0;
    volatile int* never = &dummy;
    if (threadIdx.x == 0) atomicExch(&st->status, ST_ERR_TIMEOUT);
    if (warp == 0 && lane == 0) {
      for (int s = issued - RAW > 0 ? issued - RAW : 0; s < issued; ++s)
        mbar_wait(&sm.rfull[s % RAW], (uint32_t)(s / RAW) & 1, never);
    }
    if (threadIdx.x == 64) {
      for (int s = qissued - 2 > 0 ? qissued - 2 : 0; s < qissued; ++s)
        mbar_wait(&sm.oq[s & 1], (uint32_t)(s >> 1) & 1, never);
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

}  // namespace
}  // namespace tc
}  // namespace rbrp
