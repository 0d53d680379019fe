// rbrp_batched.cu - batched adaptive RBRP: many independent column IDs of
// uneven shape (e.g. the off-diagonal blocks of a hierarchical kernel matrix)
// in one persistent launch.
//
// Each problem runs the adaptive loop of RBRP() (gpu/rbrp.cu:333-503) and of
// the notebook's blocked_rpid (python/RBRP.ipynb cell 11 lines 76-173) in the
// FP32 residual form of the one-matrix path, entirely inside one CTA of 256
// threads: column norms, block sampling, panel Gram matrix, double-float
// pivoted Cholesky with the robust filter, block swap, basis solve, projection
// W = Q^T A_res and update A_res -= Q W with exact norms, stop rule, and the
// T = R11^{-1} R12 solve.  A persistent grid (CTAs per SM x SMs) pulls problem
// indices from a device-side queue (one atomicAdd per problem), largest first,
// so thousands of uneven problems balance across the SMs without host
// round trips.  Each CTA owns one workspace slot sized for the largest
// problem; nothing in the kernel waits on another CTA.
//
// Layout of a slot (one problem at a time, ld = m rounded up to 4):
//   A_res  ld x n FP32, column major, position ordered (written by the first
//          update; the first block reads A through perm, scaled)
//   R      kcap x n double-float (float2), row major, indexed by position
//   V      ld x BB FP32 sampled panel;  Qc ld x BB / Qr m x BB FP32 basis of
//          the block (column and row major)
//   diags  n FP64 residual column norms by position;  pbuf 2n FP64 sampler
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstring>
#include <map>
#include <numeric>
#include <vector>

#include "rbrp_internal.h"
#include "rbrp_pchol_df.cuh"
#include "rbrp_sampler.cuh"

namespace rbrp {

struct BatchArgs {
  unsigned char* slots;
  int64_t slot_bytes;
  int64_t off_R, off_V, off_Qc, off_Qr, off_diag, off_pbuf;
  // host-resident problems (pinned host memory): with STAGE_A the norms pass copies
  // A into the slot at off_stage, with STAGE_PERM perm is worked on in the slot at
  // off_perm and copied out at the end
  int64_t off_stage, off_perm;
  int stage;  // STAGE_A | STAGE_PERM bits
  double tol, tol_loc;
  uint64_t seed;
  int b, sampler, kmax, compute_T;
  unsigned long long* prof;  // per-phase SM cycles summed over CTAs (NULL: off)
};

enum { STAGE_A = 1, STAGE_PERM = 2 };

namespace {

// Phases of the in-kernel profile (clock64 deltas taken by thread 0 after the
// barriers that end each phase, summed over problems and CTAs).
enum { BPH_NORMS, BPH_SAMPLE, BPH_GRAM, BPH_PIVOT, BPH_BASIS, BPH_PROJECT, BPH_UPDATE, BPH_FINISH, BPH_TSOLVE, BPH_N };
static_assert(BPH_N == RBRP_BATCH_NPHASES, "phase count");

struct PhaseClock {
  unsigned long long* acc;  // shared-memory accumulators, NULL when profiling is off
  long long t;
  __device__ __forceinline__ void start(unsigned long long* a) {
    acc = (a && threadIdx.x == 0) ? a : nullptr;
    if (acc) t = clock64();
  }
  __device__ __forceinline__ void mark(int ph) {
    if (acc) {
      const long long t1 = clock64();
      acc[ph] += (unsigned long long)(t1 - t);
      t = t1;
    }
  }
};

constexpr int BT = 256;     // threads per CTA: one problem per CTA
constexpr int BROWS = 128;  // rows per stage of the Gram / projection / update loops
constexpr int TCOL = 64;    // remaining positions per column tile
constexpr int BATCH_MAXB = 32;
constexpr int QRES_FLOATS = 8192;   // resident basis (32 KB): kept x m rounded up to 128 rows
constexpr int RING_D = 4;           // stages in flight per warp
constexpr int RING_FLOATS = RING_D * 4 * BROWS;  // per warp: D stages x up to 4 columns x 128 rows (8 KB)

// Exact scaling by 2^s as two normal-float factors, so s may cover the full
// exponent range of FP32 data (|s| <= 250).
struct Pow2 {
  float a, b;
  __device__ __forceinline__ float apply(float x) const { return __fmul_rn(__fmul_rn(x, a), b); }
};
__device__ __forceinline__ Pow2 pow2_scale(int s) {
  const int s1 = s / 2, s2 = s - s1;
  return {__int_as_float((s1 + 127) << 23), __int_as_float((s2 + 127) << 23)};
}

template <int BB>
struct BatchSmem {
  State st;
  int js[MAXB];
  int cols[MAXB];
  const float* src[TCOL];  // source column of each panel column / tile column
  double red_d[32];
  int red_i[32];
  unsigned long long pacc[BPH_N];
  union {
    float gram_Vs[BROWS][BB + 1];
    struct {
      PcholDfSmemT<BB> pc;
      dfl R11s[BB][BB + 1];  // R11 in slot order (upper)
      dfl invd[BB];
    } pan;
    struct {  // staged projection / update (any kept, any m)
      __align__(16) float Ws[BB][TCOL];  // W of the current tile, FP32, for the update
      union {
        struct {
          __align__(16) float Xs[BROWS][TCOL + 4];
          __align__(16) float Qs[BROWS][BB + 4];
        } p1;
        dfl red[BT * 16];  // projection partials: 16 per thread
        __align__(16) float p2_Qs[BB][BROWS];
      };
    } stg;
    struct {  // resident basis and one asynchronous-copy ring per warp
      __align__(16) float qres[QRES_FLOATS];  // qres[a * ldq + r], zero for r >= m
      __align__(16) float ring[BT / 32][RING_FLOATS];  // also the warp's reduction buffer
    } res;
  } u;
};

// Warp sum of double-float partials (hi, lo) on the FP32 pipe, by a fixed
// butterfly; GB300's FP64 pipe is ~1/64 of the FP32 rate, so only the final
// conversion to FP64 runs there, once per column.
__device__ __forceinline__ double warp_sum_df(float hi, float lo) {
  dfl s = df_two_sum(hi, lo);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const dfl t = {__shfl_xor_sync(0xffffffffu, s.hi, o), __shfl_xor_sync(0xffffffffu, s.lo, o)};
    s = df_add(s, t);
  }
  return (threadIdx.x & 31) == 0 ? (double)s.hi + (double)s.lo : 0.0;
}

__device__ __forceinline__ int block_max_int(int v, int* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = __reduce_max_sync(0xffffffffu, v);
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  int r = sh[0];
  for (int w = 1; w < (int)(blockDim.x >> 5); ++w) r = max(r, sh[w]);
  __syncthreads();
  return r;
}

// A warp's walk over one column, f(x0, x1, x2, x3) per group of four entries
// (zeros pad the scalar groups): 16-byte loads when the column is 16-byte
// aligned.  A lane visits its groups lane, lane + 32, lane + 64, ... in order;
// the loads of each 128-group chunk are all issued before any is used (four in
// flight per lane however short the column).  The norms pass (column_walk2) and
// its rescaled second walk see the same entries in the same groups and order.
template <typename F>
__device__ __forceinline__ void column_walk(const float* __restrict__ col, int m, int lane, bool vec, F&& f) {
  if (vec) {
    const float4* c4 = reinterpret_cast<const float4*>(col);
    const int m4 = m >> 2;
    for (int r = lane; r < m4; r += 128) {
      // groups past the end read as zeros: f adds nothing for them (exact)
      float4 v[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) v[j] = r + 32 * j < m4 ? c4[r + 32 * j] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int j = 0; j < 4; ++j) f(v[j].x, v[j].y, v[j].z, v[j].w);
    }
    for (int t = 4 * m4 + lane; t < m; t += 32) f(col[t], 0.f, 0.f, 0.f);
  } else {
    for (int r = lane; r < m; r += 32) f(col[r], 0.f, 0.f, 0.f);
  }
}

// Two columns of one matrix walked in lockstep (col1 only when two): each
// column's entries reach its own visitor in exactly the order column_walk gives,
// with twice the loads in flight.  With STORE every entry read is also written
// to dst0 / dst1 (16-byte aligned): the staging copy of a host-resident column.
template <bool STORE, typename F0, typename F1>
__device__ __forceinline__ void column_walk2(const float* __restrict__ col0, float* __restrict__ dst0,
                                             const float* __restrict__ col1, float* __restrict__ dst1, bool two,
                                             int m, int lane, bool vec, F0&& f0, F1&& f1) {
  if (vec) {
    const float4* a4 = reinterpret_cast<const float4*>(col0);
    const float4* b4 = reinterpret_cast<const float4*>(col1);
    const int m4 = m >> 2;
    for (int r = lane; r < m4; r += 128) {
      float4 u[4], v[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const bool in = r + 32 * j < m4;
        u[j] = in ? a4[r + 32 * j] : make_float4(0.f, 0.f, 0.f, 0.f);
        v[j] = in && two ? b4[r + 32 * j] : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (STORE && r + 32 * j < m4) {
          reinterpret_cast<float4*>(dst0)[r + 32 * j] = u[j];
          if (two) reinterpret_cast<float4*>(dst1)[r + 32 * j] = v[j];
        }
        f0(u[j].x, u[j].y, u[j].z, u[j].w);
        f1(v[j].x, v[j].y, v[j].z, v[j].w);
      }
    }
    for (int t = 4 * m4 + lane; t < m; t += 32) {
      const float x = col0[t], y = two ? col1[t] : 0.f;
      if (STORE) {
        dst0[t] = x;
        if (two) dst1[t] = y;
      }
      f0(x, 0.f, 0.f, 0.f);
      f1(y, 0.f, 0.f, 0.f);
    }
  } else {
    for (int r = lane; r < m; r += 32) {
      const float x = col0[r], y = two ? col1[r] : 0.f;
      if (STORE) {
        dst0[r] = x;
        if (two) dst1[r] = y;
      }
      f0(x, 0.f, 0.f, 0.f);
      f1(y, 0.f, 0.f, 0.f);
    }
  }
}

// acc += x0^2 + x1^2 + x2^2 + x3^2: an FP32 sum of the four squares (positive
// terms, relative error < 3e-7) folded into the double-float sum by TwoSum
__device__ __forceinline__ void df_add_sq4(DF& acc, float x0, float x1, float x2, float x3) {
  const float q = fmaf(x3, x3, fmaf(x2, x2, fmaf(x1, x1, x0 * x0)));
  const float t = acc.hi + q;
  const float bb = t - acc.hi;
  acc.lo += (acc.hi - (t - bb)) + (q - bb);
  acc.hi = t;
}

// a1: column maxima, squared norms (double-float; a column whose maximum lies
// outside [2^-41, 2^40) is summed again scaled by its own power of two so tiny
// entries keep their resolution) and perm = identity.
// Returns the problem's exponent emax (max |A| = f 2^emax, f in [0.5, 1)) and
// rescales diags to the problem scale 2^-emax; *bad flags non-finite entries.
// With STAGE the same pass copies A to stage (ld x n, 16-byte aligned): a
// host-resident A crosses the host link once.
template <int BB, bool STAGE>
__device__ int batch_norms(BatchSmem<BB>& sm, const float* __restrict__ A, int64_t lda, int m, int n,
                           float* __restrict__ stage, int64_t ld, int* __restrict__ perm, double* __restrict__ diags,
                           int* __restrict__ colexp, int* bad, double* res0, int* nnz) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const bool vec = (lda & 3) == 0 && (reinterpret_cast<uintptr_t>(A) & 15) == 0;
  int emax = INT_MIN, nonfinite = 0;
  // warp w takes columns w, w + 8, w + 16, ... two at a time
  constexpr int NW = BT / 32;
  for (int c0 = warp; c0 < n; c0 += 2 * NW) {
    const int c1 = c0 + NW;
    const bool two = c1 < n;
    const float* col[2] = {A + (int64_t)c0 * lda, A + (int64_t)(two ? c1 : c0) * lda};
    unsigned mx[2] = {0u, 0u};
    int nf[2] = {0, 0};
    DF raw[2] = {{0.f, 0.f}, {0.f, 0.f}};
    auto visitor = [&](int k) {
      return [&, k](float x0, float x1, float x2, float x3) {
        const float v0 = fabsf(x0), v1 = fabsf(x1), v2 = fabsf(x2), v3 = fabsf(x3);
        nf[k] |= !(v0 <= FLT_MAX) | !(v1 <= FLT_MAX) | !(v2 <= FLT_MAX) | !(v3 <= FLT_MAX);
        mx[k] = max(max(mx[k], max(__float_as_uint(v0), __float_as_uint(v1))),
                    max(__float_as_uint(v2), __float_as_uint(v3)));
        df_add_sq4(raw[k], x0, x1, x2, x3);
      };
    };
    if constexpr (STAGE) {
      float* dst0 = stage + (int64_t)c0 * ld;
      float* dst1 = stage + (int64_t)(two ? c1 : c0) * ld;
      column_walk2<true>(col[0], dst0, col[1], dst1, two, m, lane, vec, visitor(0), visitor(1));
      col[0] = dst0;  // the rescaled walk below reads the device copy (same entries, same groups)
      col[1] = dst1;
    } else {
      column_walk2<false>(col[0], nullptr, col[1], nullptr, two, m, lane, vec, visitor(0), visitor(1));
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      if (k == 1 && !two) break;
      const int c = k ? c1 : c0;
      const unsigned mxk = __reduce_max_sync(0xffffffffu, mx[k]);
      const int nfk = __any_sync(0xffffffffu, nf[k]);
      double d = 0.0;
      int e = INT_MIN, ce = INT_MIN;  // column exponent; exponent of the scale d is expressed in
      if (!nfk && mxk != 0u) {
        frexpf(__uint_as_float(mxk), &e);
        if (e >= -40 && e <= 40) {
          // squares of every entry that matters (>= max 2^-24) stay normal: the raw sum is exact enough
          d = warp_sum_df(raw[k].hi, raw[k].lo);
          ce = 0;
        } else {
          const Pow2 sc = pow2_scale(-e);
          DF acc{0.f, 0.f};
          column_walk(col[k], m, lane, vec, [&](float x0, float x1, float x2, float x3) {
            df_add_sq4(acc, sc.apply(x0), sc.apply(x1), sc.apply(x2), sc.apply(x3));
          });
          d = warp_sum_df(acc.hi, acc.lo);
          ce = e;
        }
      }
      if (lane == 0) {
        diags[c] = d;
        colexp[c] = ce;
        perm[c] = c;
      }
      emax = max(emax, e);
      nonfinite |= nfk;
    }
  }
  *bad = __syncthreads_or(nonfinite);
  emax = block_max_int(emax, sm.red_i);
  double s = 0.0;
  int cnt = 0;
  for (int c = tid; c < n; c += BT) {
    const int e = colexp[c];
    const double d = (e == INT_MIN || *bad) ? 0.0 : ldexp(diags[c], 2 * (e - emax));
    diags[c] = d;
    s += d;
    cnt += d > 0.0;
  }
  *res0 = block_sum(s, sm.red_d);
  *nnz = block_sum(cnt, sm.red_i);
  return emax;
}

// Compensated product accumulation (Ogita, Rump and Oishi's Dot2): the exact
// product by FMA, the sum by TwoSum, errors gathered in lo; as accurate as a
// double-float accumulation, normalised once by the caller.
__device__ __forceinline__ void dot2_acc(float& hi, float& lo, float x, float y) {
  const float p = x * y;
  const float e = fmaf(x, y, -p);
  const float s = hi + p;
  const float z = s - hi;
  lo += ((hi - (s - z)) + (p - z)) + e;
  hi = s;
}

// a3 (residual form): V = residual columns at the sampled positions (exact, FP32)
// and their Gram matrix in double-float (exact products), written as the Schur
// complement the pivoted Cholesky starts from.
template <int BB>
__device__ void batch_gram(BatchSmem<BB>& sm, int m, int bss, bool first, Pow2 sc, float* __restrict__ V,
                           int64_t ld) {
  constexpr int NQ = BB * BB / BT, CW = BB / NQ;
  const int tid = threadIdx.x, c1 = tid / CW, c2 = tid % CW;
  float hi[NQ], lo[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) hi[q] = lo[q] = 0.f;
  constexpr int PER = BROWS * BB / BT;  // entries a thread gathers per chunk
  static_assert(PER * BT == BROWS * BB, "gather split");
  __syncthreads();  // the caller's sm.src (source column of each panel column) is published
  for (int r0 = 0; r0 < m; r0 += BROWS) {
    // every load of the chunk is issued before the stores (the stores to V could
    // alias the sources as far as the compiler knows, which would serialise them)
    float x[PER];
#pragma unroll
    for (int u = 0; u < PER; ++u) {
      const int idx = tid + u * BT, rr = idx % BROWS, c = idx / BROWS, r = r0 + rr;
      x[u] = (r < m && c < bss) ? sm.src[c][r] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < PER; ++u) {
      const int idx = tid + u * BT, rr = idx % BROWS, c = idx / BROWS, r = r0 + rr;
      float v = x[u];
      if (r < m && c < bss) {
        if (first) v = sc.apply(v);
        V[r + (int64_t)c * ld] = v;
      }
      sm.u.gram_Vs[rr][c] = v;
    }
    __syncthreads();
    const int rows = min(BROWS, m - r0);
    if (c1 < bss) {
      for (int rr = 0; rr < rows; ++rr) {
        const float x = sm.u.gram_Vs[rr][c1];
#pragma unroll
        for (int q = 0; q < NQ; ++q) dot2_acc(hi[q], lo[q], x, sm.u.gram_Vs[rr][c2 + CW * q]);
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NQ; ++q) sm.u.pan.pc.S[c1][c2 + CW * q] = df_two_sum(hi[q], lo[q]);
  if (tid < BB) {
    sm.u.pan.pc.ord[tid] = tid;
    sm.u.pan.pc.alive[tid] = tid < bss;
  }
  __syncthreads();
}

// Q = V(:, ord[:kept]) R11^{-1}, one thread per row, double-float, stored as the
// FP32 basis in column-major (update) and row-major (projection) copies, zero
// beyond the kept columns.  Also publishes R11 (slot order) for the R rows.
template <int BB>
__device__ void batch_qsolve(BatchSmem<BB>& sm, int m, int kept, const float* __restrict__ V, int64_t ld,
                             float* __restrict__ Qc, float* __restrict__ Qr) {
  auto& P = sm.u.pan;
  const int tid = threadIdx.x;
  for (int idx = tid; idx < BB * BB; idx += BT) {
    const int a = idx / BB, c = idx % BB;
    P.R11s[a][c] = (a < kept && c < kept && c >= a) ? P.pc.R[a][P.pc.ord[c]] : dfl{0.f, 0.f};
  }
  if (tid < kept) P.invd[tid] = df_recip(P.pc.R[tid][P.pc.ord[tid]]);
  __syncthreads();
  for (int r = tid; r < m; r += BT) {
    dfl x[BB];
#pragma unroll
    for (int s = 0; s < BB; ++s) {
      x[s] = {0.f, 0.f};
      if (s < kept) {
        dfl v = {V[r + (int64_t)P.pc.ord[s] * ld], 0.f};
#pragma unroll
        for (int u = 0; u < s; ++u) v = df_fms(v, x[u], P.R11s[u][s]);
        x[s] = df_mul(v, P.invd[s]);
      }
    }
#pragma unroll
    for (int s4 = 0; s4 < BB; s4 += 4) {
      float4 q4;
      q4.x = __fadd_rn(x[s4].hi, x[s4].lo);
      q4.y = __fadd_rn(x[s4 + 1].hi, x[s4 + 1].lo);
      q4.z = __fadd_rn(x[s4 + 2].hi, x[s4 + 2].lo);
      q4.w = __fadd_rn(x[s4 + 3].hi, x[s4 + 3].lo);
      reinterpret_cast<float4*>(Qr + (int64_t)r * BB)[s4 / 4] = q4;
      Qc[r + (int64_t)s4 * ld] = q4.x;
      Qc[r + (int64_t)(s4 + 1) * ld] = q4.y;
      Qc[r + (int64_t)(s4 + 2) * ld] = q4.z;
      Qc[r + (int64_t)(s4 + 3) * ld] = q4.w;
    }
  }
  __syncthreads();
}

// a6/a7 bookkeeping after the pivots: R(I2, I2) = R11; the rows above the block
// follow the block swap of the positions (R(:i, K2) = R(:i, K1), R(:i, I2) =
// R(:i, J)); the residual columns follow it too (A_res(:, K2) = A_res(:, K1)).
template <int BB>
__device__ void batch_swaps(BatchSmem<BB>& sm, int i, int kept, int n, float2* __restrict__ R,
                            float* __restrict__ Ares, int64_t ld, bool first) {
  auto& P = sm.u.pan;
  const int tid = threadIdx.x;
  const int nK = P.pc.nK;
  for (int idx = tid; idx < kept * kept; idx += BT) {
    const int a = idx / kept, c = idx % kept;
    const dfl v = P.R11s[a][c];
    R[(int64_t)(i + a) * n + i + c] = make_float2(v.hi, v.lo);
  }
  for (int row = tid; row < i; row += BT) {
    float2* Rr = R + (int64_t)row * n;
    float2 tmp[BB];
#pragma unroll
    for (int s = 0; s < BB; ++s)
      if (s < kept) tmp[s] = Rr[P.pc.J[s]];
    for (int t = 0; t < nK; ++t) Rr[P.pc.K2[t]] = Rr[P.pc.K1[t]];
#pragma unroll
    for (int s = 0; s < BB; ++s)
      if (s < kept) Rr[i + s] = tmp[s];
  }
  if (!first) {
    const int64_t n4 = ld / 4;
    for (int t = 0; t < nK; ++t) {
      const float4* src = reinterpret_cast<const float4*>(Ares + (int64_t)P.pc.K1[t] * ld);
      float4* dst = reinterpret_cast<float4*>(Ares + (int64_t)P.pc.K2[t] * ld);
      for (int64_t r4 = tid; r4 < n4; r4 += BT) dst[r4] = src[r4];
    }
  }
  __syncthreads();
}

__device__ __forceinline__ void fold_two_sum(float& hi, float& lo, float x) {
  const float t = hi + x;
  const float bb = t - hi;
  lo += (hi - (t - bb)) + (x - bb);
  hi = t;
}

// ---------------------------------------------------------------------------
// a7/a8 per tile of 64 remaining positions p: W = Q^T X (FP32 partial sums
// folded into double-float), R(I2, p) = W, then X -= Q W written to A_res with
// the exact norms of the updated columns into diags.  X is the residual
// (A_res) or, before the first update, A(:, perm[p]) scaled.
//
// Lane layout (update, and projection when kept <= 4): the tile is walked in
// two halves of 32 positions; warp w owns positions 4w..4w+3 of a half and
// lane l rows r0 + l + 32u (u < 4) of every 128-row stage, so each load and
// store instruction of a warp touches one 128-byte row segment.  The next
// stage's 16 values per thread are loaded while the current one is used.
// ---------------------------------------------------------------------------
template <int BB>
__device__ __forceinline__ float load_x(const BatchSmem<BB>& sm, int cc, int r, int m, int ncol, bool first,
                                        Pow2 sc) {
  float v = 0.f;
  if (r < m && cc < ncol) {
    v = sm.src[cc][r];
    if (first) v = sc.apply(v);
  }
  return v;
}

// Rows [r0, r0 + 128) of the kept basis columns into p2_Qs[a][row].
template <int BB>
__device__ __forceinline__ void stage_basis(BatchSmem<BB>& sm, const float* __restrict__ Qc, int64_t ld, int m,
                                            int r0, int kept) {
  for (int idx = threadIdx.x; idx < kept * (BROWS / 4); idx += BT) {
    const int a = idx / (BROWS / 4), j = idx % (BROWS / 4), r = r0 + 4 * j;
    const float* qa = Qc + (int64_t)a * ld;
    float4 v;
    if (r + 3 < m) {
      v = *reinterpret_cast<const float4*>(qa + r);
    } else {
      v.x = r < m ? qa[r] : 0.f;
      v.y = r + 1 < m ? qa[r + 1] : 0.f;
      v.z = r + 2 < m ? qa[r + 2] : 0.f;
      v.w = r + 3 < m ? qa[r + 3] : 0.f;
    }
    *reinterpret_cast<float4*>(&sm.u.stg.p2_Qs[a][4 * j]) = v;
  }
}

// Projection from staged tiles: a thread computes 4 basis rows x 4 positions from
// staged tiles; the basis rows cover kept rounded up to 4 nq (nq a power of
// two), and the CTA's 256 / (16 nq) thread groups split each 128-row stage,
// their partials summed at the end of the tile.
template <int BB>
__device__ void proj_staged(BatchSmem<BB>& sm, int m, int n, int i, int kept, int p0, int ncol, bool first,
                            Pow2 sc, const float* __restrict__ Qr, float2* __restrict__ R) {
  constexpr int XPT = BROWS * TCOL / BT;  // staged values per thread and stage
  const int tid = threadIdx.x;
  const int nq = kept <= 4 ? 1 : kept <= 8 ? 2 : kept <= 16 ? 4 : 8;
  const int gt = 16 * nq, ng = BT / gt, grows = BROWS / ng, na = 4 * nq;
  const int g = tid / gt, lt = tid % gt, aq = lt / 16, cq = lt % 16;
  const int xr_row = tid & (BROWS - 1), xr_col = tid / BROWS;  // staging: row, first column (step BT / BROWS)
  float xr[XPT];
  auto load_stage = [&](int r0) {
#pragma unroll
    for (int j = 0; j < XPT; ++j) xr[j] = load_x(sm, xr_col + (BT / BROWS) * j, r0 + xr_row, m, ncol, first, sc);
  };
  load_stage(0);
  float hi[4][4], lo[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) hi[u][v] = lo[u][v] = 0.f;
  for (int r0 = 0; r0 < m; r0 += BROWS) {
    __syncthreads();
#pragma unroll
    for (int j = 0; j < XPT; ++j) sm.u.stg.p1.Xs[xr_row][xr_col + (BT / BROWS) * j] = xr[j];
    for (int idx = tid; idx < BROWS * nq; idx += BT) {
      const int rr = idx / nq, j = idx % nq, r = r0 + rr;
      const float4 v = r < m ? reinterpret_cast<const float4*>(Qr + (int64_t)r * BB)[j]
                             : make_float4(0.f, 0.f, 0.f, 0.f);
      *reinterpret_cast<float4*>(&sm.u.stg.p1.Qs[rr][4 * j]) = v;
    }
    __syncthreads();
    if (r0 + BROWS < m) load_stage(r0 + BROWS);
    float c[4][4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) c[u][v] = 0.f;
    const int rb = g * grows, re = min(rb + grows, m - r0);
    for (int rr = rb; rr < re; ++rr) {
      const float4 q4 = *reinterpret_cast<const float4*>(&sm.u.stg.p1.Qs[rr][4 * aq]);
      const float4 x4 = *reinterpret_cast<const float4*>(&sm.u.stg.p1.Xs[rr][4 * cq]);
      const float qv[4] = {q4.x, q4.y, q4.z, q4.w};
      const float xv[4] = {x4.x, x4.y, x4.z, x4.w};
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) c[u][v] = fmaf(qv[u], xv[v], c[u][v]);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) fold_two_sum(hi[u][v], lo[u][v], c[u][v]);
  }
  __syncthreads();
  // partials of group g at red[(g * na + a) * TCOL + c]
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) sm.u.stg.red[(g * na + 4 * aq + u) * TCOL + 4 * cq + v] = {hi[u][v], lo[u][v]};
  __syncthreads();
  for (int idx = tid; idx < kept * TCOL; idx += BT) {
    const int a = idx / TCOL, cc = idx % TCOL;
    dfl w = sm.u.stg.red[a * TCOL + cc];
    for (int gg = 1; gg < ng; ++gg) w = df_add(w, sm.u.stg.red[(gg * na + a) * TCOL + cc]);
    w = df_two_sum(w.hi, w.lo);
    if (cc < ncol) R[(int64_t)(i + a) * n + p0 + cc] = make_float2(w.hi, w.lo);
    sm.u.stg.Ws[a][cc] = w.hi;
  }
  __syncthreads();
}

// Update X -= Q W in the lane layout, the updated columns written to A_res and
// their squared norms (double-float) into diags.
template <int BB>
__device__ void update_lanes(BatchSmem<BB>& sm, int m, int kept, int p0, int ncol, bool first, Pow2 sc,
                             float* __restrict__ Ares, int64_t ld, const float* __restrict__ Qc,
                             double* __restrict__ diags) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int h = 0; h < TCOL / 32 && 32 * h < ncol; ++h) {
    const int c0 = 32 * h + 4 * warp;
    DF nrm[4];
    float x[4][4];
#pragma unroll
    for (int j = 0; j < 4; ++j) nrm[j].hi = nrm[j].lo = 0.f;
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int j = 0; j < 4; ++j) x[u][j] = load_x(sm, c0 + j, lane + 32 * u, m, ncol, first, sc);
    for (int r0 = 0; r0 < m; r0 += BROWS) {
      __syncthreads();
      stage_basis(sm, Qc, ld, m, r0, kept);
      __syncthreads();
      float xn[4][4];
      const bool more = r0 + BROWS < m;
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int j = 0; j < 4; ++j) xn[u][j] = more ? load_x(sm, c0 + j, r0 + BROWS + lane + 32 * u, m, ncol, first, sc) : 0.f;
      float acc[4][4];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[u][j] = 0.f;
      for (int a = 0; a < kept; ++a) {
        float q[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) q[u] = sm.u.stg.p2_Qs[a][lane + 32 * u];
        const float4 w4 = *reinterpret_cast<const float4*>(&sm.u.stg.Ws[a][c0]);
        const float wv[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[u][j] = fmaf(q[u], wv[j], acc[u][j]);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int r = r0 + lane + 32 * u, cc = c0 + j;
          if (r < m && cc < ncol) {
            const float y = x[u][j] - acc[u][j];
            Ares[(int64_t)(p0 + cc) * ld + r] = y;
            df_add_sq(nrm[j], y);
          }
          x[u][j] = xn[u][j];
        }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const double d = warp_sum_df(nrm[j].hi, nrm[j].lo);
      if (lane == 0 && c0 + j < ncol) diags[p0 + c0 + j] = d;
    }
  }
  __syncthreads();
}

__device__ __forceinline__ void cp_async16(float* smem, const float* gmem, int src_bytes) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(gmem), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async16_sa(unsigned sa, const float* gmem, int src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(gmem), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async4(float* smem, const float* gmem, int src_bytes) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(sa), "l"(gmem), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Sum over the 32 lanes of 16 double-float values per lane by a shuffle
// reduce-scatter (rounds at offsets 16, 8, 4, 2 halve the values each lane
// holds, the last adds the lane pair): afterwards lanes 2v and 2v + 1 hold the
// sum of value v, in a fixed order.
__device__ __forceinline__ dfl warp_reduce_scatter16(float (&hi)[16], float (&lo)[16]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 16, cnt = 16; o >= 2; o >>= 1, cnt >>= 1) {
    const bool upper = (lane & o) != 0;
    const int half = cnt / 2;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (k < half) {
        const float sh = upper ? hi[k] : hi[k + half], sl = upper ? lo[k] : lo[k + half];
        const dfl keep = upper ? dfl{hi[k + half], lo[k + half]} : dfl{hi[k], lo[k]};
        const dfl recv = {__shfl_xor_sync(0xffffffffu, sh, o), __shfl_xor_sync(0xffffffffu, sl, o)};
        const dfl r = upper ? df_add(recv, keep) : df_add(keep, recv);
        hi[k] = r.hi;
        lo[k] = r.lo;
      }
    }
  }
  const dfl mine = {hi[0], lo[0]};
  const dfl other = {__shfl_xor_sync(0xffffffffu, hi[0], 1), __shfl_xor_sync(0xffffffffu, lo[0], 1)};
  const dfl r = (lane & 1) ? df_add(other, mine) : df_add(mine, other);
  return df_two_sum(r.hi, r.lo);
}

template <int CW>
struct IssueState {
  int t;       // next stage of the warp's stream to issue
  int g, s;    // its group and its stage within the pass
  int upd;     // 0: projection pass, 1: update pass
  const float* src[CW];
};

template <int CW>
__device__ __forceinline__ void issue_sources(IssueState<CW>& is, int p, int n, bool first,
                                              const float* __restrict__ A, int64_t lda, const int* __restrict__ perm,
                                              const float* Ares, int64_t ld) {
  if (p >= n) return;
  const int nc = min(CW, n - p);
#pragma unroll
  for (int j = 0; j < CW; ++j) {
    const int pj = p + min(j, nc - 1);
    is.src[j] = first ? A + (int64_t)perm[pj] * lda : Ares + (int64_t)pj * ld;
  }
}

// Issues the next stage of a warp's stream into ring slot t % RING_D (past
// the end only an empty group is committed, which keeps the group count
// uniform): this lane's 4 rows of each of the group's columns, zero-filled
// beyond m.  Stages run projection 0..nst-1, update 0..nst-1 per group.
template <int CW>
__device__ __forceinline__ void ring_issue(IssueState<CW>& is, int total, int nst, int p_first, int stride, int n,
                                           int m, bool first, bool vec, const float* __restrict__ A, int64_t lda,
                                           const int* __restrict__ perm, const float* Ares, int64_t ld, float* ring) {
  const int lane = threadIdx.x & 31;
  if (is.t < total) {
    const int r = is.s * BROWS + 4 * lane;
    const int valid = max(0, min(4, m - r));
    const int off = valid > 0 ? r : 0;
    const unsigned sa = (unsigned)__cvta_generic_to_shared(ring + (is.t % RING_D) * CW * BROWS + 4 * lane);
#pragma unroll
    for (int j = 0; j < CW; ++j) {
      float* dst = ring + ((is.t % RING_D) * CW + j) * BROWS + 4 * lane;
      if (vec) {
        cp_async16_sa(sa + j * BROWS * (unsigned)sizeof(float), is.src[j] + off, 4 * valid);
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e) cp_async4(dst + e, e < valid ? is.src[j] + r + e : is.src[j], e < valid ? 4 : 0);
      }
    }
    if (++is.s == nst) {
      is.s = 0;
      is.upd ^= 1;
      if (!is.upd) issue_sources<CW>(is, p_first + (++is.g) * stride, n, first, A, lda, perm, Ares, ld);
    }
  }
  ++is.t;
  cp_async_commit();
}

// Resident basis (kept <= KA, kept * ldq <= QRES_FLOATS): every warp streams
// its own groups of CW = 16 / KA positions, each through projection (nst
// stages of 128 rows), a warp-level sum of the partials and update (the same
// nst stages again), with no CTA barrier.  Lane l owns rows r0 + 4l .. +3 of a
// stage.  All stages of the warp form one sequence fed by a ring of RING_D
// asynchronous copies (cp.async, 16 bytes per lane and column, or 4-byte
// copies when the caller's columns are not 16-byte aligned) that runs ahead
// across the projection/update and group boundaries; each lane reads back
// only what it copied itself.  The update's reads of a group hit L2, where
// the projection's reads left them.
template <int BB, int KA>
__device__ void project_update_resident(BatchSmem<BB>& sm, int m, int n, int i, int kept, bool first, Pow2 sc,
                                        const float* __restrict__ A, int64_t lda, const int* __restrict__ perm,
                                        float* __restrict__ Ares, int64_t ld, int ldq, float2* __restrict__ R,
                                        double* __restrict__ diags) {
  constexpr int CW = 16 / KA;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const float* __restrict__ qres = sm.u.res.qres;
  float* ring = sm.u.res.ring[warp];
  const bool vec = !first || ((lda & 3) == 0 && (reinterpret_cast<uintptr_t>(A) & 15) == 0);
  const int nst = (m + BROWS - 1) / BROWS;
  const int stride = CW * (BT / 32);
  const int p_first = i + kept + CW * warp;
  const int ngroups = p_first < n ? (n - p_first + stride - 1) / stride : 0;
  const int total = ngroups * 2 * nst;
  // issue side: source columns of the group being fetched
  IssueState<CW> is;
  is.t = is.g = is.s = is.upd = 0;
  issue_sources<CW>(is, p_first, n, first, A, lda, perm, Ares, ld);
  auto fetch = [&](int t, float (&x)[4][CW]) {
#pragma unroll
    for (int j = 0; j < CW; ++j) {
      const float4 v4 = *reinterpret_cast<const float4*>(ring + ((t % RING_D) * CW + j) * BROWS + 4 * lane);
      x[0][j] = first ? sc.apply(v4.x) : v4.x;
      x[1][j] = first ? sc.apply(v4.y) : v4.y;
      x[2][j] = first ? sc.apply(v4.z) : v4.z;
      x[3][j] = first ? sc.apply(v4.w) : v4.w;
    }
  };
#pragma unroll
  for (int t = 0; t < RING_D - 1; ++t)
    ring_issue<CW>(is, total, nst, p_first, stride, n, m, first, vec, A, lda, perm, Ares, ld, ring);
  int t = 0;
  for (int g = 0; g < ngroups; ++g) {
    const int p = p_first + g * stride, nc = min(CW, n - p);
    // projection: W(a, j) = sum_r q_a(r) x_j(r), FP32 stage sums folded into double-float
    // (FP32 sums of a lane's 16 rows, four stages, are folded at a time)
    float hi[16], lo[16], c[16];
#pragma unroll
    for (int v = 0; v < 16; ++v) hi[v] = lo[v] = c[v] = 0.f;
    for (int s = 0; s < nst; ++s, ++t) {
      ring_issue<CW>(is, total, nst, p_first, stride, n, m, first, vec, A, lda, perm, Ares, ld, ring);
      cp_async_wait<RING_D - 1>();
      float x[4][CW];
      fetch(t, x);
      const int r0 = s * BROWS + 4 * lane;
      const bool fold = (s & 3) == 3 || s == nst - 1;
#pragma unroll
      for (int a = 0; a < KA; ++a) {
        if (a < kept) {
          const float4 q4 = *reinterpret_cast<const float4*>(qres + a * ldq + r0);
          const float q[4] = {q4.x, q4.y, q4.z, q4.w};
#pragma unroll
          for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int j = 0; j < CW; ++j) c[a * CW + j] = fmaf(q[u], x[u][j], c[a * CW + j]);
          if (fold) {
#pragma unroll
            for (int j = 0; j < CW; ++j) {
              fold_two_sum(hi[a * CW + j], lo[a * CW + j], c[a * CW + j]);
              c[a * CW + j] = 0.f;
            }
          }
        }
      }
    }
    const dfl wsum = warp_reduce_scatter16(hi, lo);  // value v = lane >> 1
    {
      const int v = lane >> 1, a = v / CW, j = v % CW;
      if ((lane & 1) == 0 && a < kept && j < nc) R[(int64_t)(i + a) * n + p + j] = make_float2(wsum.hi, wsum.lo);
    }
    float w[KA][CW];
#pragma unroll
    for (int a = 0; a < KA; ++a)
#pragma unroll
      for (int j = 0; j < CW; ++j) w[a][j] = __shfl_sync(0xffffffffu, wsum.hi, 2 * (a * CW + j));
    // update X -= Q W into A_res; squared norms of the updated columns: FP32
    // sums of each lane's 8 squares, two stages (positive terms, relative error
    // < 5e-7), folded into double-float
    DF nrm[CW];
    float sq[CW];
#pragma unroll
    for (int j = 0; j < CW; ++j) nrm[j].hi = nrm[j].lo = sq[j] = 0.f;
    for (int s = 0; s < nst; ++s, ++t) {
      ring_issue<CW>(is, total, nst, p_first, stride, n, m, first, vec, A, lda, perm, Ares, ld, ring);
      cp_async_wait<RING_D - 1>();
      float x[4][CW];
      fetch(t, x);
      const int r0 = s * BROWS + 4 * lane;
      float acc[4][CW];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int j = 0; j < CW; ++j) acc[u][j] = 0.f;
#pragma unroll
      for (int a = 0; a < KA; ++a) {
        if (a < kept) {
          const float4 q4 = *reinterpret_cast<const float4*>(qres + a * ldq + r0);
          const float q[4] = {q4.x, q4.y, q4.z, q4.w};
#pragma unroll
          for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int j = 0; j < CW; ++j) acc[u][j] = fmaf(q[u], w[a][j], acc[u][j]);
        }
      }
      const int valid = max(0, min(4, m - r0));
#pragma unroll
      for (int j = 0; j < CW; ++j) {
        if (j < nc && valid > 0) {
          float y[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) y[u] = x[u][j] - acc[u][j];
          float* dst = Ares + (int64_t)(p + j) * ld + r0;
          if (valid == 4) {
            *reinterpret_cast<float4*>(dst) = make_float4(y[0], y[1], y[2], y[3]);
          } else {
#pragma unroll
            for (int u = 0; u < 4; ++u)
              if (u < valid) dst[u] = y[u];
          }
          // rows >= m give y = 0 (zero-filled x, zero basis rows)
          sq[j] = fmaf(y[3], y[3], fmaf(y[2], y[2], fmaf(y[1], y[1], fmaf(y[0], y[0], sq[j]))));
        }
      }
      if ((s & 1) || s == nst - 1) {
#pragma unroll
        for (int j = 0; j < CW; ++j) {
          fold_two_sum(nrm[j].hi, nrm[j].lo, sq[j]);
          sq[j] = 0.f;
        }
      }
    }
#pragma unroll
    for (int j = 0; j < CW; ++j) {
      const double d = warp_sum_df(nrm[j].hi, nrm[j].lo);
      if (lane == 0 && j < nc) diags[p + j] = d;
    }
  }
  cp_async_wait<0>();
  __syncthreads();
}

template <int BB>
__device__ void batch_project_update(BatchSmem<BB>& sm, int m, int n, int i, int kept, bool first, Pow2 sc,
                                     const float* __restrict__ A, int64_t lda, const int* __restrict__ perm,
                                     float* __restrict__ Ares, int64_t ld, const float* __restrict__ Qc,
                                     const float* __restrict__ Qr, float2* __restrict__ R,
                                     double* __restrict__ diags, PhaseClock& clk) {
  const int tid = threadIdx.x;
  const int ldq = (m + BROWS - 1) / BROWS * BROWS;
  const int ka = kept <= 4 ? 4 : kept <= 8 ? 8 : 16;
  if (kept <= 16 && kept * ldq <= QRES_FLOATS) {
    // stage the kept basis columns once (rows >= m zero), then barrier-free warp streams
    for (int idx = tid; idx < kept * (ldq / 4); idx += BT) {
      const int a = idx / (ldq / 4), r = 4 * (idx % (ldq / 4));
      const float* qa = Qc + (int64_t)a * ld;
      float4 v;
      if (r + 3 < m) {
        v = *reinterpret_cast<const float4*>(qa + r);
      } else {
        v.x = r < m ? qa[r] : 0.f;
        v.y = r + 1 < m ? qa[r + 1] : 0.f;
        v.z = r + 2 < m ? qa[r + 2] : 0.f;
        v.w = r + 3 < m ? qa[r + 3] : 0.f;
      }
      *reinterpret_cast<float4*>(&sm.u.res.qres[a * ldq + r]) = v;
    }
    __syncthreads();
    if (ka == 4)
      project_update_resident<BB, 4>(sm, m, n, i, kept, first, sc, A, lda, perm, Ares, ld, ldq, R, diags);
    else if (ka == 8)
      project_update_resident<BB, 8>(sm, m, n, i, kept, first, sc, A, lda, perm, Ares, ld, ldq, R, diags);
    else
      project_update_resident<BB, 16>(sm, m, n, i, kept, first, sc, A, lda, perm, Ares, ld, ldq, R, diags);
    clk.mark(BPH_UPDATE);
    return;
  }
  for (int p0 = i + kept; p0 < n; p0 += TCOL) {
    const int ncol = min(TCOL, n - p0);
    __syncthreads();
    if (tid < TCOL)
      sm.src[tid] = tid < ncol ? (first ? A + (int64_t)perm[p0 + tid] * lda : Ares + (int64_t)(p0 + tid) * ld)
                               : nullptr;
    __syncthreads();
    proj_staged<BB>(sm, m, n, i, kept, p0, ncol, first, sc, Qr, R);
    clk.mark(BPH_PROJECT);
    update_lanes<BB>(sm, m, kept, p0, ncol, first, sc, Ares, ld, Qc, diags);
    clk.mark(BPH_UPDATE);
  }
  __syncthreads();
}

// a10: T = R11^{-1} R12 in place in R (double-float back substitution, one
// thread per column of R12, eight rows per register chunk), then written to
// the caller's T (k x (n-k), column major, ld = k) in FP64.
__device__ void batch_tsolve(float2* __restrict__ R, int n, int k, dfl* __restrict__ invd, double* __restrict__ T) {
  const int tid = threadIdx.x;
  for (int a = tid; a < k; a += BT) {
    const float2 d = R[(int64_t)a * n + a];
    invd[a] = df_recip({d.x, d.y});
  }
  __syncthreads();
  const int nc = n - k;
  for (int c = tid; c < nc; c += BT) {
    float2* col = R + k + c;  // element (a, k + c) at col[a * n]
    for (int a1 = k; a1 > 0; a1 -= 8) {
      const int a0 = max(0, a1 - 8);
      dfl acc[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int a = a0 + j;
        const float2 v = a < a1 ? col[(int64_t)a * n] : make_float2(0.f, 0.f);
        acc[j] = {v.x, v.y};
      }
      for (int u = a1; u < k; ++u) {
        const float2 xv = col[(int64_t)u * n];
        const dfl xu = {xv.x, xv.y};
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          if (a0 + j < a1) {
            const float2 r = R[(int64_t)(a0 + j) * n + u];
            acc[j] = df_fms(acc[j], {r.x, r.y}, xu);
          }
        }
      }
#pragma unroll
      for (int j = 7; j >= 0; --j) {
        const int a = a0 + j;
        if (a < a1) {
          const dfl x = df_mul(acc[j], invd[a]);
          col[(int64_t)a * n] = make_float2(x.hi, x.lo);
#pragma unroll
          for (int jj = 0; jj < j; ++jj) {
            const float2 r = R[(int64_t)(a0 + jj) * n + a];
            acc[jj] = df_fms(acc[jj], {r.x, r.y}, x);
          }
        }
      }
    }
  }
  __syncthreads();
  const int64_t total = (int64_t)k * nc;
  for (int64_t idx = tid; idx < total; idx += BT) {
    const int a = (int)(idx % k);
    const int64_t c = idx / k;
    const float2 x = R[(int64_t)a * n + k + c];
    T[idx] = (double)x.x + (double)x.y;
  }
}

template <int BB, bool HOST>
__device__ void solve_problem(BatchSmem<BB>& sm, const rbrp_batch_problem& pr, int pid, unsigned char* slot,
                              const BatchArgs& args, rbrp_batch_result* res) {
  const int tid = threadIdx.x;
  const int m = pr.m, n = pr.n;
  int64_t lda = pr.lda;
  const float* A = pr.A;
  const int64_t ld = ((int64_t)m + 3) & ~(int64_t)3;
  // host-resident batch: perm lives in the slot while the problem runs, A is read
  // from the host once (norms pass) and from the slot's staged copy afterwards
  float* stage = HOST ? reinterpret_cast<float*>(slot + args.off_stage) : nullptr;
  int* perm = HOST ? reinterpret_cast<int*>(slot + args.off_perm) : pr.perm;
  float* Ares = reinterpret_cast<float*>(slot);
  float2* R = reinterpret_cast<float2*>(slot + args.off_R);
  float* V = reinterpret_cast<float*>(slot + args.off_V);
  float* Qc = reinterpret_cast<float*>(slot + args.off_Qc);
  float* Qr = reinterpret_cast<float*>(slot + args.off_Qr);
  double* diags = reinterpret_cast<double*>(slot + args.off_diag);
  double* pbuf = reinterpret_cast<double*>(slot + args.off_pbuf);
  const int mn = min(m, n);
  const int kcap = args.kmax > 0 ? min(args.kmax, mn) : mn;

  PhaseClock clk;
  clk.start(args.prof ? sm.pacc : nullptr);
  int bad = 0, nnz = 0;
  double res0 = 0.0;
  const int emax = batch_norms<BB, HOST>(sm, A, lda, m, n, stage, ld, perm, diags, reinterpret_cast<int*>(pbuf),
                                         &bad, &res0, &nnz);
  if (HOST) {
    A = stage;
    lda = ld;
  }
  const Pow2 sc = pow2_scale(emax == INT_MIN ? 0 : -emax);
  State& st = sm.st;
  if (tid == 0) {
    st.i = 0;
    st.bs_sampled = 0;
    st.bs = 0;
    st.nblocks = 0;
    st.zero_panel = 0;
    st.nK = 0;
    st.recomputes = 0;
    st.attempts = 0;
    st.draws = 0ull;
    st.res0 = res0;
    st.residual = res0;
    st.nnz_rem = nnz;
    st.status = bad ? ST_ERR_NUMERIC : 0;
    st.done = (bad || nnz == 0 || kcap <= 0) ? 1 : 0;
  }
  __syncthreads();
  clk.mark(BPH_NORMS);
  const int max_attempts = 4 * kcap + 64;
  const uint64_t seed = args.seed + (uint64_t)pid;
  double alg_bytes = 4.0 * m * n, alg_flops = 2.0 * m * n;  // thread 0's tally of the algorithmic work
  for (;;) {
    if (st.done) break;
    if (st.attempts >= max_attempts) {
      __syncthreads();
      if (tid == 0) {
        st.status = ST_ERR_NUMERIC;
        st.done = 1;
      }
      __syncthreads();
      break;
    }
    const int i = st.i;
    const bool first = i == 0;
    sample_block<BT>(&st, diags, perm, n, kcap, args.b, seed, args.sampler, pbuf,
                 reinterpret_cast<unsigned long long*>(pbuf), sm.js, sm.cols);
    const int bss = st.bs_sampled;
    clk.mark(BPH_SAMPLE);
    if (tid < bss) {
      const int p = sm.js[tid];
      sm.src[tid] = first ? A + (int64_t)perm[p] * lda : Ares + (int64_t)p * ld;
    }
    batch_gram<BB>(sm, m, bss, first, sc, V, ld);
    clk.mark(BPH_GRAM);
    const int kept = pchol_filter_df<BB>(sm.u.pan.pc, bss, min(bss, m), args.tol_loc);
    block_swap_parallel<BB>(sm.u.pan.pc, i, kept, sm.js, perm, diags, sm.u.pan.pc.J, sm.u.pan.pc.K1,
                            sm.u.pan.pc.K2, &st);
    __syncthreads();
    clk.mark(BPH_PIVOT);
    double s = 0.0;
    int c = 0;
    if (kept > 0) {
      batch_qsolve<BB>(sm, m, kept, V, ld, Qc, Qr);
      batch_swaps<BB>(sm, i, kept, n, R, Ares, ld, first);
      clk.mark(BPH_BASIS);
      batch_project_update<BB>(sm, m, n, i, kept, first, sc, A, lda, perm, Ares, ld, Qc, Qr, R, diags, clk);
      for (int p = i + kept + tid; p < n; p += BT) {
        const double d = diags[p];
        s += d;
        c += d > 0.0;
      }
    } else {
      // numerically zero panel: drop the sampled columns' weights and go on
      if (tid < bss) diags[sm.js[tid]] = 0.0;
      __syncthreads();
      for (int p = i + tid; p < n; p += BT) {
        const double d = diags[p];
        s += d;
        c += d > 0.0;
      }
    }
    s = block_sum(s, sm.red_d);
    c = block_sum(c, sm.red_i);
    if (tid == 0) {
      const double nt = (double)(n - i - kept), dm = (double)m;
      alg_bytes += 4.0 * dm * (nt + bss);
      alg_flops += 2.0 * dm * nt * kept + 4.0 * dm * bss * bss;
      st.attempts += 1;
      st.residual = s;
      st.nnz_rem = c;
      if (kept > 0) {
        st.i = i + kept;
        st.nblocks += 1;
        if ((args.tol > 0.0 && s < st.res0 * args.tol) || c == 0 || st.i >= kcap || !(s == s)) st.done = 1;
        if (!(s == s)) st.status = ST_ERR_NUMERIC;
      } else {
        st.zero_panel = 0;
        if (c == 0 || bss == 0) st.done = 1;
      }
    }
    __syncthreads();
    clk.mark(BPH_FINISH);
  }
  const int k = st.i;
  if (HOST)
    for (int p = tid; p < n; p += BT) pr.perm[p] = perm[p];
  int status = st.status == 0 ? RBRP_OK : RBRP_ERR_NUMERIC;
  if (args.compute_T && pr.T && status == RBRP_OK && k > 0 && k < n) {
    if ((int64_t)k * (n - k) > pr.T_cap)
      status = RBRP_ERR_CAPACITY;
    else
      batch_tsolve(R, n, k, reinterpret_cast<dfl*>(V), pr.T);
  }
  if (tid == 0) {
    res->k = k;
    res->nblocks = st.nblocks;
    res->status = status;
    res->attempts = st.attempts;
    res->res0 = emax == INT_MIN ? 0.0 : ldexp(st.res0, 2 * emax);
    res->err_est = st.res0 > 0.0 ? st.residual / st.res0 : 0.0;
    res->draws = st.draws;
    res->alg_bytes = alg_bytes;
    res->alg_flops = alg_flops + (double)k * k * (n - k);
  }
  __syncthreads();
  clk.mark(BPH_TSOLVE);
}

template <int BB, bool HOST>
__global__ void __launch_bounds__(BT, 2)
k_rbrp_batched(const rbrp_batch_problem* __restrict__ probs, const int* __restrict__ order, int nprob,
               int* __restrict__ queue, BatchArgs args, rbrp_batch_result* __restrict__ results) {
  extern __shared__ __align__(16) unsigned char batch_smem[];
  BatchSmem<BB>& sm = *reinterpret_cast<BatchSmem<BB>*>(batch_smem);
  __shared__ int s_q;
  unsigned char* slot = args.slots + (size_t)blockIdx.x * (size_t)args.slot_bytes;
  if (threadIdx.x < BPH_N) sm.pacc[threadIdx.x] = 0ull;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_q = atomicAdd(queue, 1);
    __syncthreads();
    const int q = s_q;
    if (q >= nprob) break;
    const int pid = order[q];
    solve_problem<BB, HOST>(sm, probs[pid], pid, slot, args, results + pid);
  }
  if (args.prof && threadIdx.x < BPH_N) atomicAdd(args.prof + threadIdx.x, sm.pacc[threadIdx.x]);
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct BatchState {
  int nprob = 0;
  std::vector<rbrp_batch_problem> probs;
  rbrp_batch_problem* d_probs = nullptr;
  int* d_order = nullptr;
  rbrp_batch_result* d_res = nullptr;
  int* d_queue = nullptr;
  size_t cap_probs = 0;
  unsigned char* slots = nullptr;
  size_t slots_bytes = 0;
  BatchArgs args{};
  int BB = 32, grid = 0, ctas_per_sm = 0, nsm = 0;
  cudaStream_t cap_stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  bool planned = false, ran = false;
  double ms_last = 0.0, ms_autotune = 0.0;
  unsigned long long* d_prof = nullptr;  // per-phase cycle sums when profiling is on
  bool profiling = false;
  std::map<std::vector<int64_t>, std::pair<int, int>> tuned;  // batch signature -> (b, CTAs per SM)
};

namespace {

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct SlotLayout {
  int64_t off_R, off_V, off_Qc, off_Qr, off_diag, off_pbuf, off_stage, off_perm, bytes;
};

SlotLayout slot_layout(const std::vector<rbrp_batch_problem>& P, int kmax, int BB, int stage) {
  size_t a_res = 0, r = 0, v = 0, qr = 0, dg = 0, pm = 0;
  for (const auto& q : P) {
    const size_t ld = ((size_t)q.m + 3) & ~(size_t)3;
    const int mn = std::min(q.m, q.n);
    const size_t kc = kmax > 0 ? std::min(kmax, mn) : mn;
    a_res = std::max(a_res, ld * q.n * sizeof(float));
    r = std::max(r, kc * q.n * sizeof(float2));
    v = std::max(v, ld * BB * sizeof(float));
    qr = std::max(qr, (size_t)q.m * BB * sizeof(float));
    dg = std::max(dg, (size_t)q.n * sizeof(double));
    pm = std::max(pm, (size_t)q.n * sizeof(int));
  }
  SlotLayout L;
  size_t off = align256(a_res);
  L.off_R = off;
  off += align256(r);
  L.off_V = off;
  off += align256(v);
  L.off_Qc = off;
  off += align256(v);
  L.off_Qr = off;
  off += align256(qr);
  L.off_diag = off;
  off += align256(dg);
  L.off_pbuf = off;
  off += align256(2 * dg);
  L.off_stage = L.off_perm = 0;
  if (stage & STAGE_A) {
    L.off_stage = off;
    off += align256(a_res);
  }
  if (stage & STAGE_PERM) {
    L.off_perm = off;
    off += align256(pm);
  }
  L.bytes = off;
  return L;
}

template <int BB>
size_t batch_smem_bytes() {
  return sizeof(BatchSmem<BB>);
}

template <int BB>
cudaError_t set_batch_attr() {
  cudaError_t e = cudaFuncSetAttribute(k_rbrp_batched<BB, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)sizeof(BatchSmem<BB>));
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_rbrp_batched<BB, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)sizeof(BatchSmem<BB>));
}

int occupancy(int BB) {
  int nb = 0, nh = 0;
  if (BB == 16) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_rbrp_batched<16, false>, BT, sizeof(BatchSmem<16>));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nh, k_rbrp_batched<16, true>, BT, sizeof(BatchSmem<16>));
  } else {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_rbrp_batched<32, false>, BT, sizeof(BatchSmem<32>));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nh, k_rbrp_batched<32, true>, BT, sizeof(BatchSmem<32>));
  }
  return std::min(nb, nh);
}

template <int BB, bool HOST>
void launch_variant(BatchState& B, cudaStream_t s) {
  k_rbrp_batched<BB, HOST><<<B.grid, BT, sizeof(BatchSmem<BB>), s>>>(B.d_probs, B.d_order, B.nprob, B.d_queue,
                                                                      B.args, B.d_res);
}

cudaError_t launch(BatchState& B, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(B.d_queue, 0, sizeof(int), s);
  if (e != cudaSuccess) return e;
  const bool host = B.args.stage != 0;
  if (B.BB == 16)
    host ? launch_variant<16, true>(B, s) : launch_variant<16, false>(B, s);
  else
    host ? launch_variant<32, true>(B, s) : launch_variant<32, false>(B, s);
  return cudaGetLastError();
}

void drop_graph(BatchState& B) {
  if (B.exec) cudaGraphExecDestroy(B.exec);
  if (B.graph) cudaGraphDestroy(B.graph);
  B.exec = nullptr;
  B.graph = nullptr;
}

// Kernel variant and grid for block size b and a CTAs-per-SM request.
void configure(BatchState& B, int b, int cps, int max_grid) {
  B.BB = b <= 16 ? 16 : 32;
  B.args.b = b;
  const int occ = std::max(1, occupancy(B.BB));
  B.ctas_per_sm = std::min(cps, occ);
  B.grid = std::max(1, std::min({B.nprob, B.nsm * B.ctas_per_sm, max_grid}));
}

}  // namespace

void batch_release(rbrp_handle h) {
  BatchState* B = h->batch;
  if (!B) return;
  drop_graph(*B);
  if (B->cap_stream) cudaStreamDestroy(B->cap_stream);
  if (B->ev0) cudaEventDestroy(B->ev0);
  if (B->ev1) cudaEventDestroy(B->ev1);
  cudaFree(B->d_probs);
  cudaFree(B->d_order);
  cudaFree(B->d_res);
  cudaFree(B->d_queue);
  cudaFree(B->slots);
  cudaFree(B->d_prof);
  delete B;
  h->batch = nullptr;
}

}  // namespace rbrp

using namespace rbrp;

namespace {

// Where a problem buffer lives: 0 memory of this device (or managed), 1 pinned host
// memory (*dev = the address kernels use for it), -1 memory CUDA does not know
// (pageable), -2 memory of another device.
int residency(const void* p, const void** dev, int device) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  if (a.type == cudaMemoryTypeManaged) return 0;
  if (a.type == cudaMemoryTypeDevice) return a.device == device ? 0 : -2;
  if (a.type == cudaMemoryTypeHost) {
    if (!a.devicePointer) return -3;  // pinned, but not mapped into the device's address space
    *dev = a.devicePointer;
    return 1;
  }
  return -1;
}

rbrp_status batch_validate(rbrp_handle h, int nprob, const rbrp_batch_problem* problems, const rbrp_params* p) {
  if (!h) return RBRP_ERR_INVALID_ARG;
  if (nprob < 1 || !problems) return set_error(h, RBRP_ERR_INVALID_ARG, "empty batch");
  if (!p) return set_error(h, RBRP_ERR_INVALID_ARG, "params is NULL");
  if (p->b > BATCH_MAXB) return set_error(h, RBRP_ERR_INVALID_ARG, "the batched form takes b <= 32 (b <= 0: autotune)");
  if (!std::isfinite(p->tol) || !std::isfinite(p->tol_loc))
    return set_error(h, RBRP_ERR_INVALID_ARG, "tol and tol_loc must be finite");
  if (p->sampler < 0 || p->sampler > 2) return set_error(h, RBRP_ERR_INVALID_ARG, "unknown sampler");
  for (int q = 0; q < nprob; ++q) {
    const rbrp_batch_problem& r = problems[q];
    const std::string at = " (problem " + std::to_string(q) + ")";
    if (r.m < 1 || r.n < 1) return set_error(h, RBRP_ERR_INVALID_ARG, "m and n must be >= 1" + at);
    if (r.lda < r.m) return set_error(h, RBRP_ERR_INVALID_ARG, "lda < m" + at);
    if (!r.A || !r.perm) return set_error(h, RBRP_ERR_INVALID_ARG, "A and perm are required" + at);
    if (reinterpret_cast<uintptr_t>(r.A) % 4 || reinterpret_cast<uintptr_t>(r.perm) % 4 ||
        reinterpret_cast<uintptr_t>(r.T) % 8)
      return set_error(h, RBRP_ERR_INVALID_ARG, "misaligned pointer" + at);
    if (r.T_cap < 0) return set_error(h, RBRP_ERR_INVALID_ARG, "T_cap < 0" + at);
    if ((int64_t)r.m * r.n > ((int64_t)1 << 31)) return set_error(h, RBRP_ERR_INVALID_ARG, "problem too large" + at);
  }
  return RBRP_OK;
}

rbrp_status batch_alloc(rbrp_handle h, BatchState& B, size_t slot_bytes, int grid) {
  if (B.cap_probs < (size_t)B.nprob) {
    cudaFree(B.d_probs);
    cudaFree(B.d_order);
    cudaFree(B.d_res);
    B.d_probs = nullptr;
    B.d_order = nullptr;
    B.d_res = nullptr;
    B.cap_probs = 0;
    rbrp_status s = cuda_check(h, cudaMalloc(&B.d_probs, sizeof(rbrp_batch_problem) * B.nprob), "cudaMalloc(batch)");
    if (s == RBRP_OK) s = cuda_check(h, cudaMalloc(&B.d_order, sizeof(int) * B.nprob), "cudaMalloc(batch order)");
    if (s == RBRP_OK) s = cuda_check(h, cudaMalloc(&B.d_res, sizeof(rbrp_batch_result) * B.nprob), "cudaMalloc(batch results)");
    if (s != RBRP_OK) return s;
    B.cap_probs = B.nprob;
  }
  if (!B.d_queue) {
    rbrp_status s = cuda_check(h, cudaMalloc(&B.d_queue, sizeof(int)), "cudaMalloc(queue)");
    if (s != RBRP_OK) return s;
  }
  const size_t need = slot_bytes * (size_t)grid;
  if (B.slots_bytes < need) {
    cudaFree(B.slots);
    B.slots = nullptr;
    B.slots_bytes = 0;
    rbrp_status s = cuda_check(h, cudaMalloc(&B.slots, need), "cudaMalloc(batch workspace)");
    if (s != RBRP_OK) return s;
    B.slots_bytes = need;
  }
  return RBRP_OK;
}

}  // namespace

extern "C" {

rbrp_status rbrp_batch_plan(rbrp_handle h, int nprob, const rbrp_batch_problem* problems, const rbrp_params* p) {
  rbrp_status s = batch_validate(h, nprob, problems, p);
  if (s != RBRP_OK) return s;
  DeviceGuard g(h->device);
  if (!g.ok) return set_error(h, RBRP_ERR_CUDA, "cudaSetDevice failed");
  if (!h->batch) {
    h->batch = new (std::nothrow) BatchState();
    if (!h->batch) return RBRP_ERR_ALLOC;
    BatchState& B = *h->batch;
    if (cudaEventCreate(&B.ev0) != cudaSuccess || cudaEventCreate(&B.ev1) != cudaSuccess ||
        cudaStreamCreateWithFlags(&B.cap_stream, cudaStreamNonBlocking) != cudaSuccess) {
      cudaGetLastError();
      batch_release(h);
      return set_error(h, RBRP_ERR_CUDA, "batch events / capture stream");
    }
    cudaDeviceGetAttribute(&B.nsm, cudaDevAttrMultiProcessorCount, h->device);
    if (set_batch_attr<16>() != cudaSuccess || set_batch_attr<32>() != cudaSuccess) {
      cudaGetLastError();
      batch_release(h);
      return set_error(h, RBRP_ERR_CUDA, "cudaFuncSetAttribute(batched kernel)");
    }
  }
  BatchState& B = *h->batch;
  drop_graph(B);
  B.planned = false;
  B.ran = false;
  B.ms_autotune = 0.0;
  B.nprob = 0;
  B.probs.assign(problems, problems + nprob);
  // pinned host buffers are read and written in place through their device
  // addresses; a host A is staged into the workspace by the norms pass and a host
  // perm is kept in the workspace while its problem runs
  int stage = 0;
  for (int q = 0; q < nprob; ++q) {
    rbrp_batch_problem& r = B.probs[q];
    const std::string at = " (problem " + std::to_string(q) + ")";
    auto where_msg = [&](int where, const char* what) {
      return std::string(what) +
             (where == -2   ? " is memory of another device"
              : where == -3 ? " is pinned host memory that is not mapped for device access (register it "
                              "with cudaHostRegisterMapped, or allocate it with cudaHostAlloc)"
                            : " is neither device nor pinned host memory") +
             at;
    };
    const void* dev = r.A;
    int where = residency(r.A, &dev, h->device);
    if (where < 0) return set_error(h, RBRP_ERR_INVALID_ARG, where_msg(where, "A"));
    if (where == 1) stage |= STAGE_A;
    r.A = static_cast<const float*>(dev);
    dev = r.perm;
    where = residency(r.perm, &dev, h->device);
    if (where < 0) return set_error(h, RBRP_ERR_INVALID_ARG, where_msg(where, "perm"));
    if (where == 1) stage |= STAGE_PERM;
    r.perm = static_cast<int*>(const_cast<void*>(dev));
    if (r.T) {
      dev = r.T;
      where = residency(r.T, &dev, h->device);
      if (where < 0) return set_error(h, RBRP_ERR_INVALID_ARG, where_msg(where, "T"));
      r.T = static_cast<double*>(const_cast<void*>(dev));
    }
  }
  if (stage) stage = STAGE_A | STAGE_PERM;  // the host variant of the kernel stages both
  B.nprob = nprob;
  B.args.stage = stage;

  // largest problems first: the queue hands them out before the small ones
  std::vector<int> order(nprob);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return (int64_t)B.probs[a].m * B.probs[a].n > (int64_t)B.probs[b].m * B.probs[b].n;
  });

  B.args.tol = p->tol > 0.0 ? p->tol : 0.0;
  B.args.seed = p->seed;
  B.args.sampler = p->sampler;
  B.args.kmax = p->kmax;
  B.args.compute_T = p->compute_T;
  B.args.prof = B.profiling ? B.d_prof : nullptr;
  const SlotLayout L = slot_layout(B.probs, p->kmax, BATCH_MAXB, stage);
  B.args.off_R = L.off_R;
  B.args.off_V = L.off_V;
  B.args.off_Qc = L.off_Qc;
  B.args.off_Qr = L.off_Qr;
  B.args.off_diag = L.off_diag;
  B.args.off_pbuf = L.off_pbuf;
  B.args.off_stage = L.off_stage;
  B.args.off_perm = L.off_perm;
  B.args.slot_bytes = L.bytes;

  // grid bounded by the memory the slots may take (80% of what is free)
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  const size_t have = B.slots_bytes + free_b;
  const int max_grid = std::max<int64_t>(1, std::min<int64_t>((int64_t)(0.8 * (double)have / (double)L.bytes),
                                                              (int64_t)B.nsm * 4));
  const int occ_max = std::max(occupancy(16), occupancy(32));
  const int grid_cap = std::max(1, std::min({nprob, B.nsm * std::max(1, occ_max), max_grid}));
  s = batch_alloc(h, B, L.bytes, grid_cap);
  if (s != RBRP_OK) return s;
  B.args.slots = B.slots;
  cudaStream_t st = h->stream;
  s = cuda_check(h, cudaMemcpyAsync(B.d_probs, B.probs.data(), sizeof(rbrp_batch_problem) * nprob,
                                    cudaMemcpyHostToDevice, st), "copy batch");
  if (s == RBRP_OK)
    s = cuda_check(h, cudaMemcpyAsync(B.d_order, order.data(), sizeof(int) * nprob, cudaMemcpyHostToDevice, st),
                   "copy batch order");
  if (s == RBRP_OK) s = cuda_check(h, cudaStreamSynchronize(st), "batch upload");
  if (s != RBRP_OK) return s;

  if (p->b > 0) {
    B.args.tol_loc = p->tol_loc > 0.0 ? p->tol_loc : 1.0 / (double)p->b;
    configure(B, p->b, 2, grid_cap);
  } else {
    // autotuner: time each (b, CTAs per SM) candidate on this batch, keep the fastest
    int64_t tol_bits = 0, tol_loc_bits = 0;
    std::memcpy(&tol_bits, &p->tol, sizeof(double));
    std::memcpy(&tol_loc_bits, &p->tol_loc, sizeof(double));
    std::vector<int64_t> sig = {nprob, p->kmax, p->sampler, tol_bits, tol_loc_bits, p->compute_T, stage};
    int64_t sm = 0, sn = 0, smn = 0;
    for (const auto& q : B.probs) {
      sm += q.m;
      sn += q.n;
      smn += (int64_t)q.m * q.n;
    }
    sig.insert(sig.end(), {sm, sn, smn});
    auto it = B.tuned.find(sig);
    if (it != B.tuned.end()) {
      B.args.tol_loc = p->tol_loc > 0.0 ? p->tol_loc : 1.0 / (double)it->second.first;
      configure(B, it->second.first, it->second.second, grid_cap);
    } else {
      float best = 1e30f, total = 0.f;
      int best_b = 16, best_c = 2;
      for (int b : {8, 16, 24, 32}) {
        for (int cps : {1, 2, 3}) {
          if (cps > occupancy(b <= 16 ? 16 : 32)) continue;
          B.args.tol_loc = p->tol_loc > 0.0 ? p->tol_loc : 1.0 / (double)b;
          configure(B, b, cps, grid_cap);
          float ms = 0.f;
          for (int rep = 0; rep < 2; ++rep) {  // the first launch warms caches and clocks
            cudaEventRecord(B.ev0, st);
            s = cuda_check(h, launch(B, st), "batched kernel (autotune)");
            if (s != RBRP_OK) return s;
            cudaEventRecord(B.ev1, st);
            s = cuda_check(h, cudaEventSynchronize(B.ev1), "batched kernel (autotune)");
            if (s != RBRP_OK) return s;
            cudaEventElapsedTime(&ms, B.ev0, B.ev1);
            total += ms;
          }
          if (ms < best) {
            best = ms;
            best_b = b;
            best_c = cps;
          }
        }
      }
      B.tuned[sig] = {best_b, best_c};
      B.ms_autotune = total;
      B.args.tol_loc = p->tol_loc > 0.0 ? p->tol_loc : 1.0 / (double)best_b;
      configure(B, best_b, best_c, grid_cap);
    }
  }
  B.planned = true;
  return RBRP_OK;
}

rbrp_status rbrp_batch_run(rbrp_handle h) {
  if (!h) return RBRP_ERR_INVALID_ARG;
  if (!h->batch || !h->batch->planned) return set_error(h, RBRP_ERR_NOT_COMPUTED, "no batch planned");
  BatchState& B = *h->batch;
  DeviceGuard g(h->device);
  if (!B.exec) {  // capture queue reset + persistent kernel once per plan
    rbrp_status s = cuda_check(h, cudaStreamBeginCapture(B.cap_stream, cudaStreamCaptureModeThreadLocal),
                               "cudaStreamBeginCapture");
    if (s != RBRP_OK) return s;
    const cudaError_t le = launch(B, B.cap_stream);
    const cudaError_t ce = cudaStreamEndCapture(B.cap_stream, &B.graph);
    s = cuda_check(h, le != cudaSuccess ? le : ce, "batch graph capture");
    if (s != RBRP_OK) {
      drop_graph(B);
      return s;
    }
    s = cuda_check(h, cudaGraphInstantiate(&B.exec, B.graph, 0), "cudaGraphInstantiate");
    if (s != RBRP_OK) {
      drop_graph(B);
      return s;
    }
  }
  cudaEventRecord(B.ev0, h->stream);
  rbrp_status s = cuda_check(h, cudaGraphLaunch(B.exec, h->stream), "cudaGraphLaunch(batch)");
  if (s != RBRP_OK) return s;
  cudaEventRecord(B.ev1, h->stream);
  B.ran = true;
  return RBRP_OK;
}

rbrp_status rbrp_batch_results(rbrp_handle h, rbrp_batch_result* out, int cap) {
  if (!h) return RBRP_ERR_INVALID_ARG;
  if (!h->batch || !h->batch->ran) return set_error(h, RBRP_ERR_NOT_COMPUTED, "no batch run");
  BatchState& B = *h->batch;
  DeviceGuard g(h->device);
  rbrp_status s = cuda_check(h, cudaEventSynchronize(B.ev1), "batched kernel");
  if (s != RBRP_OK) return s;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, B.ev0, B.ev1);
  B.ms_last = ms;
  if (out) {
    if (cap < B.nprob) return set_error(h, RBRP_ERR_CAPACITY, "result array smaller than the batch");
    s = cuda_check(h, cudaMemcpy(out, B.d_res, sizeof(rbrp_batch_result) * B.nprob, cudaMemcpyDeviceToHost),
                   "copy batch results");
  }
  return s;
}

rbrp_status rbrp_batch_set_order(rbrp_handle h, const int* order, int n) {
  if (!h) return RBRP_ERR_INVALID_ARG;
  if (!h->batch || !h->batch->planned) return set_error(h, RBRP_ERR_NOT_COMPUTED, "no batch planned");
  BatchState& B = *h->batch;
  if (!order || n != B.nprob) return set_error(h, RBRP_ERR_INVALID_ARG, "order must list every problem once");
  std::vector<char> seen(n, 0);
  for (int q = 0; q < n; ++q) {
    if (order[q] < 0 || order[q] >= n || seen[order[q]])
      return set_error(h, RBRP_ERR_INVALID_ARG, "order must list every problem once");
    seen[order[q]] = 1;
  }
  DeviceGuard g(h->device);
  // the graph reads the order from device memory at run time: no new capture needed
  rbrp_status s = cuda_check(h, cudaMemcpyAsync(B.d_order, order, sizeof(int) * n, cudaMemcpyHostToDevice, h->stream),
                             "copy batch order");
  if (s == RBRP_OK) s = cuda_check(h, cudaStreamSynchronize(h->stream), "copy batch order");
  return s;
}

rbrp_status rbrp_batch_get_info(rbrp_handle h, rbrp_batch_info* info) {
  if (!h || !info) return RBRP_ERR_INVALID_ARG;
  if (!h->batch || !h->batch->planned) return set_error(h, RBRP_ERR_NOT_COMPUTED, "no batch planned");
  const BatchState& B = *h->batch;
  info->b = B.args.b;
  info->panel_cols = B.BB;
  info->ctas = B.grid;
  info->ctas_per_sm = B.ctas_per_sm;
  info->ms_last = B.ms_last;
  info->ms_autotune = B.ms_autotune;
  info->workspace_bytes = B.slots_bytes;
  return RBRP_OK;
}

rbrp_status rbrp_batch_set_profiling(rbrp_handle h, int on) {
  if (!h) return RBRP_ERR_INVALID_ARG;
  if (!h->batch || !h->batch->planned) return set_error(h, RBRP_ERR_NOT_COMPUTED, "no batch planned");
  BatchState& B = *h->batch;
  DeviceGuard g(h->device);
  if (on && !B.d_prof) {
    rbrp_status s = cuda_check(h, cudaMalloc(&B.d_prof, sizeof(unsigned long long) * BPH_N), "cudaMalloc(profile)");
    if (s != RBRP_OK) return s;
  }
  B.profiling = on != 0;
  B.args.prof = B.profiling ? B.d_prof : nullptr;
  drop_graph(B);  // the kernel arguments changed: capture again
  if (B.profiling) return cuda_check(h, cudaMemset(B.d_prof, 0, sizeof(unsigned long long) * BPH_N), "profile reset");
  return RBRP_OK;
}

rbrp_status rbrp_batch_get_phase_cycles(rbrp_handle h, double* cycles, int cap) {
  if (!h || !cycles || cap < RBRP_BATCH_NPHASES) return RBRP_ERR_INVALID_ARG;
  if (!h->batch || !h->batch->d_prof) return set_error(h, RBRP_ERR_NOT_COMPUTED, "batch profiling is off");
  DeviceGuard g(h->device);
  unsigned long long c[BPH_N];
  rbrp_status s = cuda_check(h, cudaMemcpy(c, h->batch->d_prof, sizeof(c), cudaMemcpyDeviceToHost), "copy profile");
  for (int q = 0; q < BPH_N; ++q) cycles[q] = (double)c[q];
  return s;
}

rbrp_status rbrp_id_batched_f32(rbrp_handle h, int nprob, const rbrp_batch_problem* problems, const rbrp_params* p,
                                rbrp_batch_result* out) {
  rbrp_status s = rbrp_batch_plan(h, nprob, problems, p);
  if (s == RBRP_OK) s = rbrp_batch_run(h);
  if (s == RBRP_OK) s = rbrp_batch_results(h, out, nprob);
  return s;
}

}  // extern "C"
