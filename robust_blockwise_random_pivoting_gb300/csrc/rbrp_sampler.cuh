// rbrp_sampler.cuh - block-wide weighted sampler of one RBRP block.
//
// Shared by the one-matrix kernel (k_sample, 1024 threads) and the batched
// persistent kernel (one CTA per problem).  All state is read from and
// written to a State that may live in global or shared memory.
#pragma once
#include "rbrp_common.cuh"

namespace rbrp {
namespace {

// ===========================================================================
// a2: block sampler.  One CTA over the n - i remaining positions.
// NP: numpy Generator.choice(replace=False, p=w/sum(w)) rounds (python/RBRP.ipynb
//     cell 11 line 108): uniforms from the Philox np-compat stream, cdf by a
//     block scan, searchsorted(side='right') by binary search, first occurrences
//     kept in draw order.  (The reference CUDA sampler draws WITH replacement
//     and may return fewer indices, gpu/rbrp.cu:102-146.)
// ES: keys -log(1-u)/w (u from the exponential-key stream of the original
//     column), the bs smallest by an 8-bit radix select on the key bits.
// GREEDY: the bs largest weights (ties: lower position), same radix select.
// GIVEN: a fixed skeleton: the bs listed columns that come first in the list
//     (order_of[col] = list index, -1 for unlisted), same radix select.
// ===========================================================================
constexpr int SAMPLE_THREADS = 1024;

// Block-wide sampler body (any block size from 64 to MAXT); k_sample runs it with
// 1024 threads, the batched kernel with its CTA.
template <int MAXT = SAMPLE_THREADS>
__device__ void sample_block(State* st, const double* __restrict__ diags, const int* __restrict__ perm, int n,
                             int kmax, int b, uint64_t seed, int sampler, double* __restrict__ pbuf,
                             unsigned long long* __restrict__ kbuf, int* __restrict__ js, int* __restrict__ cols,
                             const int* __restrict__ order_of = nullptr) {
  __shared__ double shd[32];
  __shared__ int shi[32];
  __shared__ unsigned int hist[256];
  __shared__ int s_rel[MAXB];
  __shared__ int s_cand[MAXB];
  __shared__ unsigned long long s_key[MAXB];
  __shared__ int s_found, s_size, s_digit, s_krank, s_i, s_done;
  __shared__ unsigned long long s_draws;
  const int tid = threadIdx.x;
  if (tid == 0) {
    s_done = st->done;
    s_i = st->i;
    s_draws = st->draws;
  }
  __syncthreads();
  if (s_done) return;
  const int i = s_i;
  const int nrem = n - i;
  const int req = min(min(kmax - i, b), st->nnz_rem);
  const int chunk = (nrem + (int)blockDim.x - 1) / (int)blockDim.x;
  const int lo = min(nrem, tid * chunk), hi = min(nrem, lo + chunk);
  const double* w = diags + i;

  if (sampler == SAMPLER_NP) {
    // p = w / sum(w)
    double part = 0.0;
    for (int j = lo; j < hi; ++j) part += w[j];
    const double S = block_sum(part, shd);
    // one FP64 division for the block, shared: per-thread or per-entry divisions are
    // ~1/64-rate work on GB300
    __shared__ double s_invS;
    if (tid == 0) s_invS = 1.0 / S;
    __syncthreads();
    const double invS = s_invS;
    int npos = 0;
    for (int j = lo; j < hi; ++j) {
      const double pj = w[j] * invS;
      pbuf[j] = pj;
      npos += pj > 0.0;
    }
    npos = block_sum(npos, shi);
    if (tid == 0) {
      s_size = min(req, npos);
      s_found = 0;
    }
    // The cdf is never stored.  Thread t's chunk [lo, hi) keeps its total `tot`; the
    // block scan of the totals gives its offset; cdf(j) = (off + run(j)) * (1 / last),
    // run(j) the chunk-local sequential sum, last = off + tot of the chunk holding
    // index nrem - 1, whose cdf is exactly 1 (numpy's cdf /= cdf[-1]).  A draw
    // binary-searches the chunks' last cdf entries in shared memory, then scans one
    // chunk: the index searchsorted(side='right') returns on the stored cdf.
    __shared__ double s_end[MAXT];
    __shared__ double s_off[MAXT];
    __shared__ double s_last, s_inv_last;
    double tot = 0.0;
    __syncthreads();
    // Rejection rounds.  Each round draws at least one new index unless every
    // remaining positive weight is absorbed by rounding in the cdf; the cap
    // turns that (pathological) case into a smaller sample instead of a spin.
    for (int round = 0; s_found < s_size && round < 4096; ++round) {
      const int found = s_found, need = s_size - s_found;
      if (tid < found) pbuf[s_rel[tid]] = 0.0;
      __syncthreads();
      // chunk totals: every chunk in the first round, afterwards the chunks holding a drawn index
      bool dirty = round == 0;
      for (int u = 0; u < found && !dirty; ++u) {
        const int jr = s_rel[u];
        dirty = jr >= lo && jr < hi;
      }
      if (dirty) {
        double run = 0.0;
        int j = lo;
        for (; j + 8 <= hi; j += 8) {
          double v[8];
#pragma unroll
          for (int q = 0; q < 8; ++q) v[q] = pbuf[j + q];
#pragma unroll
          for (int q = 0; q < 8; ++q) run += v[q];
        }
        for (; j < hi; ++j) run += pbuf[j];
        tot = run;
      }
      const double off = block_exclusive_scan(tot, shd, (double*)nullptr);
      if (lo < hi && hi == nrem) {
        s_last = off + tot;
        s_inv_last = 1.0 / s_last;  // once, by the thread holding the last chunk
      }
      s_off[tid] = off;
      __syncthreads();
      const double inv_last = s_inv_last;
      s_end[tid] = lo < hi ? (hi == nrem ? 1.0 : (off + tot) * inv_last) : 2.0;
      __syncthreads();
      if (tid < need) {
        const double x = np_uniform(seed, s_draws + (unsigned long long)tid);
        int a = 0, z = (int)blockDim.x;  // first chunk whose last cdf entry is > x
        while (a < z) {
          const int mid = (a + z) >> 1;
          if (s_end[mid] <= x) a = mid + 1; else z = mid;
        }
        const int t = min(a, (int)blockDim.x - 1);
        const int clo = min(nrem, t * chunk), chi = min(nrem, clo + chunk);
        const double co = s_off[t];
        int pick = chi - 1;
        double run = 0.0;
        bool hit = false;
        for (int j0 = clo; j0 < chi && !hit; j0 += 8) {
          double v[8];
#pragma unroll
          for (int q = 0; q < 8; ++q) v[q] = j0 + q < chi ? pbuf[j0 + q] : 0.0;
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const int j = j0 + q;
            if (!hit && j < chi) {
              run += v[q];
              const double c = j == nrem - 1 ? 1.0 : (co + run) * inv_last;
              if (c > x) {
                pick = j;
                hit = true;
              }
            }
          }
        }
        s_cand[tid] = pick < nrem ? pick : nrem - 1;
      }
      __syncthreads();
      if (tid == 0) {
        int f = found;
        for (int t = 0; t < need; ++t) {
          const int c = s_cand[t];
          bool dup = false;
          for (int u = 0; u < t; ++u) dup |= (s_cand[u] == c);
          if (!dup) s_rel[f++] = c;
        }
        s_found = f;
        s_draws += (unsigned long long)need;
      }
      __syncthreads();
    }
    if (tid == 0) s_size = s_found;
    __syncthreads();
  } else {
    // keys (ascending = preferred); each thread also keeps its smallest (key, position)
    int npos = 0;
    unsigned long long bk = ~0ull;
    int bj = 0x7fffffff;
    for (int j = lo; j < hi; ++j) {
      const double wj = w[j];
      unsigned long long key = ~0ull;
      if (sampler == SAMPLER_GIVEN) {
        // fixed skeleton: columns of the list (order_of[col] >= 0), earliest first
        const int o = order_of[perm[i + j]];
        if (wj > 0.0 && o >= 0) {
          ++npos;
          key = (unsigned long long)o;
        }
      } else if (wj > 0.0) {
        ++npos;
        if (sampler == SAMPLER_ES) {
          const double u = es_uniform(seed, (uint64_t)st->attempts, (uint64_t)perm[i + j]);
          const double e = -log(1.0 - u) / wj;
          key = (unsigned long long)__double_as_longlong(e);
        } else {
          key = 0x7FF0000000000000ull - (unsigned long long)__double_as_longlong(wj);
        }
      }
      kbuf[j] = key;
      if (key < bk) bk = key, bj = j;
    }
    npos = block_sum(npos, shi);
    const int size = min(req, npos);
    if (size == 1) {
      // one index (greedy b = 1 is column-pivoted QR): argmin of (key, position),
      // the element the radix select below would return
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long ok = __shfl_xor_sync(0xffffffffu, bk, o);
        const int oj = __shfl_xor_sync(0xffffffffu, bj, o);
        if (ok < bk || (ok == bk && oj < bj)) bk = ok, bj = oj;
      }
      if ((tid & 31) == 0) {
        s_key[tid >> 5] = bk;
        s_cand[tid >> 5] = bj;
      }
      __syncthreads();
      if (tid == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
          if (s_key[w] < s_key[0] || (s_key[w] == s_key[0] && s_cand[w] < s_cand[0])) s_key[0] = s_key[w], s_cand[0] = s_cand[w];
        s_rel[0] = s_cand[0];
        s_size = 1;
        s_found = 1;
      }
      __syncthreads();
    } else {
      // radix select of the size-th smallest key
      unsigned long long prefix = 0ull, mask = 0ull;
      int krank = size;
      for (int shift = 56; shift >= 0 && size > 0; shift -= 8) {
        for (int d = tid; d < 256; d += blockDim.x) hist[d] = 0u;
        __syncthreads();
        for (int j = lo; j < hi; ++j) {
          const unsigned long long k = kbuf[j];
          if ((k & mask) == prefix) atomicAdd(&hist[(k >> shift) & 0xFF], 1u);
        }
        __syncthreads();
        if (tid == 0) {
          int cum = 0, d = 0;
          for (; d < 255; ++d) {
            if (cum + (int)hist[d] >= krank) break;
            cum += (int)hist[d];
          }
          s_digit = d;
          s_krank = krank - cum;
        }
        __syncthreads();
        prefix |= (unsigned long long)s_digit << shift;
        mask |= 0xFFull << shift;
        krank = s_krank;
        __syncthreads();
      }
      const unsigned long long kth = prefix;
      int nlt = 0, neq = 0;
      for (int j = lo; j < hi; ++j) {
        const unsigned long long k = kbuf[j];
        nlt += k < kth;
        neq += k == kth;
      }
      int tot_lt, tot_eq;
      const int off_lt = block_exclusive_scan(nlt, shi, &tot_lt);
      const int off_eq = block_exclusive_scan(neq, shi, &tot_eq);
      const int ties = size - tot_lt;
      int a = off_lt, e = off_eq;
      if (size > 0) {
        for (int j = lo; j < hi; ++j) {
          const unsigned long long k = kbuf[j];
          if (k < kth) {
            s_key[a] = k;
            s_cand[a] = j;
            ++a;
          } else if (k == kth) {
            if (e < ties) {
              s_key[tot_lt + e] = k;
              s_cand[tot_lt + e] = j;
            }
            ++e;
          }
        }
      }
      __syncthreads();
      if (tid < size) {
        const unsigned long long k = s_key[tid];
        const int j = s_cand[tid];
        int rank = 0;
        for (int u = 0; u < size; ++u) {
          const unsigned long long ku = s_key[u];
          rank += (ku < k) || (ku == k && s_cand[u] < j);
        }
        s_rel[rank] = j;
      }
      if (tid == 0) {
        s_size = size;
        s_found = size;
      }
      __syncthreads();
    }
  }
  const int size = s_size;
  if (tid < size) {
    const int p = i + s_rel[tid];
    js[tid] = p;
    cols[tid] = perm[p];
  }
  if (tid == 0) {
    st->bs_sampled = size;
    st->draws = s_draws;
  }
  __syncthreads();
}

}  // namespace
}  // namespace rbrp
