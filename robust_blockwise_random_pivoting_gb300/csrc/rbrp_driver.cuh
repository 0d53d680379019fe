// rbrp_driver.cuh - host loop of adaptive RBRP (instantiated per element type).
//
// One adaptive block per iteration, all sizes read by the kernels from the
// device-resident State; the host reads the 80-byte State back once per block
// (pinned memory) to learn whether to continue.  Follows the control flow of
// RBRP() in gpu/rbrp.cu:333-503 and blocked_rpid in python/RBRP.ipynb cell 11
// lines 76-173, with the stopping rule of cell 11 line 164 (squared tol).
#pragma once
#include <algorithm>
#include <type_traits>

#include "rbrp_internal.h"
#include "rbrp_kernels.cuh"
#include "rbrp_panel_df.cuh"
#include "rbrp_tc.cuh"
#include "rbrp_update_tc.cuh"

namespace rbrp {

template <typename T>
rbrp_status run_rbrp(rbrp_handle h, int m, int n, const T* dA, int64_t lda, const rbrp_params& p,
                     int* dPerm, rbrp_result* out) {
  // FP64: the notebook's implicit form (projections of A, downdated norms) -
  // the parity path.  FP32: the explicit residual form (see k_proj_w).
  constexpr bool RES = sizeof(T) == sizeof(float);
  const int kmax = p.kmax > 0 ? std::min(p.kmax, std::min(m, n)) : std::min(m, n);
  const Layout L = make_layout(m, n, kmax, sizeof(T), RES);
  rbrp_status s = ensure_workspace(h, L);
  if (s != RBRP_OK) return s;
  {  // function attributes are per device context: set them on every call (cheap)
    for (const void* fn : {(const void*)k_pchol, (const void*)k_panel1, (const void*)k_chol2}) {
      s = cuda_check(h, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(PanelSmem)),
                     "cudaFuncSetAttribute(panel)");
      if (s != RBRP_OK) return s;
    }
    s = cuda_check(h, cudaFuncSetAttribute(k_panel2<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)sizeof(PanelSmem)), "cudaFuncSetAttribute(k_panel2)");
    if (s != RBRP_OK) return s;
    if (RES) {
      s = cuda_check(h, cudaFuncSetAttribute(k_pchol_df, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)sizeof(PcholDfSmem)), "cudaFuncSetAttribute(panel df)");
      if (s != RBRP_OK) return s;
      s = cuda_check(h, cudaFuncSetAttribute(k_panel_q_df, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)sizeof(QSolveSmem)), "cudaFuncSetAttribute(basis df)");
      if (s != RBRP_OK) return s;
      s = cuda_check(h, cudaFuncSetAttribute(k_resid_update, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)P2_SMEM), "cudaFuncSetAttribute(k_resid_update)");
      if (s != RBRP_OK) return s;
      s = cuda_check(h, cudaFuncSetAttribute(tc::k_proj_w_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)tc::PROJ_SMEM), "cudaFuncSetAttribute(k_proj_w_tc)");
      if (s != RBRP_OK) return s;
      s = cuda_check(h, cudaFuncSetAttribute(tc::k_resid_update_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)tc::U_SMEM), "cudaFuncSetAttribute(k_resid_update_tc)");
      if (s != RBRP_OK) return s;
    }
  }
  cudaStream_t st = h->stream;
  const bool use_tc = RES && h->variant == 0;
  CUtensorMap tmA, tmQ, tmWth, tmWtl, tmQrh, tmQrl;
  if (use_tc) {  // TMA views: A_res (m x n) and the split basis (m x 64), boxes of 32 rows; for the
                 // update, W^T (64 per position, boxes of 64 positions) and the basis by rows (boxes of 128)
    s = make_tmap_f32(h, &tmA, h->Ares, m, n, L.ld_res, tc::BK, tc::BM);
    // the split basis: Qh and Ql are adjacent workspace arrays (ld_res x 64 each), viewed as
    // one m x 128 array so that one box fetches a stage's hi and lo tiles
    if (h->Ql != h->Qh + L.ld_res * MAXB) return set_error(h, RBRP_ERR_INVALID_ARG, "basis hi / lo arrays not adjacent");
    if (s == RBRP_OK) s = make_tmap_f32(h, &tmQ, h->Qh, m, 2 * MAXB, L.ld_res, tc::BK, 2 * tc::BN);
    if (s == RBRP_OK) s = make_tmap_f32(h, &tmWth, h->Wth, MAXB, n, MAXB, tc::BK, tc::U_POS);
    if (s == RBRP_OK) s = make_tmap_f32(h, &tmWtl, h->Wtl, MAXB, n, MAXB, tc::BK, tc::U_POS);
    if (s == RBRP_OK) s = make_tmap_f32(h, &tmQrh, h->Qrh, MAXB, m, MAXB, tc::BK, tc::U_ROWS);
    if (s == RBRP_OK) s = make_tmap_f32(h, &tmQrl, h->Qrl, MAXB, m, MAXB, tc::BK, tc::U_ROWS);
    if (s != RBRP_OK) return s;
    cudaMemsetAsync(h->Qh, 0, (size_t)L.ld_res * MAXB * sizeof(float), st);
    cudaMemsetAsync(h->Ql, 0, (size_t)L.ld_res * MAXB * sizeof(float), st);
  }
  T* Q = static_cast<T*>(h->Q);
  T* Cpart = static_cast<T*>(h->Cpart);
  T* C = static_cast<T*>(h->C);
  const double tol = p.tol > 0.0 ? p.tol : 0.0;
  const double tol_loc = p.tol_loc > 0.0 ? p.tol_loc : 1.0 / (double)p.b;
  const int ntiles = L.ntiles;
  const size_t panel_smem = sizeof(PanelSmem);
  h->have_result = false;

  const double es = (double)sizeof(T), dm = (double)m;
  h->marks.clear();
  h->prof_next = 0;
  cudaEventRecord(h->ev_start, st);
  cudaMemsetAsync(h->st, 0, sizeof(State), st);
  int ev = prof_begin(h);
  if (RES)  // the residual starts as A, in position (= column) order
    cudaMemcpy2DAsync(h->Ares, (size_t)L.ld_res * sizeof(float), dA, (size_t)lda * sizeof(T), (size_t)m * sizeof(T),
                      n, cudaMemcpyDeviceToDevice, st);
  k_colnorm<T><<<(n + 7) / 8, 256, 0, st>>>(dA, lda, m, n, h->diags, h->perm, h->st);
  k_init<<<1, 1024, 0, st>>>(h->st, h->diags, n, kmax);
  prof_end(h, RBRP_PHASE_NORMS, ev, (RES ? 3.0 : 1.0) * dm * n * es + 16.0 * n, 2.0 * dm * n, RES ? 3 : 2);
  cudaMemcpyAsync(h->hst, h->st, sizeof(State), cudaMemcpyDeviceToHost, st);
  s = cuda_check(h, cudaStreamSynchronize(st), "initial column norms");
  if (s != RBRP_OK) return s;
  if (h->hst->status) return set_error(h, RBRP_ERR_NUMERIC, "non-finite entries in A");

  const int max_attempts = 4 * kmax + 64;
  std::vector<int> attempt_of_block;
  attempt_of_block.reserve(kmax);
  int attempts = 0, nb_host = 0;
  while (!h->hst->done) {
    if (attempts >= max_attempts)
      return set_error(h, RBRP_ERR_NUMERIC, "no progress: block attempts exceeded 4*kmax+64");
    const int i = h->hst->i;
    const size_t mark0 = h->marks.size();
    ev = prof_begin(h);
    k_sample<<<1, SAMPLE_THREADS, 0, st>>>(h->st, h->diags, h->perm, n, kmax, p.b, p.seed, p.sampler,
                                           h->pbuf, h->kbuf, h->js, h->cols, h->given_order);
    prof_end(h, RBRP_PHASE_SAMPLE, ev, 28.0 * (n - i), 0.0, 1);
    ev = prof_begin(h);
    if (!RES && i > 0) {
      const int tiles = (i + 31) / 32;
      int splits = splits_for(i, m);
      int rps = ((m + splits - 1) / splits + 31) / 32 * 32;
      splits = (m + rps - 1) / rps;
      k_cgs_coef<T><<<dim3(tiles, 1, splits), 256, 0, st>>>(Q, m, dA, lda, h->cols, h->st, m, rps,
                                                             (int64_t)i * MAXB, Cpart);
      const int64_t cnt = (int64_t)i * MAXB;
      k_reduce_parts<T><<<(int)std::min<int64_t>(1024, (cnt + 255) / 256), 256, 0, st>>>(Cpart, splits, cnt, cnt, C);
    }
    const int dtiles = (m + DF_ROWS - 1) / DF_ROWS;   // row tiles of the double-float Gram kernel
    if (RES) {  // panel = residual columns at the sampled positions (FP32, exact), Gram in double-float
      k_gram_df<<<dtiles, 256, 0, st>>>(h->Ares, L.ld_res, h->js, h->st, m, (float*)h->V, h->Gpart);
      k_reduce_parts<double><<<16, 256, 0, st>>>(h->Gpart, dtiles, MAXB * MAXB, MAXB * MAXB, h->G);
    } else {
      k_cgs_update<T><<<ntiles, 256, 0, st>>>(dA, lda, h->cols, Q, m, C, h->st, m, h->V, h->Gpart, 1);
      k_reduce_parts<double><<<16, 256, 0, st>>>(h->Gpart, ntiles, MAXB * MAXB, MAXB * MAXB, h->G);
    }
    prof_end(h, RBRP_PHASE_CGS, ev, 0.0, 0.0, (!RES && i > 0) ? 4 : 2);
    ev = prof_begin(h);
    if (RES) {
      // R11 and its inverse as double-float pairs: the FP64 R11 / R2 buffers of the same
      // size (R2 serves only the FP64 form's second CholQR pass), reinterpreted
      float2* R11df = reinterpret_cast<float2*>(h->R11);
      float2* Rinvdf = reinterpret_cast<float2*>(h->R2);
      k_pchol_df<<<1, LEAN_THREADS, sizeof(PcholDfSmem), st>>>(h->G, m, h->st, tol_loc, h->js, h->perm, h->diags,
                                                               R11df, Rinvdf, h->ord, h->J, h->K1, h->K2);
      k_panel_q_df<<<(m + QS_ROWS - 1) / QS_ROWS, 256, sizeof(QSolveSmem), st>>>(
          (const float*)h->V, m, h->st, Rinvdf, h->ord, (float*)Q, L.ld_res, use_tc ? h->Qh : nullptr,
          use_tc ? h->Ql : nullptr, L.ld_res, use_tc ? h->Qrh : nullptr, use_tc ? h->Qrl : nullptr);
      k_write_r11<<<1, 256, 0, st>>>(h->st, R11df, h->R, n);
    } else {
      k_pchol<<<1, 256, panel_smem, st>>>(h->G, m, h->st, tol_loc, h->js, h->perm, h->diags, h->R11, h->ord,
                                          h->J, h->K1, h->K2);
      k_panel1<<<ntiles, 256, panel_smem, st>>>(h->V, m, h->st, h->R11, h->ord, h->Q1, h->G2part);
      k_reduce_parts<double><<<16, 256, 0, st>>>(h->G2part, ntiles, MAXB * MAXB, MAXB * MAXB, h->G2);
      k_chol2<<<1, 256, panel_smem, st>>>(h->G2, h->st, h->R11, h->R2, h->R, n);
    }
    if (i > 0) k_swap_R<<<(i + 127) / 128, 128, 0, st>>>(h->R, n, h->st, h->J, h->K1, h->K2);
    if (RES)
      k_swap_cols<<<dim3((m + 1023) / 1024, MAXB), 256, 0, st>>>(h->Ares, L.ld_res, h->st, m, h->K1, h->K2);
    if (!RES) k_panel2<T><<<ntiles, 256, panel_smem, st>>>(h->Q1, m, h->st, h->R2, Q, m, 1);
    prof_end(h, RBRP_PHASE_PANEL, ev, 0.0, 0.0, RES ? (i > 0 ? 5 : 4) : (i > 0 ? 6 : 5));
    int nproj;
    ev = prof_begin(h);
    if (RES) {
      int wsplit = 0;
      if (use_tc) {
        // row split: one CTA per SM fits (shared memory), so the launch runs in
        // ceil(ctiles * split / SMs) waves of sps stages each plus a fixed cost per CTA
        // (TMEM allocation, pipeline fill and final drains: about 4 stages); take the
        // split with the least wave time (the smallest on ties: fewer partials to sum)
        const int ctiles = (n - i + tc::BM - 1) / tc::BM;
        const int nstages = (m + tc::BK - 1) / tc::BK;
        const int maxsplit = std::min(P1_MAX_SPLIT, std::max(1, nstages / tc::CHUNK));
        int sps = nstages;
        wsplit = 1;
        long best = -1;
        for (int w = 1; w <= maxsplit; ++w) {
          const int s_w = (nstages + w - 1) / w;
          const int ws = (nstages + s_w - 1) / s_w;
          const long waves = ((long)ctiles * ws + h->sms - 1) / h->sms;
          const long cost = waves * (s_w + 4);
          if (best < 0 || cost < best) {
            best = cost;
            wsplit = ws;
            sps = s_w;
          }
        }
        tc::k_proj_w_tc<<<dim3(ctiles, wsplit), tc::NTHREADS, tc::PROJ_SMEM, st>>>(
            tmA, tmQ, h->st, m, n, sps, reinterpret_cast<float2*>(h->Wpart),
            h->wait_budget > 0 ? h->wait_budget : kWaitBudgetDefault);
      } else {
        k_proj_w<<<(n - i + 63) / 64, 128, 0, st>>>((const float*)Q, L.ld_res, h->Ares, L.ld_res, h->st, m, n, h->R,
                                                    n);
      }
      prof_end(h, RBRP_PHASE_PROJECT, ev, 0.0, 0.0, 1);
      ev = prof_begin(h);
      int nsplit = 1;
      if (use_tc) {
        // W^T parts (and R(I2, p)), then the tensor-core update.  Row split by the wave rule
        // with one CTA per SM (shared memory) and a fixed cost per CTA of about two chunks
        // (TMEM allocation, the W^T tile, pipeline fill and drain)
        tc::k_upd_w_prep<<<(n - i + 31) / 32, 256, 0, st>>>(h->st, n, reinterpret_cast<const float2*>(h->Wpart),
                                                            wsplit, h->R, n, h->Wth, h->Wtl);
        const int ctiles = (n - i + tc::U_POS - 1) / tc::U_POS;
        int rps = (m + tc::U_ROWS - 1) / tc::U_ROWS * tc::U_ROWS;
        long best = -1;
        for (int w = 1; w <= P2_MAX_SPLIT_WS; ++w) {
          const int r_w = ((m + w - 1) / w + tc::U_ROWS - 1) / tc::U_ROWS * tc::U_ROWS;
          const int ws = (m + r_w - 1) / r_w;
          const long waves = ((long)ctiles * ws + h->sms - 1) / h->sms;
          const long cost = waves * (r_w / tc::U_ROWS + 2);
          if (best < 0 || cost < best) {
            best = cost;
            nsplit = ws;
            rps = r_w;
          }
        }
        tc::k_resid_update_tc<<<dim3(ctiles, nsplit), tc::U_THREADS, tc::U_SMEM, st>>>(
            tmWth, tmWtl, tmQrh, tmQrl, h->st, h->Ares, L.ld_res, m, n, rps, h->part_norm,
            h->wait_budget > 0 ? h->wait_budget : kWaitBudgetDefault);
      } else {
        const int ctiles = (n - i + P2_COLS - 1) / P2_COLS;
        // row split by the same wave rule, two CTAs per SM (registers and shared memory), with
        // a fixed cost per CTA of about two stages (W staging, norm partials)
        int rps = (m + P2_ROWS - 1) / P2_ROWS * P2_ROWS;
        long best = -1;
        for (int w = 1; w <= P2_MAX_SPLIT; ++w) {
          const int r_w = ((m + w - 1) / w + P2_ROWS - 1) / P2_ROWS * P2_ROWS;
          const int ws = (m + r_w - 1) / r_w;
          const long waves = ((long)ctiles * ws + 2 * h->sms - 1) / (2 * h->sms);
          const long cost = waves * (r_w + 2 * P2_ROWS);
          if (best < 0 || cost < best) {
            best = cost;
            nsplit = ws;
            rps = r_w;
          }
        }
        k_resid_update<<<dim3(ctiles, nsplit), P2_THREADS, P2_SMEM, st>>>((const float*)Q, L.ld_res, h->Ares,
                                                                         L.ld_res, h->st, m, n, rps, h->R, n,
                                                                         h->part_norm);
      }
      nproj = (n - i + 255) / 256;
      k_norm_reduce<<<nproj, 256, 0, st>>>(h->part_norm, nsplit, n, h->st, h->diags, h->part_res, h->part_nnz);
      prof_end(h, RBRP_PHASE_UPDATE, ev, 0.0, 0.0, use_tc ? 3 : 2);
    } else {
      // basis tile height: the smallest KB >= b (kept <= b); b <= 8 takes the column-streaming form
      auto project = [&](auto kb) {
        constexpr int KB = decltype(kb)::value;
        nproj = (n - i + ProjTile<KB>::PC - 1) / ProjTile<KB>::PC;
        k_project<T, KB><<<nproj, 256, 0, st>>>(Q, m, dA, lda, h->perm, h->st, m, n, h->R, n, h->diags,
                                                h->part_res, h->part_nnz);
      };
      auto skinny = [&](auto kb) {
        constexpr int KB = decltype(kb)::value;
        nproj = (n - i + SKINNY_COLS - 1) / SKINNY_COLS;
        k_project_skinny<T, KB><<<nproj, 256, 0, st>>>(Q, m, dA, lda, h->perm, h->st, m, n, h->R, n, h->diags,
                                                       h->part_res, h->part_nnz);
      };
      if (p.b <= 1) skinny(std::integral_constant<int, 1>{});
      else if (p.b <= 4) skinny(std::integral_constant<int, 4>{});
      else if (p.b <= 8) skinny(std::integral_constant<int, 8>{});
      else if (p.b <= 16) project(std::integral_constant<int, 16>{});
      else if (p.b <= 32) project(std::integral_constant<int, 32>{});
      else project(std::integral_constant<int, 64>{});
      prof_end(h, RBRP_PHASE_PROJECT, ev, 0.0, 0.0, 1);
    }
    ev = prof_begin(h);
    k_finish<<<1, 1024, 0, st>>>(h->st, h->part_res, h->part_nnz, nproj, h->diags, h->js, n, kmax, tol,
                                 h->trace_rank, h->trace_err, h->trace_samp);
    prof_end(h, RBRP_PHASE_FINISH, ev, 16.0 * nproj, 0.0, 1);
    while ((int)h->block_events.size() <= attempts) {
      cudaEvent_t e;
      s = cuda_check(h, cudaEventCreate(&e), "cudaEventCreate");
      if (s != RBRP_OK) return s;
      h->block_events.push_back(e);
    }
    cudaEventRecord(h->block_events[attempts], st);
    cudaMemcpyAsync(h->hst, h->st, sizeof(State), cudaMemcpyDeviceToHost, st);
    s = cuda_check(h, cudaStreamSynchronize(st), "RBRP block");
    if (s != RBRP_OK) return s;
    if (h->hst->status == tc::ST_ERR_TIMEOUT)
      return set_error(h, RBRP_ERR_DEVICE_TIMEOUT, "a device-side wait timed out; the kernel aborted cleanly");
    if (h->hst->status) return set_error(h, RBRP_ERR_NUMERIC, "non-finite residual during pivoting");
    {  // the loop state must stay in range: a block adds at most one trace entry and b positions
      const State& q = *h->hst;
      if (q.i < i || q.i > kmax || q.i - i > MAXB || q.nblocks < nb_host || q.nblocks > nb_host + 1 ||
          q.bs_sampled < 0 || q.bs_sampled > MAXB || q.nK < 0 || q.nK > MAXB)
        return set_error(h, RBRP_ERR_NUMERIC,
                         "device loop state out of range after block attempt " + std::to_string(attempts) +
                             " (i " + std::to_string(q.i) + ", nblocks " + std::to_string(q.nblocks) +
                             ", sampled " + std::to_string(q.bs_sampled) + ", nK " + std::to_string(q.nK) + ")");
    }
    if (h->hst->nblocks > nb_host) {
      attempt_of_block.push_back(attempts);
      nb_host = h->hst->nblocks;
    }
    if (h->profiling) {  // algorithmic bytes / flops of this block, now that its sizes are known
      const double bss = h->hst->bs_sampled, kept = h->hst->i - i, di = i;
      const double nrem = (double)n - i - kept;
      for (size_t q = mark0; q < h->marks.size(); ++q) {
        auto& mk = h->marks[q];
        if (mk.phase == RBRP_PHASE_CGS) {
          const double dq = RES ? 0.0 : di;  // the residual form gathers, no Gram-Schmidt
          mk.bytes = 2.0 * dm * dq * es + (RES ? 1.0 : 2.0) * dm * bss * es + 8.0 * dm * bss;
          mk.flops = 4.0 * dm * dq * bss + 2.0 * dm * bss * bss;
        } else if (mk.phase == RBRP_PHASE_PANEL) {
          mk.bytes = 8.0 * dm * bss + 16.0 * dm * kept + es * dm * kept;
          mk.flops = 4.0 * dm * kept * kept;
        } else if (mk.phase == RBRP_PHASE_PROJECT) {
          // one read of the remaining columns and the basis, W written to R
          mk.bytes = es * dm * nrem + (RES ? 2.0 : 1.0) * es * dm * kept + 8.0 * kept * nrem +
                     (RES ? 0.0 : 20.0 * nrem);
          mk.flops = 2.0 * dm * nrem * kept;
        } else if (mk.phase == RBRP_PHASE_UPDATE) {
          // read + write of the remaining residual columns, W read, norms written
          mk.bytes = 2.0 * es * dm * nrem + es * dm * kept + 8.0 * kept * nrem + 8.0 * nrem;
          mk.flops = 2.0 * dm * nrem * kept + 2.0 * dm * nrem;
        }
      }
    }
    ++attempts;
  }
  cudaEventRecord(h->ev_loop, st);
  const int k = h->hst->i;
  h->m = m;
  h->n = n;
  h->k = k;
  h->kmax = kmax;
  if (p.compute_T && k > 0 && k < n) {
    ev = prof_begin(h);
    s = solve_T(h, k, n);
    if (s != RBRP_OK) return s;
    const double dk = k, nc = (double)n - k;
    prof_end(h, RBRP_PHASE_TSOLVE, ev, 16.0 * dk * nc + 4.0 * dk * dk, dk * dk * nc, 2);
  }
  if (dPerm) cudaMemcpyAsync(dPerm, h->perm, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, st);
  cudaEventRecord(h->ev_end, st);
  s = cuda_check(h, cudaStreamSynchronize(st), "RBRP finalisation");
  if (s != RBRP_OK) return s;

  prof_collect(h);
  const int nb = h->hst->nblocks;
  h->h_ranks.assign(nb, 0);
  h->h_err.assign(nb, 0.0);
  h->h_tms.assign(nb, 0.0);
  h->h_samp.assign(nb, 0);
  if (nb) {
    cudaMemcpy(h->h_samp.data(), h->trace_samp, sizeof(int) * nb, cudaMemcpyDeviceToHost);
    cudaMemcpy(h->h_ranks.data(), h->trace_rank, sizeof(int) * nb, cudaMemcpyDeviceToHost);
    cudaMemcpy(h->h_err.data(), h->trace_err, sizeof(double) * nb, cudaMemcpyDeviceToHost);
    for (int t = 0; t < nb; ++t) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, h->ev_start, h->block_events[attempt_of_block[t]]);
      h->h_tms[t] = ms;
    }
  }
  rbrp_result r{};
  r.k = k;
  r.nblocks = nb;
  r.res0 = h->hst->res0;
  r.err_est = h->hst->res0 > 0.0 ? h->hst->residual / h->hst->res0 : 0.0;
  r.draws = h->hst->draws;
  r.recomputes = h->hst->recomputes;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, h->ev_start, h->ev_end);
  r.ms_total = ms;
  cudaEventElapsedTime(&ms, h->ev_start, h->ev_loop);
  r.ms_loop = ms;
  cudaEventElapsedTime(&ms, h->ev_loop, h->ev_end);
  r.ms_T = ms;
  h->res = r;
  h->prec = sizeof(T) == 8 ? RBRP_PREC_F64 : RBRP_PREC_F32_MIXED;
  h->have_result = true;
  if (out) *out = r;
  return cuda_check(h, cudaGetLastError(), "RBRP kernels");
}

}  // namespace rbrp
