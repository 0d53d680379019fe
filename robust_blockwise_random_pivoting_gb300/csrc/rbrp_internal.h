// rbrp_internal.h - host-side handle and workspace of the RBRP library.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/rbrp_gb300.h"
#include "rbrp_common.cuh"

namespace rbrp {

// clock64 limit of a bounded device-side wait (~2 s at GB300's 2.07 GHz SM clock)
constexpr long long kWaitBudgetDefault = 4ll << 30;

constexpr int P2_MAX_SPLIT_WS = 8;  // row ranges of the residual update (workspace sizing)
constexpr int P1_MAX_SPLIT = 8;     // row ranges of the tensor-core projection
struct BatchState;                  // batched form (rbrp_batched.cu)
}

struct rbrp_handle_st {
  int device = 0;
  int sms = 152;   // SM count of the device (set at create)
  cudaStream_t stream = nullptr;
  std::string last_error;

  // device workspace (one allocation, carved; grown on demand)
  void* ws = nullptr;
  size_t ws_bytes = 0;
  rbrp::State* st = nullptr;
  rbrp::State* hst = nullptr;  // pinned host mirror of the state
  double* diags = nullptr;
  int* perm = nullptr;
  void* Q = nullptr;           // m x kmax, element type of A
  double* R = nullptr;         // kmax x n, row major
  double* V = nullptr;         // m x MAXB
  double* Q1 = nullptr;        // m x MAXB
  void* Cpart = nullptr;       // split partials of Q^T A_J
  void* C = nullptr;           // kmax x MAXB
  double* Gpart = nullptr;
  double* G = nullptr;
  double* G2part = nullptr;
  double* G2 = nullptr;
  double* R11 = nullptr;
  double* R2 = nullptr;
  int* ord = nullptr;
  double* pbuf = nullptr;      // 2n: weights and cdf
  unsigned long long* kbuf = nullptr;
  int* js = nullptr;
  int* cols = nullptr;
  int* J = nullptr;
  int* K1 = nullptr;
  int* K2 = nullptr;
  double* part_res = nullptr;
  int* part_nnz = nullptr;
  int* trace_rank = nullptr;
  double* trace_err = nullptr;
  int* trace_samp = nullptr;
  double* err_part = nullptr;  // partial sums of the ID-error kernel
  float* Ares = nullptr;       // residual form: position-ordered FP32 residual, ld_res x n
  int64_t ld_res = 0;
  double* part_norm = nullptr; // residual form: partial column norms per row range
  double* Wpart = nullptr;     // residual form: row-split partial projections, P1_MAX_SPLIT x 64 x n
                               // double-float pairs (float2, 8 bytes each)
  float* Qh = nullptr;         // residual form: TF32 hi / lo parts of the block basis, ld_res x 64
  float* Ql = nullptr;
  float* Qrh = nullptr;        // the same parts by rows (m x 64, row major) for the tensor-core update
  float* Qrl = nullptr;
  float* Wth = nullptr;        // TF32 hi / lo parts of W^T (n x 64, position major) for the same
  float* Wtl = nullptr;
  int variant = 0;             // 0: tensor-core projection and update, 1: CUDA-core ones
  bool tsolve_fp64 = false;    // T solve on the FP64 pipe instead of double-float
  long long wait_budget = 0;   // clock64 limit of bounded device waits (0: the default, ~2 s)

  // interpolation matrix of the last run
  double* T = nullptr;
  size_t T_bytes = 0;
  void* df_buf = nullptr;      // double-float operands of the T solve
  size_t df_bytes = 0;

  // Gaussian sketch matrix (rbrp_sketch.cu)
  void* sketch_ws = nullptr;
  size_t sketch_bytes = 0;
  // LU-pivot workspace (rbrp_lupp.cu): W^T, argmax partials, barrier, positions
  void* lupp_ws = nullptr;
  size_t lupp_bytes = 0;

  // truncated-SVD interpolation (rbrp_matdivide.cu): Jacobi workspace, R11 | R12 operands
  void* md_ws = nullptr;
  size_t md_bytes = 0;
  void* md_aux = nullptr;
  size_t md_aux_bytes = 0;

  // fixed-skeleton adjoint workspace (rbrp_adjoint.cu)
  void* adj_ws = nullptr;
  size_t adj_bytes = 0;

  // fixed-skeleton runs: order_of[col] = index of col in the given skeleton, -1 otherwise
  int* given_order = nullptr;
  size_t given_cap = 0;

  // device copy of a host matrix (host-buffer entry points)
  void* hostA_dev = nullptr;
  size_t hostA_bytes = 0;

  // last-run results
  bool have_result = false;
  int m = 0, n = 0, k = 0, kmax = 0, prec = 0;
  rbrp_result res{};
  std::vector<int> h_ranks;
  std::vector<double> h_err;
  std::vector<double> h_tms;
  std::vector<int> h_samp;
  std::vector<cudaEvent_t> block_events;
  cudaEvent_t ev_start = nullptr, ev_loop = nullptr, ev_end = nullptr;
  bool smem_attr_set = false;
  bool smem_attr_gemm_tc = false;  // the adjoint's tcgen05 GEMMs (rbrp_adjoint.cu)
  bool smem_attr_sketch_tc = false;  // the sketch's tcgen05 GEMM (rbrp_sketch.cu)

  // per-phase profiling
  bool profiling = false;
  rbrp_phase_stats stats{};
  struct PhaseMark {
    int phase;
    int ev0, ev1;
    double bytes, flops;
    int launches;
  };
  std::vector<cudaEvent_t> prof_events;
  std::vector<PhaseMark> marks;
  int prof_next = 0;

  // batched form (rbrp_batched.cu): plan, workspace slots, captured graph
  rbrp::BatchState* batch = nullptr;
};

namespace rbrp {

// RAII guard that makes the handle's device current for one call.
struct DeviceGuard {
  int prev = -1;
  bool ok = false;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    ok = cudaSetDevice(dev) == cudaSuccess;
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

// Frees the batched form's device state of a handle (rbrp_batched.cu).
void batch_release(rbrp_handle h);

struct Layout {
  int m, n, kmax, ntiles, nproj, cpart_rows;
  size_t elem;    // sizeof element of A / Q
  bool residual;  // FP32 residual form: Q holds one block, A_res is allocated
  int64_t ld_res;
};

rbrp_status ensure_workspace(rbrp_handle h, const Layout& L);
rbrp_status set_error(rbrp_handle h, rbrp_status s, const std::string& msg);
rbrp_status cuda_check(rbrp_handle h, cudaError_t e, const char* what);

template <typename T>
rbrp_status run_rbrp(rbrp_handle h, int m, int n, const T* dA, int64_t lda, const rbrp_params& p,
                     int* dPerm, rbrp_result* out);

rbrp_status solve_T(rbrp_handle h, int k, int n);

// 2-D FP32 TMA descriptor (inner dimension contiguous, 128-byte swizzle).
rbrp_status make_tmap_f32(rbrp_handle h, void* map, const float* base, uint64_t inner, uint64_t outer,
                          uint64_t ld_elems, uint32_t box_inner, uint32_t box_outer);

template <typename T>
rbrp_status id_error(rbrp_handle h, int m, int n, const T* dA, int64_t lda, double* err);

int splits_for(int i, int m);

// Profiling helpers: prof_begin records an event and returns its index (-1 when off).
int prof_begin(rbrp_handle h);
void prof_end(rbrp_handle h, int phase, int ev0, double bytes, double flops, int launches);
void prof_collect(rbrp_handle h);  // after a stream sync: fold the marks into h->stats
Layout make_layout(int m, int n, int kmax, size_t elem, bool residual);

}  // namespace rbrp
