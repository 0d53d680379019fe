// rbrp_noalloc.cu - ID-error entry point that allocates no memory.
//
// Some callers cannot let a library call cudaMalloc: a host runtime (Go, the
// JVM, Node) that hands the library a fixed pool of device memory and owns
// every allocation, a service with a hard device-memory budget, or code that
// enqueues work where an allocation would synchronise the device.  For them,
// rbrp_id_error_f64_noalloc computes the squared relative ID error
// ||A(:, rd) - A(:, S) T||_F^2 / ||A||_F^2 without a handle and without any
// allocation: its partial sums live in a file-scope device array of fixed size,
// g_noalloc_parts (2 MiB), that every GPU loading this library holds until the
// process exits.
//
// The array is shared by all calls on a device and keeps the previous call's
// contents; every partial that a call reads is written by that call first.
// Calls that overlap on the GPU (two streams, or two host threads) race on the
// array and must be serialised by the caller.
//
// Set-up: the first call in each CUDA context (the device's primary context, or
// a context the caller created with cuCtxCreate and made current) looks up the
// array's address in that context (cudaGetSymbolAddress) and caches it under
// the context's unique id (cuCtxGetId), so a later context on the same device,
// for instance after cudaDeviceReset, gets its own lookup; make the first call
// in a context before any stream capture begins.
//
// k == 0 and k == n are valid IDs: their errors are written as 1.0 and 0.0, as
// the handle's rbrp_id_error_f64 reports them.
#include <cudaTypedefs.h>

#include <mutex>
#include <utility>
#include <vector>

#include "rbrp_internal.h"

namespace {

constexpr int64_t kMaxParts = 262144;  // partial sums: ceil((n-k)/32) * ceil(m/64) <= 262144
constexpr size_t kMaxContexts = 64;  // cached (context id, address) pairs

static __device__ __align__(256) double g_noalloc_parts[kMaxParts];

std::mutex g_mu;
std::vector<std::pair<unsigned long long, double*>> g_parts_by_ctx;  // newest last

// Unique id of the calling thread's current CUDA context (the runtime's primary
// context is made current first when there is none).
rbrp_status current_context_id(unsigned long long* id) {
  static PFN_cuCtxGetCurrent_v4000 get_current = nullptr;
  static PFN_cuCtxGetId_v12000 get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(p);
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(p);
    cudaGetLastError();
  });
  if (!get_current || !get_id) return RBRP_ERR_CUDA;
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != CUDA_SUCCESS) return RBRP_ERR_CUDA;
  if (!ctx) {  // no context yet on this thread: bind the current device's primary context
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaSetDevice(dev) != cudaSuccess) {
      cudaGetLastError();
      return RBRP_ERR_CUDA;
    }
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return RBRP_ERR_CUDA;
  }
  return get_id(ctx, id) == CUDA_SUCCESS ? RBRP_OK : RBRP_ERR_CUDA;
}

// Address of g_noalloc_parts in the current context (looked up once per context).
rbrp_status parts_for_current_context(double** out) {
  unsigned long long id = 0;
  const rbrp_status s = current_context_id(&id);
  if (s != RBRP_OK) return s;
  std::lock_guard<std::mutex> lock(g_mu);
  for (const auto& e : g_parts_by_ctx)
    if (e.first == id) {
      *out = e.second;
      return RBRP_OK;
    }
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_noalloc_parts) != cudaSuccess || !p) {
    cudaGetLastError();
    return RBRP_ERR_CUDA;
  }
  // context ids are never reused, so dropping the oldest entry only costs a new lookup
  if (g_parts_by_ctx.size() >= kMaxContexts) g_parts_by_ctx.erase(g_parts_by_ctx.begin());
  g_parts_by_ctx.emplace_back(id, static_cast<double*>(p));
  *out = static_cast<double*>(p);
  return RBRP_OK;
}

// Same arithmetic as the handle's ID-error kernel: one 64-row x 32-column tile
// of E = A(:, rd) - A(:, S) T per CTA in FP64, its squared sum into parts[].
__global__ void __launch_bounds__(256)
k_id_error_parts(const double* __restrict__ A, int64_t lda, const int* __restrict__ perm,
                 const double* __restrict__ Tm, int64_t ldt, int k, int m, int n, double* __restrict__ parts) {
  __shared__ double As[64][33];
  __shared__ double Ts[32][33];
  __shared__ double red[32];
  const int tid = threadIdx.x;
  const int r0 = blockIdx.y * 64, c0 = blockIdx.x * 32;
  const int ncols = n - k;
  const int x = tid >> 2;
  double acc[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) acc[q] = 0.0;
  for (int a0 = 0; a0 < k; a0 += 32) {
    __syncthreads();
    for (int idx = tid; idx < 64 * 32; idx += 256) {
      const int xr = idx & 63, y = idx >> 6;
      const int r = r0 + xr, a = a0 + y;
      As[xr][y] = (r < m && a < k) ? A[r + (int64_t)perm[a] * lda] : 0.0;
    }
    for (int idx = tid; idx < 32 * 32; idx += 256) {
      const int y = idx & 31, c = idx >> 5;
      Ts[y][c] = (a0 + y < k && c0 + c < ncols) ? Tm[(a0 + y) + (int64_t)(c0 + c) * ldt] : 0.0;
    }
    __syncthreads();
#pragma unroll 4
    for (int y = 0; y < 32; ++y) {
      const double av = As[x][y];
#pragma unroll
      for (int q = 0; q < 8; ++q) acc[q] = fma(av, Ts[y][(tid & 3) + 4 * q], acc[q]);
    }
  }
  double s = 0.0;
  const int r = r0 + x;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int c = c0 + (tid & 3) + 4 * q;
    if (r < m && c < ncols) {
      const double e = A[r + (int64_t)perm[k + c] * lda] - acc[q];
      s = fma(e, e, s);
    }
  }
  s = rbrp::block_sum(s, red);
  if (tid == 0) parts[(int64_t)blockIdx.y * gridDim.x + blockIdx.x] = s;
}

// err = (sum of the nparts partials, fixed order) / normA2.
// The error of an empty skeleton (1) or of a full one (0).
__global__ void k_store_err(double v, double* __restrict__ err) { *err = v; }

__global__ void __launch_bounds__(256) k_sum_parts(const double* __restrict__ parts, int64_t nparts, double normA2,
                                                   double* __restrict__ err) {
  __shared__ double red[32];
  double s = 0.0;
  for (int64_t z = threadIdx.x; z < nparts; z += blockDim.x) s += parts[z];
  s = rbrp::block_sum(s, red);
  if (threadIdx.x == 0) *err = normA2 > 0.0 ? s / normA2 : 0.0;
}

}  // namespace

extern "C" rbrp_status rbrp_id_error_f64_noalloc(int m, int n, const double* dA, int64_t lda, const int* dPerm,
                                                 int k, const double* dT, int64_t ldt, double normA2, double* dErr,
                                                 void* stream) {
  if (m < 1 || n < 1 || k < 0 || k > n || lda < m) return RBRP_ERR_INVALID_ARG;
  if (!dErr) return RBRP_ERR_INVALID_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (k == 0 || k == n) {  // nothing to reconstruct: the whole matrix, or nothing, is left over
    k_store_err<<<1, 1, 0, st>>>(k == 0 ? 1.0 : 0.0, dErr);
    return cudaGetLastError() == cudaSuccess ? RBRP_OK : RBRP_ERR_CUDA;
  }
  if (!dA || !dPerm || !dT || ldt < k) return RBRP_ERR_INVALID_ARG;
  const int64_t gx = (n - k + 31) / 32, gy = (m + 63) / 64;
  if (gx * gy > kMaxParts || gy > 65535) return RBRP_ERR_CAPACITY;  // beyond the fixed scratch
  double* parts = nullptr;
  rbrp_status s = parts_for_current_context(&parts);
  if (s != RBRP_OK) return s;
  k_id_error_parts<<<dim3((unsigned)gx, (unsigned)gy), 256, 0, st>>>(dA, lda, dPerm, dT, ldt, k, m, n, parts);
  k_sum_parts<<<1, 256, 0, st>>>(parts, gx * gy, normA2, dErr);
  if (cudaGetLastError() != cudaSuccess) return RBRP_ERR_CUDA;
  return RBRP_OK;
}
