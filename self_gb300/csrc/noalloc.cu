// Dot product that allocates nothing: an FP64 two-pass reduction over contiguous tiles whose per-tile partial
// sums live in a fixed device array of this file instead of memory obtained from cudaMalloc.
//
// Some callers cannot allocate device memory at the point where they need a norm or an inner product:
// Fortran codes whose device arrays live in their own OpenACC / CUDA Fortran data regions and that forbid
// allocation inside the time loop, and latency-bound loops where an allocation stall is not acceptable.  They
// pass device pointers for the inputs and the output; the scratch is this file's array.
//
// Result: sum over tiles (in tile order per thread, then a fixed tree) of the tile sums; deterministic for a
// given n, and equal to self_cg2d_dot on the same vectors up to rounding (that entry point sums in a different
// order, grid-stride per block).
//
// Limits and sharing:
//  * the array holds kMaxTiles = 4096 partial sums (32 KiB); each tile covers kTile = 16384 elements, so
//    n <= kMaxTiles * kTile = 67,108,864 elements; larger n is rejected with SELF_ERR_INVALID;
//  * every call writes each partial it later reads, so nothing has to start at zero; the array keeps the last
//    call's partials;
//  * the array is shared by every call on a device: two calls whose kernels overlap on the GPU (different
//    streams, or different host threads) race on it, so the caller serialises them;
//  * every GPU that loads the library holds the array until the process exits;
//  * the first call in a CUDA context looks up the array's device address (cudaGetSymbolAddress) with that
//    context's device current; the address is kept per context (keyed by the CUDA context ID), so a new
//    context on the same device -- after cudaDeviceReset, say -- looks it up again on its first call.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "internal.hpp"

namespace {

constexpr int kThreads = 256;
constexpr long long kTile = 16384;  // elements per partial sum (kThreads x 64)
constexpr int kMaxTiles = 4096;
constexpr long long kMaxN = kTile * kMaxTiles;

static __device__ __align__(256) double g_dot_partials[kMaxTiles];

// partials[t] = sum over tile t of x*y (FP64), tile t = [t*kTile, min(n, (t+1)*kTile))
__global__ void __launch_bounds__(kThreads) dot_tiles(const double* __restrict__ x, const double* __restrict__ y,
                                                      long long n, double* __restrict__ partials) {
  const long long t0 = (long long)blockIdx.x * kTile;
  const long long t1 = (t0 + kTile < n) ? t0 + kTile : n;
  double s = 0.0;
  for (long long k = t0 + threadIdx.x; k < t1; k += kThreads) s += x[k] * y[k];
  __shared__ double sh[kThreads / 32];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = (threadIdx.x < kThreads / 32) ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) partials[blockIdx.x] = v;
  }
}

// result = sum of the ntiles partials, in tile order per thread then tree order
__global__ void __launch_bounds__(kThreads) dot_finish(const double* __restrict__ partials, int ntiles,
                                                       double* __restrict__ result) {
  double s = 0.0;
  for (int k = threadIdx.x; k < ntiles; k += kThreads) s += partials[k];
  __shared__ double sh[kThreads / 32];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = (threadIdx.x < kThreads / 32) ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) *result = v;
  }
}

// Driver entry points for the current context's ID, fetched through the runtime (no link against libcuda).
using PfnCtxGetCurrent = CUresult (*)(CUcontext*);
using PfnCtxGetId = CUresult (*)(CUcontext, unsigned long long*);

constexpr int kMaxContexts = 64;
struct ScratchEntry {
  unsigned long long ctx_id;
  double* addr;
};
std::mutex g_mu;
ScratchEntry g_scratch[kMaxContexts];
int g_nscratch = 0;
PfnCtxGetCurrent g_get_current = nullptr;
PfnCtxGetId g_get_id = nullptr;

void fail(const char* what, cudaError_t e) {
  char msg[320];
  snprintf(msg, sizeof(msg), "self_dot_noalloc: %s: %s", what, cudaGetErrorString(e));
  selfgpu::set_global_error(msg);
}

// Device address of g_dot_partials in the current context (looked up once per context).
int scratch_address(double** out) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_get_current || !g_get_id) {
    cudaDriverEntryPointQueryResult q1, q2;
    cudaError_t e1 = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", (void**)&g_get_current, 12000,
                                                      cudaEnableDefault, &q1);
    cudaError_t e2 = cudaGetDriverEntryPointByVersion("cuCtxGetId", (void**)&g_get_id, 12000, cudaEnableDefault,
                                                      &q2);
    if (e1 != cudaSuccess || e2 != cudaSuccess || q1 != cudaDriverEntryPointSuccess ||
        q2 != cudaDriverEntryPointSuccess || !g_get_current || !g_get_id) {
      g_get_current = nullptr;
      g_get_id = nullptr;
      fail("driver entry points for the context ID are unavailable", e1 != cudaSuccess ? e1 : e2);
      return SELF_ERR_CUDA;
    }
  }
  // the current context: the caller's, or (none current yet) the primary context of the current device, which
  // the runtime makes current on its first call (here the symbol lookup)
  CUcontext cu = nullptr;
  void* p = nullptr;
  if (g_get_current(&cu) != CUDA_SUCCESS) cu = nullptr;
  if (!cu) {
    cudaError_t e = cudaGetSymbolAddress(&p, g_dot_partials);
    if (e != cudaSuccess || !p) {
      fail("cudaGetSymbolAddress of the scratch array failed", e);
      return SELF_ERR_CUDA;
    }
    if (g_get_current(&cu) != CUDA_SUCCESS) cu = nullptr;
  }
  unsigned long long id = 0;
  if (!cu || g_get_id(cu, &id) != CUDA_SUCCESS) {
    selfgpu::set_global_error("self_dot_noalloc: cannot read the current CUDA context's ID");
    return SELF_ERR_CUDA;
  }
  for (int k = 0; k < g_nscratch; ++k)
    if (g_scratch[k].ctx_id == id) {
      *out = g_scratch[k].addr;
      return SELF_OK;
    }
  if (!p) {
    cudaError_t e = cudaGetSymbolAddress(&p, g_dot_partials);
    if (e != cudaSuccess || !p) {
      fail("cudaGetSymbolAddress of the scratch array failed", e);
      return SELF_ERR_CUDA;
    }
  }
  // a full table drops its oldest entry (contexts that long outlived are the likeliest to be gone)
  if (g_nscratch == kMaxContexts) {
    for (int k = 1; k < kMaxContexts; ++k) g_scratch[k - 1] = g_scratch[k];
    --g_nscratch;
  }
  g_scratch[g_nscratch++] = {id, static_cast<double*>(p)};
  *out = static_cast<double*>(p);
  return SELF_OK;
}

}  // namespace

extern "C" int self_dot_noalloc(const double* x, const double* y, long long n, double* result, void* stream) {
  if (n < 0 || !result || (n > 0 && (!x || !y))) {
    selfgpu::set_global_error("self_dot_noalloc: null pointer or negative length");
    return SELF_ERR_INVALID;
  }
  if (n > kMaxN) {
    char msg[256];
    snprintf(msg, sizeof(msg),
             "self_dot_noalloc: n = %lld exceeds the %lld-element limit of its static scratch (%d partial sums of "
             "%lld elements)",
             n, kMaxN, kMaxTiles, kTile);
    selfgpu::set_global_error(msg);
    return SELF_ERR_INVALID;
  }
  // an error left pending by earlier, unrelated work is reported as such and not blamed on this call
  cudaError_t e = cudaPeekAtLastError();
  if (e != cudaSuccess) {
    fail("an earlier CUDA error is pending (not from this call); nothing was launched", e);
    return SELF_ERR_CUDA;
  }
  double* partials = nullptr;
  int rc = scratch_address(&partials);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int ntiles = (int)((n + kTile - 1) / kTile);
  if (ntiles > 0) dot_tiles<<<ntiles, kThreads, 0, st>>>(x, y, n, partials);
  dot_finish<<<1, kThreads, 0, st>>>(partials, ntiles, result);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    fail("launch failed", e);
    return SELF_ERR_CUDA;
  }
  return SELF_OK;
}
