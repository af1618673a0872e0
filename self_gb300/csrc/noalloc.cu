// Dot product that allocates nothing: the FP64 two-pass reduction of self_cg2d_dot, with its per-tile
// partial sums kept in a fixed device array of this file instead of memory obtained from cudaMalloc.
//
// Some callers cannot allocate device memory at the point where they need a norm or an inner product:
// Fortran codes whose device arrays live in their own OpenACC / CUDA Fortran data regions and that forbid
// allocation inside the time loop, code that runs while a stream is being captured into a CUDA graph (where
// cudaMalloc is not permitted), and latency-bound loops where an allocation stall is not acceptable.  They pass
// device pointers for the inputs and the output; the scratch is this file's array.
//
// Limits and sharing:
//  * the array holds kMaxTiles = 4096 partial sums (32 KiB); each tile covers kTile = 16384 elements, so
//    n <= kMaxTiles * kTile = 67,108,864 elements; larger n is rejected with SELF_ERR_INVALID;
//  * every call writes each partial it later reads, so nothing has to start at zero; the array keeps the last
//    call's partials;
//  * the array is shared by every call on a device: two calls whose kernels overlap on the GPU (different
//    streams, or different host threads) race on it, so the caller serialises them;
//  * every GPU that loads the library holds the array until the process exits;
//  * the first call on a device looks up the array's device address (cudaGetSymbolAddress) with that device
//    current; make that first call before any stream capture.
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

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_scratch[kMaxDevices] = {};

// Device address of g_dot_partials on the current device (looked up once per device).
int scratch_address(int dev, double** out) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_dot_partials);
    if (e != cudaSuccess || !p) {
      char msg[256];
      snprintf(msg, sizeof(msg), "self_dot_noalloc: cudaGetSymbolAddress failed on device %d: %s", dev,
               cudaGetErrorString(e));
      selfgpu::set_global_error(msg);
      return SELF_ERR_CUDA;
    }
    g_scratch[dev] = static_cast<double*>(p);
  }
  *out = g_scratch[dev];
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
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    selfgpu::set_global_error("self_dot_noalloc: no current CUDA device");
    return SELF_ERR_CUDA;
  }
  double* partials = nullptr;
  int rc = scratch_address(dev, &partials);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int ntiles = (int)((n + kTile - 1) / kTile);
  if (ntiles > 0) dot_tiles<<<ntiles, kThreads, 0, st>>>(x, y, n, partials);
  dot_finish<<<1, kThreads, 0, st>>>(partials, ntiles, result);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    char msg[256];
    snprintf(msg, sizeof(msg), "self_dot_noalloc: launch failed: %s", cudaGetErrorString(e));
    selfgpu::set_global_error(msg);
    return SELF_ERR_CUDA;
  }
  return SELF_OK;
}
