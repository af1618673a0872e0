// Internal definitions of libselfgpu: context, error reporting, device buffers.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/self_gpu.h"

struct self_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int num_sms = 0;
  std::string last_error;
  std::atomic<long long> launches{0};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  void* flush_buf = nullptr;
  size_t flush_bytes = 0;
  int host_loop = 0;  // (P)CG solves looped from the host (profilers), see self_ctx_host_loop
};

namespace selfgpu {

int set_error(self_ctx* ctx, int status, const char* fmt, ...);
// Global fallback error text for calls made before a context exists.
void set_global_error(const char* msg);

#define SELF_CUDA_TRY(ctx, call)                                                                       \
  do {                                                                                                 \
    cudaError_t e_ = (call);                                                                           \
    if (e_ != cudaSuccess)                                                                             \
      return ::selfgpu::set_error((ctx), SELF_ERR_CUDA, "%s failed: %s (%s:%d)", #call,                \
                                  cudaGetErrorString(e_), __FILE__, __LINE__);                         \
  } while (0)

// Launch accounting + error check after each kernel launch.
#define SELF_LAUNCHED(ctx)                                                                             \
  do {                                                                                                 \
    (ctx)->launches.fetch_add(1, std::memory_order_relaxed);                                          \
    cudaError_t e_ = cudaGetLastError();                                                               \
    if (e_ != cudaSuccess)                                                                             \
      return ::selfgpu::set_error((ctx), SELF_ERR_CUDA, "kernel launch failed: %s (%s:%d)",           \
                                  cudaGetErrorString(e_), __FILE__, __LINE__);                         \
  } while (0)

// A device allocation owned by a handle.
template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaError_t alloc(size_t count) {
    free();
    n = count;
    if (count == 0) return cudaSuccess;
    return cudaMalloc((void**)&p, count * sizeof(T));
  }
  void free() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  size_t bytes() const { return n * sizeof(T); }
  ~DevBuf() { free(); }
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
};

// Device-visible address of the host range [p, p + bytes) when it lies inside one block returned by
// self_host_alloc (page-locked and mapped), else null: such buffers are read and written by kernels directly.
void host_blocks_add(const void* p, size_t bytes);
void host_blocks_remove(const void* p);
void* mapped_host(const void* p, size_t bytes);

}  // namespace selfgpu
