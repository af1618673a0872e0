// Peak-rate probe used by the benchmark to state FP64 rooflines: a dependent-free stream of fused
// multiply-adds (8 independent accumulators per thread), one result per thread written to `out`.
#include <cuda_runtime.h>

#include <algorithm>

#include "internal.hpp"

namespace {

template <typename T>
__global__ void __launch_bounds__(256) fma_stream(T* __restrict__ out, int iters, T a, T b) {
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int k = 0; k < iters; ++k) {
    x0 = fma(x0, a, b);
    x1 = fma(x1, a, b);
    x2 = fma(x2, a, b);
    x3 = fma(x3, a, b);
    x4 = fma(x4, a, b);
    x5 = fma(x5, a, b);
    x6 = fma(x6, a, b);
    x7 = fma(x7, a, b);
  }
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

}  // namespace

extern "C" int self_probe_fma_peak(self_ctx* ctx, int fp64, double* tflops) {
  if (!ctx || !tflops) return SELF_ERR_INVALID;
  SELF_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  const int blocks = ctx->num_sms * 8, threads = 256, iters = 1 << 14;
  const size_t n = (size_t)blocks * threads;
  selfgpu::DevBuf<double> out;
  if (out.alloc(n) != cudaSuccess) return selfgpu::set_error(ctx, SELF_ERR_ALLOC, "probe allocation");
  double best = 0.0;
  for (int rep = 0; rep < 3; ++rep) {
    int rc = self_ctx_timer_start(ctx);
    if (rc) return rc;
    if (fp64)
      fma_stream<double><<<blocks, threads, 0, ctx->stream>>>(out.p, iters, 0.999999, 1e-7);
    else
      fma_stream<float><<<blocks, threads, 0, ctx->stream>>>(reinterpret_cast<float*>(out.p), iters, 0.999999f,
                                                             1e-7f);
    SELF_LAUNCHED(ctx);
    double ms = 0;
    if ((rc = self_ctx_timer_stop(ctx, &ms))) return rc;
    const double flops = 2.0 * 8.0 * iters * (double)n;
    best = std::max(best, flops / (ms * 1e-3) / 1e12);
  }
  *tflops = best;
  return SELF_OK;
}
