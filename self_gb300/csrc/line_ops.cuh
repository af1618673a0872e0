// Line helpers of the one-thread-per-grid-line element operators (single-problem and batched CGSEM applies): a
// thread holds the N1 values of one grid line of an element in registers.
#pragma once
#include <cuda_runtime.h>

#include <cstring>

namespace selfgpu {

template <int N1>
__device__ __forceinline__ float row_dot(const float* __restrict__ drow, const float (&x)[N1]) {
  // drow: N1 floats padded to a multiple of 4 (zeros), 16-byte aligned; x: registers
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < (N1 + 3) / 4; ++k) {
    const float4 d = *reinterpret_cast<const float4*>(drow + 4 * k);
    if (4 * k + 0 < N1) s = fmaf(d.x, x[4 * k + 0], s);
    if (4 * k + 1 < N1) s = fmaf(d.y, x[4 * k + 1], s);
    if (4 * k + 2 < N1) s = fmaf(d.z, x[4 * k + 2], s);
    if (4 * k + 3 < N1) s = fmaf(d.w, x[4 * k + 3], s);
  }
  return s;
}

// a line of N1 consecutive 4- or 8-byte values: 16-byte loads when a line is a whole number of 16-byte chunks (the
// line then starts on a 16-byte boundary: the element base is a multiple of NN values and every vector's length a
// multiple of a line), 8-byte loads for a whole number of 8-byte chunks, single values otherwise
template <int N1, typename T>
__device__ __forceinline__ void load_line(const T* __restrict__ p, T (&x)[N1]) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8, "32- or 64-bit values");
  constexpr int B = N1 * (int)sizeof(T);
  if constexpr (B % 16 == 0) {
#pragma unroll
    for (int k = 0; k < B / 16; ++k) {
      const int4 v = reinterpret_cast<const int4*>(p)[k];
      memcpy(reinterpret_cast<char*>(x) + 16 * k, &v, 16);
    }
  } else if constexpr (B % 8 == 0) {
#pragma unroll
    for (int k = 0; k < B / 8; ++k) {
      const int2 v = reinterpret_cast<const int2*>(p)[k];
      memcpy(reinterpret_cast<char*>(x) + 8 * k, &v, 8);
    }
  } else {
#pragma unroll
    for (int k = 0; k < N1; ++k) x[k] = p[k];
  }
}

template <int N1, typename T>
__device__ __forceinline__ void store_line(T* __restrict__ p, const T (&x)[N1]) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8, "32- or 64-bit values");
  constexpr int B = N1 * (int)sizeof(T);
  if constexpr (B % 16 == 0) {
#pragma unroll
    for (int k = 0; k < B / 16; ++k) {
      int4 v;
      memcpy(&v, reinterpret_cast<const char*>(x) + 16 * k, 16);
      reinterpret_cast<int4*>(p)[k] = v;
    }
  } else if constexpr (B % 8 == 0) {
#pragma unroll
    for (int k = 0; k < B / 8; ++k) {
      int2 v;
      memcpy(&v, reinterpret_cast<const char*>(x) + 8 * k, 8);
      reinterpret_cast<int2*>(p)[k] = v;
    }
  } else {
#pragma unroll
    for (int k = 0; k < N1; ++k) p[k] = x[k];
  }
}

}  // namespace selfgpu
