// Line helpers of the one-thread-per-grid-line element operators (single-problem and batched CGSEM applies): a
// thread holds the N1 values of one grid line of an element in registers.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

namespace selfgpu {

// request the 128-byte line holding p into L2 (no register result; the load that follows later hits L2)
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

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

// ------------------------------------------------------------------------------------ FP64 even-odd matvec
// A derivative matrix on nodes symmetric about 0 is centro-antisymmetric, A(N-i, N-m) = -A(i, m), and so is its
// transpose.  For such a matrix A, with H = N1/2, xe(m) = x(m) + x(N-m) and xo(m) = x(m) - x(N-m)
// (m < H),
//   y(i) = ye(i) + yo(i),  y(N-i) = yo(i) - ye(i),  ye(i) = sum_m E(i,m) xe(m) [+ A(i,H) x(H)],  yo(i) = sum_m O(i,m) xo(m),
// E(i,m) = (A(i,m) + A(i,N-m))/2, O(i,m) = (A(i,m) - A(i,N-m))/2, and for odd N1 the middle row y(H) = sum_m O(H,m) xo(m)
// (the even-odd decomposition of Solomonoff, 1992).  At N1 = 8 a line costs 48 FP64 operations instead of 64.  The
// FP64 element operators are bound by the FP64 pipe on this part (a few FP64 operations per byte), so the count is
// the time.  Both the GLL collocation matrix (CGSEM) and the Legendre-Gauss weak-derivative matrix
// -M^-1 D^T M (DGSEM) have the property.
template <int N1>
struct EOTable {
  static constexpr int H = N1 / 2, ODD = N1 & 1;
  double E[H][H + ODD];  // E(i, m), then A(i, H) for odd N1
  double O[H + ODD][H];  // O(i, m); for odd N1 row H is the middle row
};

template <int N1>
struct EOPair {
  EOTable<N1> D, Dt;  // D and its transpose
};

// host: the tables of the column-major N1 x N1 matrix A (A(i, m) = a[i + N1 m]); false when A is not
// centro-antisymmetric to 1e-13 of its largest entry (a derivative matrix of non-symmetric nodes)
template <int N1>
inline bool eo_table(const double* a, bool transpose, EOTable<N1>& T) {
  constexpr int N = N1 - 1, H = N1 / 2;
  auto A = [&](int i, int m) { return transpose ? a[m + N1 * i] : a[i + N1 * m]; };
  double amax = 0, dev = 0;
  for (int i = 0; i < N1; ++i)
    for (int m = 0; m < N1; ++m) {
      amax = std::max(amax, std::fabs(A(i, m)));
      dev = std::max(dev, std::fabs(A(N - i, N - m) + A(i, m)));
    }
  if (!(dev <= 1e-13 * amax)) return false;
  for (int i = 0; i < H + (N1 & 1); ++i)
    for (int m = 0; m < H; ++m) {
      if (i < H) T.E[i][m] = 0.5 * (A(i, m) + A(i, N - m));
      T.O[i][m] = 0.5 * (A(i, m) - A(i, N - m));
    }
  if (N1 & 1)
    for (int i = 0; i < H; ++i) T.E[i][H] = A(i, H);
  return true;
}

template <int N1>
__device__ __forceinline__ void eo_matvec(const EOTable<N1>& T, const double (&x)[N1], double (&y)[N1]) {
  constexpr int N = N1 - 1, H = N1 / 2;
  double xe[H], xo[H];
#pragma unroll
  for (int m = 0; m < H; ++m) {
    xe[m] = x[m] + x[N - m];
    xo[m] = x[m] - x[N - m];
  }
#pragma unroll
  for (int i = 0; i < H; ++i) {
    double ye = T.E[i][0] * xe[0], yo = T.O[i][0] * xo[0];
#pragma unroll
    for (int m = 1; m < H; ++m) {
      ye = fma(T.E[i][m], xe[m], ye);
      yo = fma(T.O[i][m], xo[m], yo);
    }
    if constexpr (N1 & 1) ye = fma(T.E[i][H + (N1 & 1) - 1], x[H], ye);
    y[i] = ye + yo;
    y[N - i] = yo - ye;
  }
  if constexpr (N1 & 1) {
    double ym = T.O[H + (N1 & 1) - 1][0] * xo[0];
#pragma unroll
    for (int m = 1; m < H; ++m) ym = fma(T.O[H + (N1 & 1) - 1][m], xo[m], ym);
    y[H] = ym;
  }
}

// Warp-synchronous when a warp holds whole elements (32 % N1 == 0: the transposes stay inside the warp), else block
// barriers.
template <int N1>
__device__ __forceinline__ void line_sync() {
  if constexpr (32 % N1 == 0)
    __syncwarp();
  else
    __syncthreads();
}

// sum_m D(i, m) x[m] (T = false) or sum_m D(m, i) x[m] (T = true), m in order (D column-major): with i and m
// known at compile time and D a kernel parameter every D entry is a constant-bank operand of its FMA, no load
template <int N1, bool T>
__device__ __forceinline__ float drow(const float (&D)[N1 * N1], int i, const float (&x)[N1]) {
  float s = 0.f;
#pragma unroll
  for (int m = 0; m < N1; ++m) s = fmaf(T ? D[m + N1 * i] : D[i + N1 * m], x[m], s);
  return s;
}

// The FP32 CGSEM element operator on line t (nodes (i, t)) of element le of a block pass, one thread per grid line
// (every thread of the block calls it, threads without a line pass active = false and only join the barriers):
//   Lu = -( D_s^T (G11 us + G12 up) + D_p^T (G12 us + G22 up) ) - M u  [ - (B1 us + B2 up) for NF = 6 ],
// us = D_s u from the line in registers, up = D_p u and the second transposed contraction through the padded
// transpose buffers X, Y (row stride N1 + 1); fl(f, G) loads the line's values of factor f (G11, G12, G22, M, B1,
// B2).  Four barriers (line_sync); on return X and Y are free.
template <int N1, int NF, class FL>
__device__ __forceinline__ void line_op_f32(const float (&D)[N1 * N1], const FL& fl, bool active, int le, int t,
                                            float* X, float* Y, const float (&u)[N1], float (&Lu)[N1]) {
  constexpr int LS = N1 + 1;
  float* Xl = X + (size_t)(le * N1 + t) * LS;
  float* Yl = Y + (size_t)(le * N1 + t) * LS;
  float us[N1], up[N1], a[N1];
  if (active) {
#pragma unroll
    for (int i = 0; i < N1; ++i) {
      us[i] = drow<N1, false>(D, i, u);
      Xl[i] = u[i];
    }
  }
  line_sync<N1>();
  if (active) {  // column pass: column c = t, up(c, .) = D u(c, .)
    float uc[N1];
#pragma unroll
    for (int m = 0; m < N1; ++m) uc[m] = X[(size_t)(le * N1 + m) * LS + t];
#pragma unroll
    for (int j = 0; j < N1; ++j) Y[(size_t)(le * N1 + j) * LS + t] = drow<N1, false>(D, j, uc);
  }
  line_sync<N1>();
  if (active) {
    float F1[N1], G11[N1], G12[N1], G22[N1];
    fl(0, G11);
    fl(1, G12);
    fl(2, G22);
#pragma unroll
    for (int i = 0; i < N1; ++i) {
      up[i] = Yl[i];
      F1[i] = G11[i] * us[i] + G12[i] * up[i];
      Xl[i] = G12[i] * us[i] + G22[i] * up[i];  // F2(i, t)
    }
#pragma unroll
    for (int i = 0; i < N1; ++i) a[i] = drow<N1, true>(D, i, F1);  // (D^T F1)(i, t)
  }
  line_sync<N1>();
  if (active) {  // column pass: (D^T F2)(c, .)
    float fc[N1];
#pragma unroll
    for (int m = 0; m < N1; ++m) fc[m] = X[(size_t)(le * N1 + m) * LS + t];
#pragma unroll
    for (int j = 0; j < N1; ++j) Y[(size_t)(le * N1 + j) * LS + t] = drow<N1, true>(D, j, fc);
  }
  line_sync<N1>();
  if (active) {
    float Mv[N1];
    fl(3, Mv);
#pragma unroll
    for (int i = 0; i < N1; ++i) Lu[i] = -(a[i] + Yl[i]) - Mv[i] * u[i];
    if constexpr (NF == 6) {
      float B1[N1], B2[N1];
      fl(4, B1);
      fl(5, B2);
#pragma unroll
      for (int i = 0; i < N1; ++i) Lu[i] -= B1[i] * us[i] + B2[i] * up[i];
    }
  }
}

}  // namespace selfgpu
