// Batched CGSEM solves of many uneven problems (mixed mesh sizes and polynomial degrees) on one GPU.
//
// Each problem keeps its own device arrays (operator factors, topology, vectors); the batch is driven by
// device-resident work tables: per-CTA tiles (problem, N, first element, count) for the element operator,
// (problem, first group, count) for the direct-stiffness sum, (problem, first node, count) for the vector
// phases, and a per-problem scalar block.  One launch per phase covers every active problem whatever its
// degree (a switch on N selects the compile-time-specialised element body inside the kernel), and a CUDA
// graph replays a chunk of iterations; problems that converged skip their tiles.  Elements per CTA for each
// (N, element-count bucket) come from a measured autotuning table (self_cgbatch_autotune).
//
// Solver: FP32-inner preconditioned CG under FP64 iterative refinement (the FP32 form of self_cg2d_solve),
// or plain FP64 PCG.  Per problem it is the same recurrence as CGsemElliptic_2D%Solve (:1114-1207) with the
// Jacobi preconditioner; dot products accumulate in FP64 per tile and are reduced per problem in tile order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "cg2d_api.hpp"
#include "internal.hpp"

using namespace selfgpu;

namespace selfgpu {
namespace cgb {

constexpr int kThreads = 256;
constexpr int kVecChunk = kThreads * 8;  // nodes per vector tile

// Device descriptor of one problem.
struct Prob {
  int N, n, nEl, ngroups;
  long long nl;
  const float* fac32;
  const double* fac64;
  const float* dinv32;
  const double* dinv64;
  const int* src;
  const int* gptr;
  const int* gidx;
  const unsigned char* gdir;
  double* f;    // load (FP64)
  double* x;    // solution (FP64)
  double* r;    // FP64 residual
  double* v64;  // FP64 work (FP64 PCG)
  double* w64;
  double* z64;
  float* u32;  // FP32 inner solve: correction
  float* r32;
  float* v32;
  float* w32;
  float* z32;
};

// Per-problem solver scalars.
// done: the current inner solve of this problem finished; conv: the problem reached the outer tolerance.
struct Scal {
  double num, den, rr, r0, tol, rin0;
  int iter, done, total, conv;
};

// gate 0 skips problems whose inner solve is done, gate 1 skips problems that converged
__device__ __forceinline__ bool skip(const Scal& s, int gate) { return gate ? s.conv != 0 : s.done != 0; }

struct ETile {
  int prob, N, e0, ne;
};
struct GTile {
  int prob, g0, ng;
};
struct VTile {
  int prob;
  long long s0, s1;
};

template <int N1>
constexpr int max_epb() {
  return (N1 * N1 >= 256) ? 1 : (256 / (N1 * N1));
}

// vector selectors
enum Vec { V_X = 0, V_R = 1, V_V = 2, V_W = 3, V_Z = 4, V_U = 5 };

template <typename R>
__device__ __forceinline__ R* vec(const Prob& p, int which);
template <>
__device__ __forceinline__ float* vec<float>(const Prob& p, int which) {
  switch (which) {
    case V_R: return p.r32;
    case V_V: return p.v32;
    case V_W: return p.w32;
    case V_Z: return p.z32;
    default: return p.u32;
  }
}
template <>
__device__ __forceinline__ double* vec<double>(const Prob& p, int which) {
  switch (which) {
    case V_X: return p.x;
    case V_R: return p.r;
    case V_V: return p.v64;
    case V_W: return p.w64;
    default: return p.z64;
  }
}

// --------------------------------------------------------------------------- element operator (mixed N)
template <int N1, typename R>
__device__ __forceinline__ void apply_body(const Prob& p, const R* D, int e0, int ne, const R* x, const double* rhs,
                                           R* out, R* sh) {
  constexpr int NN = N1 * N1;
  constexpr int EPBM = max_epb<N1>();
  const int tid = threadIdx.x % NN, le = threadIdx.x / NN;
  const bool active = (le < EPBM) && (le < ne);
  R* su = sh;                 // [EPBM][NN]
  R* s1 = sh + EPBM * NN;     // [EPBM][NN]
  R* s2 = sh + 2 * EPBM * NN; // [EPBM][NN]
  const int e = e0 + le;
  const int i = tid % N1, j = tid / N1;
  const size_t l = (size_t)e * NN + tid;
  const R* fac = (sizeof(R) == 4) ? (const R*)p.fac32 : (const R*)p.fac64;
  R u = 0, us = 0, up = 0;
  if (active) {
    u = x[p.src[l]];
    su[le * NN + tid] = u;
  }
  __syncthreads();
  if (active) {
#pragma unroll
    for (int m = 0; m < N1; ++m) {
      us += D[i + N1 * m] * su[le * NN + m + N1 * j];
      up += D[j + N1 * m] * su[le * NN + i + N1 * m];
    }
    const R* fe = fac + (size_t)e * 4 * NN;
    const R G11 = fe[tid], G12 = fe[NN + tid], G22 = fe[2 * NN + tid];
    s1[le * NN + tid] = G11 * us + G12 * up;
    s2[le * NN + tid] = G12 * us + G22 * up;
  }
  __syncthreads();
  if (active) {
    R a = 0, b = 0;
#pragma unroll
    for (int m = 0; m < N1; ++m) {
      a += D[m + N1 * i] * s1[le * NN + m + N1 * j];
      b += D[m + N1 * j] * s2[le * NN + i + N1 * m];
    }
    const R M = fac[(size_t)e * 4 * NN + 3 * NN + tid];
    const R Lu = -(a + b) - M * u;
    out[l] = rhs ? (R)(rhs[l] - (double)Lu) : Lu;
  }
}

// out = L(unmask(in)) [or rhs - L(...)] for every tile; D matrices for N = 2..9 in one table
struct DTable {
  float d32[10][100];
  double d64[10][100];
};

template <typename R>
__global__ void __launch_bounds__(kThreads) batch_apply(const ETile* __restrict__ tiles, const Prob* __restrict__ probs,
                                                        const Scal* __restrict__ S, const DTable* __restrict__ DT,
                                                        int vin, int vout, int residual, int gate) {
  __shared__ R sh[3 * 256];
  __shared__ R D[100];
  const ETile t = tiles[blockIdx.x];
  if (skip(S[t.prob], gate)) return;
  const Prob& p = probs[t.prob];
  const int n = t.N + 1;
  for (int k = threadIdx.x; k < n * n; k += blockDim.x)
    D[k] = (sizeof(R) == 4) ? (R)DT->d32[t.N][k] : (R)DT->d64[t.N][k];
  __syncthreads();
  const R* x = vec<R>(p, vin);
  R* out = vec<R>(p, vout);
  const double* rhs = residual ? p.f : nullptr;
  switch (n) {
    case 3: apply_body<3, R>(p, D, t.e0, t.ne, x, rhs, out, sh); break;
    case 4: apply_body<4, R>(p, D, t.e0, t.ne, x, rhs, out, sh); break;
    case 5: apply_body<5, R>(p, D, t.e0, t.ne, x, rhs, out, sh); break;
    case 6: apply_body<6, R>(p, D, t.e0, t.ne, x, rhs, out, sh); break;
    case 7: apply_body<7, R>(p, D, t.e0, t.ne, x, rhs, out, sh); break;
    case 8: apply_body<8, R>(p, D, t.e0, t.ne, x, rhs, out, sh); break;
    case 9: apply_body<9, R>(p, D, t.e0, t.ne, x, rhs, out, sh); break;
    case 10: apply_body<10, R>(p, D, t.e0, t.ne, x, rhs, out, sh); break;
    default: break;
  }
}

template <typename R>
__global__ void __launch_bounds__(kThreads) batch_dss(const GTile* __restrict__ tiles, const Prob* __restrict__ probs,
                                                      const Scal* __restrict__ S, int vsel, int gate) {
  const GTile t = tiles[blockIdx.x];
  if (skip(S[t.prob], gate)) return;
  const Prob& p = probs[t.prob];
  R* v = vec<R>(p, vsel);
  for (int g = t.g0 + threadIdx.x; g < t.g0 + t.ng; g += blockDim.x) {
    const int a = p.gptr[g], b = p.gptr[g + 1];
    if (p.gdir[g]) {
      for (int k = a; k < b; ++k) v[p.gidx[k]] = 0;
      continue;
    }
    R s = 0;
    for (int k = a; k < b; ++k) s += v[p.gidx[k]];
    v[p.gidx[a]] = s;
    for (int k = a + 1; k < b; ++k) v[p.gidx[k]] = 0;
  }
}

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double sh[kThreads / 32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, ln = threadIdx.x & 31;
  if (ln == 0) sh[w] = v;
  __syncthreads();
  double r = 0;
  if (w == 0) {
    r = (ln < kThreads / 32) ? sh[ln] : 0.0;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  }
  __syncthreads();
  return r;
}

// Vector phases of the (P)CG iteration, per tile, with the tile's partial dot written to partial[tile].
// op 0: w = r*dinv, partial <r,w>            op 1: v = w + beta v (beta from the problem's num/den)
// op 2: partial <v,z>                         op 3: u += a v, r -= a z, partial <r,r>   (a = num / vz)
// op 4: partial <r,r>
template <typename R>
__global__ void __launch_bounds__(kThreads) batch_vec(const VTile* __restrict__ tiles, const Prob* __restrict__ probs,
                                                      const Scal* __restrict__ S, const double* __restrict__ red,
                                                      double* __restrict__ partial, int op, int precond,
                                                      int gate) {
  const VTile t = tiles[blockIdx.x];
  const Scal& s = S[t.prob];
  if (skip(s, gate)) return;
  const Prob& p = probs[t.prob];
  R* r = vec<R>(p, V_R);
  R* v = vec<R>(p, V_V);
  R* w = vec<R>(p, V_W);
  R* z = vec<R>(p, V_Z);
  R* u = (sizeof(R) == 4) ? (R*)p.u32 : (R*)p.x;
  const R* dinv = (sizeof(R) == 4) ? (const R*)p.dinv32 : (const R*)p.dinv64;
  double acc = 0;
  if (op == 0) {
    for (long long k = t.s0 + threadIdx.x; k < t.s1; k += blockDim.x) {
      const R wk = precond ? r[k] * dinv[k] : r[k];
      w[k] = wk;
      acc += (double)r[k] * (double)wk;
    }
  } else if (op == 1) {
    const bool first = s.iter == 0;
    const R beta = first ? R(0) : (R)(red[t.prob] / s.den);
    for (long long k = t.s0 + threadIdx.x; k < t.s1; k += blockDim.x) v[k] = first ? w[k] : w[k] + beta * v[k];
  } else if (op == 2) {
    for (long long k = t.s0 + threadIdx.x; k < t.s1; k += blockDim.x) acc += (double)v[k] * (double)z[k];
  } else if (op == 3) {
    const R a = (R)(s.num / red[t.prob]);
    for (long long k = t.s0 + threadIdx.x; k < t.s1; k += blockDim.x) {
      u[k] += a * v[k];
      const R rk = r[k] - a * z[k];
      r[k] = rk;
      acc += (double)rk * (double)rk;
    }
  } else {
    for (long long k = t.s0 + threadIdx.x; k < t.s1; k += blockDim.x) acc += (double)r[k] * (double)r[k];
  }
  if (op != 1) {
    acc = block_sum(acc);
    if (threadIdx.x == 0) partial[blockIdx.x] = acc;
  }
}

// Per-problem reduction of its tiles' partials (tile order), one warp per problem.
__global__ void batch_reduce(const int* __restrict__ vt_ptr, const double* __restrict__ partial,
                             const Scal* __restrict__ S, double* __restrict__ red, int nprob, int gate) {
  const int p = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int ln = threadIdx.x & 31;
  if (p >= nprob) return;
  if (skip(S[p], gate)) return;
  double v = 0;
  for (int k = vt_ptr[p] + ln; k < vt_ptr[p + 1]; k += 32) v += partial[k];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (ln == 0) red[p] = v;
}

// Scalar updates per problem.
// mode 0: num = red (after op 0);  mode 1: end of iteration: den = num, rr = red, convergence test
// mode 0: num = red (after op 0); mode 1: end of an inner iteration (den = num, rr, inner stop test)
__global__ void batch_scal(Scal* __restrict__ S, const double* __restrict__ red, int nprob, int mode, int maxIters,
                           int maxInner) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nprob) return;
  Scal& s = S[p];
  if (s.done || s.conv) return;
  if (mode == 0) {
    s.num = red[p];
  } else {
    const double rn = sqrt(red[p]);
    s.den = s.num;
    s.iter += 1;
    s.total += 1;
    s.rr = rn;
    if (!(rn == rn) || rn / s.rin0 < s.tol || s.total >= maxIters || s.iter >= maxInner) s.done = 1;
  }
}

// FP64 -> FP32 residual, FP32 correction -> FP64 solution, zeroing the inner correction
__global__ void batch_convert(const VTile* __restrict__ tiles, const Prob* __restrict__ probs,
                              const Scal* __restrict__ S, int dir) {
  const VTile t = tiles[blockIdx.x];
  if (S[t.prob].conv) return;
  const Prob& p = probs[t.prob];
  for (long long k = t.s0 + threadIdx.x; k < t.s1; k += blockDim.x) {
    if (dir == 0) {
      p.r32[k] = (float)p.r[k];
      p.u32[k] = 0.f;
    } else {
      p.x[k] += (double)p.u32[k];
    }
  }
}

}  // namespace cgb
}  // namespace selfgpu
