// Batched CGSEM solves of many uneven problems (mixed mesh sizes and polynomial degrees) on one GPU.
//
// Each problem keeps its own device arrays (operator factors, topology, vectors).  Work is described by tile
// tables: ETile (problem, N, first element, count) for the element operator, GTile (problem, first group, count)
// for the direct-stiffness sum, VTile (problem, first node, last node) for vector phases.  The host uploads the
// tables of every problem in the pool ("all") when the pool changes; at every tick two compacted sets -- "outer"
// (problems waiting for their FP64 residual) and "inner" (problems running inner iterations) -- are rebuilt from
// them on the device (bk_compact_offsets / bk_compact_copy), and the outer decision (converged, next inner solve)
// is made on the device too (bk_decide).  A tick is therefore one captured graph with no host round trip, and a
// whole batched solve is one launch of a graph whose conditional while node repeats the tick until bk_decide finds
// no problem running.  Every kernel is a fixed-size grid over the table capacity (blocks past the current count
// exit at once).  One inner PCG iteration is three launches over all active problems (a switch on N selects the
// compile-time element body):
//   bk_apply : v_new = w + beta v_old (per-problem parity picks the buffers), z = L(v_new) per element, tile
//              partial <v_new, z>;
//   bk_dss   : z = Mask(GlobalSum(z));
//   bk_update: a = num/<v,z>, u += a v, r -= a z, w = dinv r, tile partials <r,w>, <r,r>.
// The last tile of a problem to finish (per-problem atomic ticket) adds that problem's tile partials in tile
// order and updates its scalars, so every sum is deterministic and independent of the other problems.
// Elements per element tile for each (N, element-count bucket) come from a measured autotuning table
// (self_cgbatch_autotune).
//
// Solver: FP32-inner preconditioned CG under FP64 iterative refinement (the FP32 form of self_cg2d_solve),
// or plain FP64 PCG.  Per problem it is the recurrence of CGsemElliptic_2D%Solve (:1114-1207) with the Jacobi
// preconditioner.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "cg2d_api.hpp"
#include "internal.hpp"
#include "line_ops.cuh"

using namespace selfgpu;

namespace selfgpu {
namespace cgb {

constexpr int kThreads = 256;
constexpr int kVecChunk = kThreads * 8;  // nodes per vector tile
constexpr int kRoundsInFlight = 1;        // rounds of an element tile processed together (loads in flight)

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
  double* v2_64;  // second direction buffers (v and v2 alternate with the iteration parity)
  float* v2_32;
};

// Per-problem solver state.  phase: 0 inner iterations running, 1 waiting for the outer (FP64 residual)
// update, 2 finished (converged or out of budget), 3 empty slot.
struct Scal {
  double num, den, rr, r0, tol, rin0, vz;
  double alpha, beta;             // step lengths, formed once per problem by its last tile (no per-thread division)
  float alpha32, beta32;
  int iter, phase, total, fresh;  // fresh: no outer update yet (initial residual pending)
  int max_total, max_inner;       // iteration limits of the current solve
  int outer, pad;                 // refinement steps taken (the outer decision runs on the device)
};

// Parameters of the outer decision (bk_decide), fixed per captured graph.
struct DecideArgs {
  double tol, inner_tol;
  int fp32, max_outer, max_total;
  unsigned int max_bodies;  // bound of the persistent loop (bodies run before its condition is cleared)
};

// gate 0 runs problems in phase 0, gate 1 those in phase 1, gate 2 those in phase 1 that are not fresh,
// gate 3 those in phase 0 that just entered it (iter == 0)
__device__ __forceinline__ bool skip(const Scal& s, int gate) {
  switch (gate) {
    case 0: return s.phase != 0;
    case 1: return s.phase != 1;
    case 2: return s.phase != 1 || s.fresh;
    default: return s.phase != 0 || s.iter != 0;
  }
}

struct ETile {
  int prob, N, e0, ne, epr;  // ne elements from e0, processed epr at a time (one node per thread)
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

// D matrices for N = 2..9 in one table
struct DTable {
  float d32[10][100];
  double d64[10][100];
};

// Device view of one compacted tile-table set.  cnt[0..2]: ETiles, GTiles, VTiles; eptr/vptr[p]: first tile of
// problem p (eptr[p + 1] - eptr[p] tiles; zero for problems outside the set).
struct TileView {
  const ETile* et;
  const GTile* gt;
  const VTile* vt;
  const int* cnt;
  const int* eptr;
  const int* vptr;
};

// Sum over a 256-thread block: warp sums in the working precision, the 8 warp sums in FP64 (valid in thread 0).
template <typename R>
__device__ __forceinline__ double block_sum_r(R v) {
  __shared__ double sh[kThreads / 32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, ln = threadIdx.x & 31;
  if (ln == 0) sh[w] = (double)v;
  __syncthreads();
  double r = 0;
  if (w == 0) {
    r = (ln < kThreads / 32) ? sh[ln] : 0.0;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  }
  __syncthreads();
  return r;
}

// Tile partial(s) of problem p (NS sums; thread 0 holds the block values): written at partial[s * stride + t];
// the last of the problem's `count` tiles adds the problem's partials (tile order, from `first`) into tot
// (thread 0) and returns true (block-uniform).
template <int NS>
__device__ __forceinline__ bool tile_last(const double (&bv)[NS], double* __restrict__ partial, size_t stride, int t,
                                          unsigned int* __restrict__ ticket, int first, int count, double (&tot)[NS]) {
  __shared__ bool s_last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int s = 0; s < NS; ++s) partial[s * stride + t] = bv[s];
    __threadfence();
    s_last = atomicAdd(ticket, 1u) == (unsigned)(count - 1);
  }
  __syncthreads();
  const bool last = s_last;
  __syncthreads();  // s_last is rewritten by the next tile of this block
  if (!last) return false;
  __threadfence();
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    double a = 0;
    for (int k = threadIdx.x; k < count; k += kThreads) a += __ldcg(&partial[s * stride + first + k]);
    tot[s] = block_sum_r<double>(a);
  }
  if (threadIdx.x == 0) *ticket = 0u;
  return true;
}

// ------------------------------------------------------------------ FP32 element operator, one thread per line
// The FP32 inner iterations run the element operator as one thread per grid line (line_op_f32, the operator of the
// single-problem FP32 PCG apply): a round covers up to 256 / N1 elements, thread (le, t) holding line t (nodes
// (i, t)) of element e0 + le in registers; the two column passes go through padded transpose buffers (row stride
// N1 + 1), warp-synchronous when a warp holds whole elements; the derivative matrix is read as constant-bank FMA
// operands from c_dline.
constexpr int kLineBuf = 256 * 11;  // transpose buffer floats: (256 / N1) * N1 * (N1 + 1) <= 256 * 11 for N1 <= 10

// D (column-major) of degrees N = 2..9 (N1 = 3..10) in constant memory, one table per device shared by every batch
// (set by the first problem of a degree; add() refuses a problem whose D differs from the table)
__constant__ float c_dline[8][100];

template <int N1>
constexpr int line_round_elems() {
  return 256 / N1;
}
int line_round_elems_rt(int N) { return 256 / (N + 1); }

// One round of ne <= 256 / N1 elements from e0.  FUSED: v_new = w + beta v_old (written), u = v_new gathered through
// src, z = L(u), returns the thread's sum of u * Lu; otherwise out = L(w gathered through src), or with rhs
// out = rhs - L in FP64, rounded (the plain apply's result).
template <int N1, bool FUSED>
__device__ __noinline__ float line_round(const Prob& p, int e0, int ne, const float* __restrict__ w,
                                         const float* __restrict__ vold, float* __restrict__ vnew, float beta,
                                         bool first, float* __restrict__ z, const double* __restrict__ rhs, float* X,
                                         float* Y) {
  constexpr int NN = N1 * N1, EPL = line_round_elems<N1>();
  const int le = threadIdx.x / N1, t = threadIdx.x - le * N1;
  const bool active = le < EPL && le < ne;
  const int e = e0 + le;
  const size_t l0 = (size_t)e * NN + (size_t)N1 * t;
  const float* fe = p.fac32 + (size_t)e * 4 * NN + (size_t)N1 * t;
  float u[N1], Lu[N1];
  if (active) {
#pragma unroll
    for (int f = 0; f < 4; ++f) prefetch_l2(fe + f * NN);  // the factor lines are read two barriers later
    int sl[N1];
    load_line<N1>(p.src + l0, sl);
    if (FUSED) {
      float wl[N1], vn[N1];
      load_line<N1>(w + l0, wl);
      if (first) {
#pragma unroll
        for (int i = 0; i < N1; ++i) vn[i] = wl[i];
      } else {
        float vl[N1];
        load_line<N1>(vold + l0, vl);
#pragma unroll
        for (int i = 0; i < N1; ++i) vn[i] = wl[i] + beta * vl[i];
      }
#pragma unroll
      for (int i = 0; i < N1; ++i)
        u[i] = sl[i] == (int)(l0 + i) ? vn[i] : (first ? w[sl[i]] : w[sl[i]] + beta * vold[sl[i]]);
      store_line<N1>(vnew + l0, vn);
    } else {
#pragma unroll
      for (int i = 0; i < N1; ++i) u[i] = w[sl[i]];
    }
  }
  auto fl = [&](int f, float (&G)[N1]) { load_line<N1>(fe + f * NN, G); };
  line_op_f32<N1, 4>(reinterpret_cast<const float(&)[N1 * N1]>(c_dline[N1 - 3][0]), fl, active,
                     le < EPL ? le : 0, t, X, Y, u, Lu);
  float prod = 0.f;
  if (active) {
    if (FUSED) {
      store_line<N1>(z + l0, Lu);
#pragma unroll
      for (int i = 0; i < N1; ++i) prod += u[i] * Lu[i];
    } else {
      if (rhs) {
#pragma unroll
        for (int i = 0; i < N1; ++i) Lu[i] = (float)(rhs[l0 + i] - (double)Lu[i]);
      }
      store_line<N1>(z + l0, Lu);
    }
  }
  return prod;
}

// all rounds of element tile t in the line form (the tile's table entry is loaded by the caller's switch)
template <int N1, bool FUSED>
__device__ __forceinline__ float line_tile(const Prob& p, const ETile& t, const float* w, const float* vold,
                                           float* vnew, float beta, bool first, float* z, const double* rhs, float* X,
                                           float* Y) {
  constexpr int EPL = line_round_elems<N1>();
  float prod = 0.f;
  for (int r0 = 0; r0 < t.ne; r0 += EPL) {
    __syncthreads();  // the transpose buffers of the previous round (or tile) are free
    prod += line_round<N1, FUSED>(p, t.e0 + r0, min(EPL, t.ne - r0), w, vold, vnew, beta, first, z, rhs, X, Y);
  }
  return prod;
}

// out = L(unmask(in)) [or rhs - L(...)] for the view's element tiles (outer residual, autotuning)
template <typename R>
__global__ void __launch_bounds__(kThreads) bk_apply_plain(TileView V, const Prob* __restrict__ probs,
                                                           const Scal* __restrict__ S, const DTable* __restrict__ DT,
                                                           int vin, int vout, int residual, int gate) {
  const int nt = V.cnt[0];
  {  // one tile per block
    const int ti = blockIdx.x;
    if (ti >= nt) return;
    const ETile t = V.et[ti];
    if (skip(S[t.prob], gate)) return;
    const Prob& p = probs[t.prob];
    const int n = t.N + 1;
    const R* x = vec<R>(p, vin);
    R* out = vec<R>(p, vout);
    const double* rhs = residual ? p.f : nullptr;
    if constexpr (sizeof(R) == 4) {  // FP32: the line form of the inner iterations (what the autotuner times)
      __shared__ __align__(16) float X[kLineBuf];
      __shared__ __align__(16) float Y[kLineBuf];
#define SELF_BK_LINE(NV)                                                                                         \
  case NV:                                                                                                       \
    line_tile<NV, false>(p, t, x, nullptr, nullptr, 0.f, true, out, rhs, X, Y);                                  \
    break;
      switch (n) {
        SELF_BK_LINE(3)
        SELF_BK_LINE(4)
        SELF_BK_LINE(5)
        SELF_BK_LINE(6)
        SELF_BK_LINE(7)
        SELF_BK_LINE(8)
        SELF_BK_LINE(9)
        SELF_BK_LINE(10)
        default: break;
      }
#undef SELF_BK_LINE
      return;
    } else {
    __shared__ R sh[3 * 256];
    __shared__ R D[100];
    for (int k = threadIdx.x; k < n * n; k += blockDim.x) D[k] = (R)DT->d64[t.N][k];
    __syncthreads();
    for (int r0 = 0; r0 < t.ne; r0 += t.epr) {
      const int ne = min(t.epr, t.ne - r0);
      if (r0 > 0) __syncthreads();
      switch (n) {
        case 3: apply_body<3, R>(p, D, t.e0 + r0, ne, x, rhs, out, sh); break;
        case 4: apply_body<4, R>(p, D, t.e0 + r0, ne, x, rhs, out, sh); break;
        case 5: apply_body<5, R>(p, D, t.e0 + r0, ne, x, rhs, out, sh); break;
        case 6: apply_body<6, R>(p, D, t.e0 + r0, ne, x, rhs, out, sh); break;
        case 7: apply_body<7, R>(p, D, t.e0 + r0, ne, x, rhs, out, sh); break;
        case 8: apply_body<8, R>(p, D, t.e0 + r0, ne, x, rhs, out, sh); break;
        case 9: apply_body<9, R>(p, D, t.e0 + r0, ne, x, rhs, out, sh); break;
        case 10: apply_body<10, R>(p, D, t.e0 + r0, ne, x, rhs, out, sh); break;
        default: break;
      }
    }
    }
  }
}

// v_new = w + beta v_old on the nodes of P consecutive rounds (round q: elements e0 + q epr .. of at most epr),
// z = L(v_new gathered through src); returns the thread's sum of u * Lu.  All independent loads of the P rounds
// are issued before the gathers, so each thread keeps P chains of loads in flight.
template <int N1, typename R, int P>
__device__ __noinline__ R apply_fused_rounds(const Prob& p, const R* D, int e0, int ne, int epr, const R* w,
                                                const R* vold, R* vnew, R beta, bool first, R* z, R* sh) {
  constexpr int NN = N1 * N1;
  constexpr int EPBM = max_epb<N1>();
  const int tid = threadIdx.x % NN, le = threadIdx.x / NN;
  const int i = tid % N1, j = tid / N1;
  const R* fac = (sizeof(R) == 4) ? (const R*)p.fac32 : (const R*)p.fac64;
  bool act[P];
  int e[P], sl[P];
  size_t l[P];
  R u[P], wl[P], vl[P], G11[P], G12[P], G22[P], M[P];
#pragma unroll
  for (int q = 0; q < P; ++q) {
    const int nq = min(epr, ne - q * epr);
    e[q] = e0 + q * epr + le;
    act[q] = (le < EPBM) && (le < nq);
    l[q] = (size_t)e[q] * NN + tid;
    u[q] = G11[q] = G12[q] = G22[q] = M[q] = R(0);
    if (act[q]) {
      sl[q] = p.src[l[q]];
      wl[q] = w[l[q]];
      vl[q] = first ? R(0) : vold[l[q]];
      const R* fe = fac + (size_t)e[q] * 4 * NN;
      G11[q] = fe[tid];
      G12[q] = fe[NN + tid];
      G22[q] = fe[2 * NN + tid];
      M[q] = fe[3 * NN + tid];
    }
  }
#pragma unroll
  for (int q = 0; q < P; ++q)
    if (act[q]) {
      const R ws = w[sl[q]], vs = first ? R(0) : vold[sl[q]];
      u[q] = first ? ws : ws + beta * vs;
      vnew[l[q]] = first ? wl[q] : wl[q] + beta * vl[q];
      sh[(q * 3) * EPBM * NN + le * NN + tid] = u[q];
    }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < P; ++q)
    if (act[q]) {
      const R* su = sh + (q * 3) * EPBM * NN + le * NN;
      R us = 0, up = 0;
#pragma unroll
      for (int m = 0; m < N1; ++m) {
        us += D[i + N1 * m] * su[m + N1 * j];
        up += D[j + N1 * m] * su[i + N1 * m];
      }
      sh[(q * 3 + 1) * EPBM * NN + le * NN + tid] = G11[q] * us + G12[q] * up;
      sh[(q * 3 + 2) * EPBM * NN + le * NN + tid] = G12[q] * us + G22[q] * up;
    }
  __syncthreads();
  R prod = 0;
#pragma unroll
  for (int q = 0; q < P; ++q)
    if (act[q]) {
      const R* s1 = sh + (q * 3 + 1) * EPBM * NN + le * NN;
      const R* s2 = sh + (q * 3 + 2) * EPBM * NN + le * NN;
      R a = 0, b = 0;
#pragma unroll
      for (int m = 0; m < N1; ++m) {
        a += D[m + N1 * i] * s1[m + N1 * j];
        b += D[m + N1 * j] * s2[i + N1 * m];
      }
      const R Lu = -(a + b) - M[q] * u[q];
      z[l[q]] = Lu;
      prod += u[q] * Lu;
    }
  return prod;
}

template <typename R>
__device__ __forceinline__ void dirs(const Prob& p, int iter, R*& vold, R*& vnew) {
  R* a = vec<R>(p, V_V);
  R* b = (sizeof(R) == 4) ? (R*)p.v2_32 : (R*)p.v2_64;
  vold = (iter & 1) ? b : a;
  vnew = (iter & 1) ? a : b;
}

// inner iteration, part 1 (problems in phase 0)
template <typename R>
__global__ void __launch_bounds__(kThreads) bk_apply(TileView V, const Prob* __restrict__ probs, Scal* __restrict__ S,
                                                     const DTable* __restrict__ DT, double* __restrict__ partial,
                                                     unsigned int* __restrict__ ticket) {
  const int nt = V.cnt[0];
  {  // one tile per block
    const int ti = blockIdx.x;
    if (ti >= nt) return;
    const ETile t = V.et[ti];
    Scal& s = S[t.prob];
    if (skip(s, 0)) return;
    const Prob& p = probs[t.prob];
    const int n = t.N + 1;
    const bool first = s.iter == 0;
    const R beta = first ? R(0) : (sizeof(R) == 4 ? (R)s.beta32 : (R)s.beta);
    R *vold, *vnew;
    dirs<R>(p, s.iter, vold, vnew);
    const R* w = vec<R>(p, V_W);
    R* z = vec<R>(p, V_Z);
    R prod = 0;
    if constexpr (sizeof(R) == 4) {  // FP32: one thread per grid line
      __shared__ __align__(16) float X[kLineBuf];
      __shared__ __align__(16) float Y[kLineBuf];
#define SELF_BK_LINE(NV)                                                                                         \
  case NV:                                                                                                       \
    prod = line_tile<NV, true>(p, t, w, vold, vnew, beta, first, z, nullptr, X, Y);                              \
    break;
      switch (n) {
        SELF_BK_LINE(3)
        SELF_BK_LINE(4)
        SELF_BK_LINE(5)
        SELF_BK_LINE(6)
        SELF_BK_LINE(7)
        SELF_BK_LINE(8)
        SELF_BK_LINE(9)
        SELF_BK_LINE(10)
        default: break;
      }
#undef SELF_BK_LINE
    } else {
    __shared__ R sh[kRoundsInFlight * 3 * 256];
    __shared__ R D[100];
    for (int k = threadIdx.x; k < n * n; k += blockDim.x) D[k] = (R)DT->d64[t.N][k];
    __syncthreads();
    const int epr = t.epr;  // elements per round (one node per thread); the tile holds several rounds
    for (int r0 = 0; r0 < t.ne; r0 += kRoundsInFlight * epr) {
      const int ne = min(kRoundsInFlight * epr, t.ne - r0);
      if (r0 > 0) __syncthreads();  // scratch reuse between passes
#define SELF_BK_CASE(NV)                                                                                       \
  case NV:                                                                                                     \
    prod += apply_fused_rounds<NV, R, kRoundsInFlight>(p, D, t.e0 + r0, ne, epr, w, vold, vnew, beta, first, z, \
                                                       sh);                                                    \
    break;
      switch (n) {
        SELF_BK_CASE(3)
        SELF_BK_CASE(4)
        SELF_BK_CASE(5)
        SELF_BK_CASE(6)
        SELF_BK_CASE(7)
        SELF_BK_CASE(8)
        SELF_BK_CASE(9)
        SELF_BK_CASE(10)
        default: break;
      }
#undef SELF_BK_CASE
    }
    }
    const double bv[1] = {block_sum_r<R>(prod)};
    double tot[1];
    const int first_t = V.eptr[t.prob], count = V.eptr[t.prob + 1] - first_t;
    if (tile_last<1>(bv, partial, 0, ti, ticket + t.prob, first_t, count, tot) && threadIdx.x == 0) {
      s.vz = tot[0];
      s.alpha = s.num / tot[0];
      s.alpha32 = (float)s.alpha;
    }
  }
}

// direct-stiffness sum + mask of vector vsel on the view's group tiles
template <typename R>
__global__ void __launch_bounds__(kThreads) bk_dss(TileView V, const Prob* __restrict__ probs,
                                                   const Scal* __restrict__ S, int vsel, int gate) {
  const int nt = V.cnt[1];
  {  // one tile per block
    const int ti = blockIdx.x;
    if (ti >= nt) return;
    const GTile t = V.gt[ti];
    if (skip(S[t.prob], gate)) return;
    const Prob& p = probs[t.prob];
    R* v = vec<R>(p, vsel);
    for (int g = t.g0 + threadIdx.x; g < t.g0 + t.ng; g += blockDim.x) {
      const int a = p.gptr[g], b = p.gptr[g + 1];
      if (p.gdir[g]) {
        for (int k = a; k < b; ++k) v[p.gidx[k]] = 0;
        continue;
      }
      R sum = 0;
      for (int k = a; k < b; ++k) sum += v[p.gidx[k]];
      v[p.gidx[a]] = sum;
      for (int k = a + 1; k < b; ++k) v[p.gidx[k]] = 0;
    }
  }
}

// inner iteration, part 3: a = num / <v,z>; u += a v_new; r -= a z; w = dinv r; <r,w>, <r,r>; the problem's last
// tile closes the iteration (den = num, num = <r,w>, ||r||, inner stop test -> phase 1)
template <typename R>
__global__ void __launch_bounds__(kThreads) bk_update(TileView V, const Prob* __restrict__ probs, Scal* __restrict__ S,
                                                      double* __restrict__ partial, size_t pstride,
                                                      unsigned int* __restrict__ ticket) {
  const int nt = V.cnt[2];
  {  // one tile per block
    const int ti = blockIdx.x;
    if (ti >= nt) return;
    const VTile t = V.vt[ti];
    Scal& s = S[t.prob];
    if (skip(s, 0)) return;
    const Prob& p = probs[t.prob];
    R *vold, *v;
    dirs<R>(p, s.iter, vold, v);
    R* r = vec<R>(p, V_R);
    R* w = vec<R>(p, V_W);
    const R* z = vec<R>(p, V_Z);
    R* u = (sizeof(R) == 4) ? (R*)p.u32 : (R*)p.x;
    const R* dinv = (sizeof(R) == 4) ? (const R*)p.dinv32 : (const R*)p.dinv64;
    const R a = sizeof(R) == 4 ? (R)s.alpha32 : (R)s.alpha;
    R rw = 0, rr = 0;
    // all loads of the thread's kVecChunk / kThreads nodes first (independent), then the updates
    constexpr int Q = kVecChunk / kThreads;
    R uu[Q], vv[Q], rq[Q], zz[Q], dd[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const long long k = t.s0 + threadIdx.x + (long long)q * kThreads;
      if (k < t.s1) {
        uu[q] = u[k];
        vv[q] = v[k];
        rq[q] = r[k];
        zz[q] = z[k];
        dd[q] = dinv[k];
      }
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const long long k = t.s0 + threadIdx.x + (long long)q * kThreads;
      if (k < t.s1) {
        u[k] = uu[q] + a * vv[q];
        const R rk = rq[q] - a * zz[q];
        r[k] = rk;
        const R wk = rk * dd[q];
        w[k] = wk;
        rw += rk * wk;
        rr += rk * rk;
      }
    }
    const double bv[2] = {block_sum_r<R>(rw), block_sum_r<R>(rr)};
    double tot[2];
    const int first_t = V.vptr[t.prob], count = V.vptr[t.prob + 1] - first_t;
    if (tile_last<2>(bv, partial, pstride, ti, ticket + t.prob, first_t, count, tot) && threadIdx.x == 0) {
      const double rn = sqrt(tot[1]);
      s.den = s.num;
      s.num = tot[0];
      s.beta = s.num / s.den;
      s.beta32 = (float)s.beta;
      s.iter += 1;
      s.total += 1;
      s.rr = rn;
      if (!(rn == rn) || rn / s.rin0 < s.tol || s.total >= s.max_total || s.iter >= s.max_inner) s.phase = 1;
    }
  }
}

// start of an inner solve (problems in phase 0 with iter 0): FP32: r32 = r, u32 = 0; then w = dinv r, num = <r,w>
template <typename R>
__global__ void __launch_bounds__(kThreads) bk_start(TileView V, const Prob* __restrict__ probs, Scal* __restrict__ S,
                                                     double* __restrict__ partial, unsigned int* __restrict__ ticket) {
  const int nt = V.cnt[2];
  {  // one tile per block
    const int ti = blockIdx.x;
    if (ti >= nt) return;
    const VTile t = V.vt[ti];
    Scal& s = S[t.prob];
    if (skip(s, 3)) return;
    const Prob& p = probs[t.prob];
    R* r = vec<R>(p, V_R);
    R* w = vec<R>(p, V_W);
    const R* dinv = (sizeof(R) == 4) ? (const R*)p.dinv32 : (const R*)p.dinv64;
    R acc = 0;
    constexpr int Q = kVecChunk / kThreads;
    R rq[Q], dd[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const long long k = t.s0 + threadIdx.x + (long long)q * kThreads;
      if (k < t.s1) {
        rq[q] = (sizeof(R) == 4) ? (R)p.r[k] : r[k];
        dd[q] = dinv[k];
      }
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const long long k = t.s0 + threadIdx.x + (long long)q * kThreads;
      if (k < t.s1) {
        if (sizeof(R) == 4) {
          r[k] = rq[q];
          p.u32[k] = 0.f;
        }
        const R wk = rq[q] * dd[q];
        w[k] = wk;
        acc += rq[q] * wk;
      }
    }
    const double bv[1] = {block_sum_r<R>(acc)};
    double tot[1];
    const int first_t = V.vptr[t.prob], count = V.vptr[t.prob + 1] - first_t;
    if (tile_last<1>(bv, partial, 0, ti, ticket + t.prob, first_t, count, tot) && threadIdx.x == 0) s.num = tot[0];
  }
}

// outer step (problems in phase 1): FP32 form adds the inner correction (x += u32) unless the problem is fresh
__global__ void __launch_bounds__(kThreads) bk_correct(TileView V, const Prob* __restrict__ probs,
                                                       const Scal* __restrict__ S) {
  const int nt = V.cnt[2];
  {  // one tile per block
    const int ti = blockIdx.x;
    if (ti >= nt) return;
    const VTile t = V.vt[ti];
    if (skip(S[t.prob], 2)) return;
    const Prob& p = probs[t.prob];
    for (long long k = t.s0 + threadIdx.x; k < t.s1; k += blockDim.x) p.x[k] += (double)p.u32[k];
  }
}

// outer step: red[p] = <r, r> (FP64) of every problem in phase 1
__global__ void __launch_bounds__(kThreads) bk_rr(TileView V, const Prob* __restrict__ probs,
                                                  const Scal* __restrict__ S, double* __restrict__ partial,
                                                  unsigned int* __restrict__ ticket, double* __restrict__ red) {
  const int nt = V.cnt[2];
  {  // one tile per block
    const int ti = blockIdx.x;
    if (ti >= nt) return;
    const VTile t = V.vt[ti];
    if (skip(S[t.prob], 1)) return;
    const Prob& p = probs[t.prob];
    double acc = 0;
    for (long long k = t.s0 + threadIdx.x; k < t.s1; k += blockDim.x) acc += p.r[k] * p.r[k];
    const double bv[1] = {block_sum_r<double>(acc)};
    double tot[1];
    const int first_t = V.vptr[t.prob], count = V.vptr[t.prob + 1] - first_t;
    if (tile_last<1>(bv, partial, 0, ti, ticket + t.prob, first_t, count, tot) && threadIdx.x == 0) red[t.prob] = tot[0];
  }
}

// Outer decision of every problem in phase 1 once its FP64 residual norm squared is in red[p] -- the per-tick
// decision of the host loop, moved onto the device so that ticks need no host round trip: the first residual
// becomes r0; converged (||r||/||r0|| < tol, or r0 = 0, or a NaN), out of iterations or out of refinement steps ->
// phase 2; otherwise the next inner solve (phase 0, inner stop relative to this residual).  counters[0] = problems
// still running (phase 0 or 1); counters[1] counts loop bodies.  With use_cond, clears the persistent loop's
// condition when no problem is running or the body budget is spent.  One block.
__global__ void __launch_bounds__(kThreads) bk_decide(Scal* __restrict__ S, const double* __restrict__ red, int cap,
                                                      DecideArgs a, unsigned int* __restrict__ counters,
                                                      cudaGraphConditionalHandle cond, int use_cond) {
  int active = 0;
  for (int p = threadIdx.x; p < cap; p += kThreads) {
    Scal& s = S[p];
    if (s.phase == 1) {
      const double rn = sqrt(red[p]);
      s.rr = rn;
      if (s.fresh) {
        s.r0 = rn;
        s.fresh = 0;
      }
      const bool conv = s.r0 == 0.0 || rn / s.r0 < a.tol || !(rn == rn);
      if (conv || s.total >= a.max_total || s.outer >= a.max_outer) {
        s.phase = 2;
      } else {
        s.outer += 1;
        s.phase = 0;
        s.iter = 0;
        s.num = s.den = s.vz = 0;
        s.rin0 = rn;
        s.tol = a.fp32 ? a.inner_tol : a.tol * s.r0 / rn;
      }
    }
    if (s.phase == 0 || s.phase == 1) {
      s.max_total = a.max_total;
      s.max_inner = a.max_total;
      ++active;
    }
  }
  const double tot = block_sum_r<double>((double)active);
  if (threadIdx.x == 0) {
    counters[0] = (unsigned int)tot;
    const unsigned int bodies = ++counters[1];
    if (use_cond) cudaGraphSetConditional(cond, (tot > 0.0 && bodies < a.max_bodies) ? 1u : 0u);
  }
}

// Device compaction of a tile-table set: the tiles of the problems in phase ph, copied in order from the view of
// every problem in the pool (problem p's tiles are A.et[a_e[p] .. a_e[p+1]), A.gt[a_g[p] ..], A.vt[a_v[p] ..]).
// Part 1 (one block of 1024 threads): per-problem first tile in the compacted tables (prefix sums over the
// problems) and the tile counts.
constexpr int kScanThreads = 1024;
__global__ void __launch_bounds__(kScanThreads) bk_compact_offsets(const int* __restrict__ a_e, const int* __restrict__ a_g,
                                                                   const int* __restrict__ a_v,
                                                                   const Scal* __restrict__ S, int cap, int ph,
                                                                   int* __restrict__ d_e, int* __restrict__ d_g,
                                                                   int* __restrict__ d_v, int* __restrict__ d_cnt) {
  __shared__ int wsum[3][kScanThreads / 32];
  __shared__ int carry[3];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x < 3) carry[threadIdx.x] = 0;
  __syncthreads();
  for (int base = 0; base < cap; base += kScanThreads) {
    const int p = base + threadIdx.x;
    int c[3] = {0, 0, 0};
    if (p < cap && S[p].phase == ph) {
      c[0] = a_e[p + 1] - a_e[p];
      c[1] = a_g[p + 1] - a_g[p];
      c[2] = a_v[p + 1] - a_v[p];
    }
    int inc[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      int v = c[k];
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
      }
      inc[k] = v;
      if (lane == 31) wsum[k][wid] = v;
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        int v = wsum[k][lane];
        for (int o = 1; o < 32; o <<= 1) {
          const int t = __shfl_up_sync(0xffffffffu, v, o);
          if (lane >= o) v += t;
        }
        wsum[k][lane] = v;  // inclusive prefix over the warps
      }
    }
    __syncthreads();
    int excl[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) excl[k] = carry[k] + (wid > 0 ? wsum[k][wid - 1] : 0) + inc[k] - c[k];
    if (p < cap) {
      d_e[p] = excl[0];
      d_g[p] = excl[1];
      d_v[p] = excl[2];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
      for (int k = 0; k < 3; ++k) carry[k] += wsum[k][kScanThreads / 32 - 1];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    d_e[cap] = carry[0];
    d_g[cap] = carry[1];
    d_v[cap] = carry[2];
    d_cnt[0] = carry[0];
    d_cnt[1] = carry[1];
    d_cnt[2] = carry[2];
  }
}

// Part 2: copy the selected problems' tiles (grid-stride over every tile of the full view).
__global__ void __launch_bounds__(kThreads) bk_compact_copy(TileView A, const int* __restrict__ a_g,
                                                            const Scal* __restrict__ S, int ph, ETile* __restrict__ det,
                                                            GTile* __restrict__ dgt, VTile* __restrict__ dvt,
                                                            const int* __restrict__ d_e, const int* __restrict__ d_g,
                                                            const int* __restrict__ d_v) {
  const int ne = A.cnt[0], ng = A.cnt[1], nv = A.cnt[2];
  const int total = ne + ng + nv;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    if (i < ne) {
      const ETile t = A.et[i];
      if (S[t.prob].phase == ph) det[d_e[t.prob] + (i - A.eptr[t.prob])] = t;
    } else if (i < ne + ng) {
      const int j = i - ne;
      const GTile t = A.gt[j];
      if (S[t.prob].phase == ph) dgt[d_g[t.prob] + (j - a_g[t.prob])] = t;
    } else {
      const int j = i - ne - ng;
      const VTile t = A.vt[j];
      if (S[t.prob].phase == ph) dvt[d_v[t.prob] + (j - A.vptr[t.prob])] = t;
    }
  }
}

}  // namespace cgb
}  // namespace selfgpu

// =============================================================================================== host side
// Slots are stable problem indices; an empty slot is in phase 3 and owns no memory.
struct self_cgbatch {
  self_ctx* ctx = nullptr;
  struct Mem {
    DevBuf<float> fac32, dinv32, u32, r32, v32, w32, z32, v2_32;
    DevBuf<double> fac64, dinv64, f, x, r, v64, w64, z64, v2_64;
    DevBuf<int> src, gptr, gidx;
    DevBuf<unsigned char> gdir;
  };
  struct Slot {
    bool used = false;
    std::unique_ptr<Mem> mem;
    std::vector<double> Jww;
    std::vector<int> src, dirnodes;
    long long bytes = 0;
  };
  // one compacted tile-table set on the device (fixed capacity; contents re-uploaded when the set changes)
  struct View {
    DevBuf<selfgpu::cgb::ETile> et;
    DevBuf<selfgpu::cgb::GTile> gt;
    DevBuf<selfgpu::cgb::VTile> vt;
    DevBuf<int> cnt, eptr, vptr, gptr;  // gptr[p]: first group tile of problem p
    std::vector<int> members;  // problems of the set at the last upload
    bool valid = false;
    size_t cap_e = 0, cap_g = 0, cap_v = 0;  // table capacities
    int n_e = 0, n_g = 0, n_v = 0;           // tiles at the last upload
    selfgpu::cgb::TileView dev() const { return {et.p, gt.p, vt.p, cnt.p, eptr.p, vptr.p}; }
  };
  std::vector<Slot> slots;
  std::vector<selfgpu::cgb::Prob> hp;
  std::vector<selfgpu::cgb::Scal> hs;
  int cap = 0;
  DevBuf<selfgpu::cgb::Prob> probs;
  DevBuf<selfgpu::cgb::Scal> S;
  DevBuf<double> red, partial;
  DevBuf<unsigned int> ticket;
  DevBuf<selfgpu::cgb::DTable> DT;
  selfgpu::cgb::DTable hDT;
  bool haveD[10] = {};
  // all: every problem in the pool (uploaded by the host when the pool changes); inner / outer: the problems in
  // phase 0 / 1, compacted from `all` on the device at every tick; tune: autotuning tables
  View all, inner, outer, tune;
  DevBuf<unsigned int> counters;  // bk_decide: problems running, loop bodies
  // tick graphs (one tick = outer step + decision + inner iterations) per precision and grid level, and the
  // persistent solve graphs (the tick inside a conditional while node), captured for one set of DecideArgs
  cudaGraphExec_t tick_graphs[2][4] = {};
  cudaGraphExec_t loop_graphs[2][4] = {};
  long long tick_launches[2][4] = {};
  selfgpu::cgb::DecideArgs graph_args{};
  bool graph_args_set = false;
  size_t cap_et = 0, cap_gt = 0, cap_vt = 0;  // table capacities (tiles of every problem in the pool)
  bool dirty = true;
  int epb[10][4];
  // inner-iteration graphs per precision and grid level: level L launches capacity >> (2 L) blocks per kernel,
  // the smallest level that covers the current tile counts is replayed (blocks past the count exit at once)
  static constexpr int kLevels = 4;
  cudaGraphExec_t graphs[2][kLevels] = {};
  long long graph_launches[2][kLevels] = {};
  const double* partial_graph = nullptr;                 // partial-sum array the graphs were captured with
  int graph_k = 8;
  long long bytes_in_use = 0;
  ~self_cgbatch() {
    for (auto* set : {&graphs, &tick_graphs, &loop_graphs})
      for (auto& row : *set)
        for (auto& g : row)
          if (g) cudaGraphExecDestroy(g);
  }
};

namespace {

using namespace selfgpu::cgb;

int bucket_of(int nEl) { return nEl <= 256 ? 0 : nEl <= 1024 ? 1 : nEl <= 4096 ? 2 : 3; }
int max_epb_rt(int N) {
  const int nn = (N + 1) * (N + 1);
  return nn >= 256 ? 1 : 256 / nn;
}

template <typename T>
int put(self_ctx* ctx, DevBuf<T>& b, const T* src, size_t n) {
  if (b.alloc(n) != cudaSuccess) return set_error(ctx, SELF_ERR_ALLOC, "batch: device allocation failed");
  if (src && n) SELF_CUDA_TRY(ctx, cudaMemcpy(b.p, src, n * sizeof(T), cudaMemcpyHostToDevice));
  return SELF_OK;
}
template <typename T>
int zeros(self_ctx* ctx, DevBuf<T>& b, size_t n) {
  if (b.alloc(n) != cudaSuccess) return set_error(ctx, SELF_ERR_ALLOC, "batch: device allocation failed");
  if (n) SELF_CUDA_TRY(ctx, cudaMemset(b.p, 0, n * sizeof(T)));
  return SELF_OK;
}

void drop_graphs(self_cgbatch* b) {
  for (auto* set : {&b->graphs, &b->tick_graphs, &b->loop_graphs})
    for (auto& row : *set)
      for (auto& g : row) {
        if (g) cudaGraphExecDestroy(g);
        g = nullptr;
      }
}

// grow the slot arrays (host and device) to hold at least `want` problems
int ensure_cap(self_cgbatch* b, int want) {
  if (want <= b->cap) return SELF_OK;
  int nc = std::max(want, std::max(16, 2 * b->cap));
  b->slots.resize(nc);
  Prob empty;
  std::memset(&empty, 0, sizeof(empty));
  b->hp.resize(nc, empty);
  Scal e;
  std::memset(&e, 0, sizeof(e));
  e.phase = 3;
  b->hs.resize(nc, e);
  const int old_cap = b->cap;
  b->cap = nc;
  int rc;
  // the device slot states are the live ones (the outer decisions run on the device): the grown array keeps them,
  // and the new slots start empty (phase 3)
  DevBuf<Scal> S2;
  if (S2.alloc(nc) != cudaSuccess) return set_error(b->ctx, SELF_ERR_ALLOC, "batch: device allocation failed");
  SELF_CUDA_TRY(b->ctx, cudaStreamSynchronize(b->ctx->stream));
  if (old_cap > 0 && b->S.p)
    SELF_CUDA_TRY(b->ctx, cudaMemcpy(S2.p, b->S.p, (size_t)old_cap * sizeof(Scal), cudaMemcpyDeviceToDevice));
  SELF_CUDA_TRY(b->ctx, cudaMemcpy(S2.p + old_cap, b->hs.data() + old_cap, (size_t)(nc - old_cap) * sizeof(Scal),
                                   cudaMemcpyHostToDevice));
  std::swap(b->S.p, S2.p);
  std::swap(b->S.n, S2.n);
  if ((rc = zeros(b->ctx, b->probs, nc)) || (rc = zeros(b->ctx, b->red, nc)) || (rc = zeros(b->ctx, b->ticket, nc)))
    return rc;
  drop_graphs(b);  // the captured graphs hold the old arrays
  b->cap_et = b->cap_gt = b->cap_vt = 0;  // per-problem pointer tables are sized by the slot count
  b->dirty = true;
  return SELF_OK;
}

// Elements per element tile: a multiple of the round size max_epb_rt(N) (one node per thread, the FP64 body); the
// default is one round of the FP32 line body (256 / (N + 1) elements) rounded down to that multiple, the
// autotuner may choose another multiple.
int default_tile_elems(int N) {
  const int r = max_epb_rt(N);
  return std::max(r, (line_round_elems_rt(N) / r) * r);
}
int tile_elems(const self_cgbatch* b, const Prob& P, int force) {
  const int bk = bucket_of(P.nEl);
  const int r = max_epb_rt(P.N);
  int e = force > 0 ? force : (b->epb[P.N][bk] > 0 ? b->epb[P.N][bk] : default_tile_elems(P.N));
  return std::max(r, (e / r) * r);
}

// Upload the compacted tile tables of the problems in `members` (ascending slots) into view v.  With onlyN >= 0
// only element tiles of that degree and bucket are listed, at forceEpb elements per tile (autotuning).
int upload_view(self_cgbatch* b, self_cgbatch::View& v, const std::vector<int>& members, int onlyN = -1,
                int onlyBucket = -1, int forceEpb = 0) {
  std::vector<ETile> et;
  std::vector<GTile> gt;
  std::vector<VTile> vt;
  std::vector<int> eptr(b->cap + 1, 0), vptr(b->cap + 1, 0), gptr(b->cap + 1, 0);
  size_t m = 0;
  for (int p = 0; p < b->cap; ++p) {
    eptr[p] = (int)et.size();
    vptr[p] = (int)vt.size();
    gptr[p] = (int)gt.size();
    if (m >= members.size() || members[m] != p) continue;
    ++m;
    const Prob& P = b->hp[p];
    const bool sel = (onlyN < 0 || P.N == onlyN) && (onlyBucket < 0 || bucket_of(P.nEl) == onlyBucket);
    const int e = tile_elems(b, P, forceEpb);
    if (sel)
      for (int e0 = 0; e0 < P.nEl; e0 += e) et.push_back(ETile{p, P.N, e0, std::min(e, P.nEl - e0), max_epb_rt(P.N)});
    for (int g0 = 0; g0 < P.ngroups; g0 += kThreads) gt.push_back(GTile{p, g0, std::min(kThreads, P.ngroups - g0)});
    for (long long s0 = 0; s0 < P.nl; s0 += kVecChunk)
      vt.push_back(VTile{p, s0, std::min<long long>(P.nl, s0 + kVecChunk)});
  }
  eptr[b->cap] = (int)et.size();
  vptr[b->cap] = (int)vt.size();
  gptr[b->cap] = (int)gt.size();
  if (et.size() > v.cap_e || gt.size() > v.cap_g || vt.size() > v.cap_v)
    return set_error(b->ctx, SELF_ERR_INVALID, "batch: tile tables exceed their capacity");
  const int cnt[3] = {(int)et.size(), (int)gt.size(), (int)vt.size()};
  cudaStream_t st = b->ctx->stream;
  // the copies are ordered before the next launches of the stream (host vectors are copied synchronously
  // with respect to the host for pageable memory)
  if (!et.empty()) SELF_CUDA_TRY(b->ctx, cudaMemcpyAsync(v.et.p, et.data(), et.size() * sizeof(ETile), cudaMemcpyHostToDevice, st));
  if (!gt.empty()) SELF_CUDA_TRY(b->ctx, cudaMemcpyAsync(v.gt.p, gt.data(), gt.size() * sizeof(GTile), cudaMemcpyHostToDevice, st));
  if (!vt.empty()) SELF_CUDA_TRY(b->ctx, cudaMemcpyAsync(v.vt.p, vt.data(), vt.size() * sizeof(VTile), cudaMemcpyHostToDevice, st));
  SELF_CUDA_TRY(b->ctx, cudaMemcpyAsync(v.cnt.p, cnt, sizeof(cnt), cudaMemcpyHostToDevice, st));
  SELF_CUDA_TRY(b->ctx, cudaMemcpyAsync(v.eptr.p, eptr.data(), eptr.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  SELF_CUDA_TRY(b->ctx, cudaMemcpyAsync(v.vptr.p, vptr.data(), vptr.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  SELF_CUDA_TRY(b->ctx, cudaMemcpyAsync(v.gptr.p, gptr.data(), gptr.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  SELF_CUDA_TRY(b->ctx, cudaStreamSynchronize(st));  // host vectors go out of scope
  v.members = members;
  v.valid = onlyN < 0;
  v.n_e = cnt[0];
  v.n_g = cnt[1];
  v.n_v = cnt[2];
  return SELF_OK;
}

int alloc_view(self_cgbatch* b, self_cgbatch::View& v, size_t ce, size_t cg, size_t cv) {
  int rc;
  v.cap_e = std::max<size_t>(1, ce);
  v.cap_g = std::max<size_t>(1, cg);
  v.cap_v = std::max<size_t>(1, cv);
  if ((rc = zeros(b->ctx, v.et, v.cap_e)) || (rc = zeros(b->ctx, v.gt, v.cap_g)) || (rc = zeros(b->ctx, v.vt, v.cap_v)) ||
      (rc = zeros(b->ctx, v.cnt, 3)) || (rc = zeros(b->ctx, v.eptr, (size_t)b->cap + 1)) ||
      (rc = zeros(b->ctx, v.vptr, (size_t)b->cap + 1)) || (rc = zeros(b->ctx, v.gptr, (size_t)b->cap + 1)))
    return rc;
  v.members.clear();
  v.valid = false;
  v.n_e = v.n_g = v.n_v = 0;
  return SELF_OK;
}

// c_dline of this device for N1 = n: set from D (column-major FP64, rounded to FP32) by the first problem of the
// degree, compared with it for every later one (the batched FP32 operator reads the table, not the problem's D)
int set_dline(self_ctx* ctx, int n, const std::vector<double>& D) {
  static std::mutex mu;
  static std::vector<std::vector<float>> tables;  // [device * 8 + n - 3]
  std::lock_guard<std::mutex> lock(mu);
  const size_t slot = (size_t)ctx->device * 8 + (size_t)(n - 3);
  if (tables.size() <= slot) tables.resize(slot + 1);
  std::vector<float> d32(D.begin(), D.begin() + (size_t)n * n);
  std::vector<float>& T = tables[slot];
  if (T.empty()) {
    SELF_CUDA_TRY(ctx, cudaMemcpyToSymbol(c_dline, d32.data(), d32.size() * sizeof(float),
                                          (size_t)(n - 3) * 100 * sizeof(float), cudaMemcpyHostToDevice));
    T = d32;
  } else if (T != d32) {
    return set_error(ctx, SELF_ERR_UNSUPPORTED,
                     "batched solver: derivative matrix of degree %d differs from the one in use on this device", n - 1);
  }
  return SELF_OK;
}

// After the pool changed: upload the problem descriptors, size the tables for every problem (at the largest
// tile count any element-per-tile choice gives) and drop the captured graphs if the table buffers moved.
int refresh(self_cgbatch* b) {
  if (!b->dirty) return SELF_OK;
  int rc;
  // descriptors and derivative tables are copied into the existing arrays (the captured graphs hold them)
  SELF_CUDA_TRY(b->ctx, cudaMemcpy(b->probs.p, b->hp.data(), (size_t)b->cap * sizeof(Prob), cudaMemcpyHostToDevice));
  if (!b->DT.p) {
    if ((rc = put(b->ctx, b->DT, &b->hDT, 1))) return rc;
  } else {
    SELF_CUDA_TRY(b->ctx, cudaMemcpy(b->DT.p, &b->hDT, sizeof(DTable), cudaMemcpyHostToDevice));
  }
  size_t ne = 0, ng = 0, nv = 0, ne1 = 0;
  for (int p = 0; p < b->cap; ++p) {
    if (!b->slots[p].used) continue;
    const Prob& P = b->hp[p];
    const size_t te = (size_t)tile_elems(b, P, 0), r = (size_t)max_epb_rt(P.N);
    ne += ((size_t)P.nEl + te - 1) / te;
    ne1 += ((size_t)P.nEl + r - 1) / r;  // one round per tile: the most tiles the autotuner lists
    ng += ((size_t)P.ngroups + kThreads - 1) / kThreads;
    nv += ((size_t)P.nl + kVecChunk - 1) / kVecChunk;
  }
  if (ne > b->cap_et || ng > b->cap_gt || nv > b->cap_vt || !b->inner.et.p) {
    // the inner iteration graph launches one block per table slot, so the capacity is its grid
    b->cap_et = std::max(ne, b->cap_et + b->cap_et / 4);
    b->cap_gt = std::max(ng, b->cap_gt + b->cap_gt / 4);
    b->cap_vt = std::max(nv, b->cap_vt + b->cap_vt / 4);
    if ((rc = alloc_view(b, b->inner, b->cap_et, b->cap_gt, b->cap_vt)) ||
        (rc = alloc_view(b, b->outer, b->cap_et, b->cap_gt, b->cap_vt)) ||
        (rc = alloc_view(b, b->all, b->cap_et, b->cap_gt, b->cap_vt)))
      return rc;
    drop_graphs(b);
  } else {
    b->inner.valid = b->outer.valid = b->all.valid = false;  // same buffers, new contents on the next use
  }
  if (!b->counters.p && (rc = zeros(b->ctx, b->counters, 2))) return rc;
  if (ne1 > b->tune.cap_e || !b->tune.et.p)
    if ((rc = alloc_view(b, b->tune, ne1, ng, nv))) return rc;
  const size_t np = std::max({b->cap_et, 2 * b->cap_vt, b->tune.cap_e});
  if (b->partial.n < np && (rc = zeros(b->ctx, b->partial, np))) return rc;
  if (b->partial_graph != b->partial.p) drop_graphs(b);
  b->partial_graph = b->partial.p;
  b->dirty = false;
  return SELF_OK;
}

int ensure_view(self_cgbatch* b, self_cgbatch::View& v, const std::vector<int>& members) {
  if (v.valid && v.members == members) return SELF_OK;
  return upload_view(b, v, members);
}

// grids: one block per tile; launches inside the captured inner graph use the table capacity (the tile count
// changes between ticks), direct launches use the count of the last upload
template <typename R>
int k_apply_plain(self_cgbatch* b, const self_cgbatch::View& v, int vin, int vout, int residual, int gate) {
  if (v.n_e == 0) return SELF_OK;
  bk_apply_plain<R><<<v.n_e, kThreads, 0, b->ctx->stream>>>(v.dev(), b->probs.p, b->S.p, b->DT.p, vin, vout,
                                                            residual, gate);
  SELF_LAUNCHED(b->ctx);
  return SELF_OK;
}
template <typename R>
int k_dss(self_cgbatch* b, const self_cgbatch::View& v, int vsel, int gate, bool in_graph) {
  const int grid = in_graph ? (int)v.cap_g : v.n_g;
  if (grid == 0) return SELF_OK;
  bk_dss<R><<<grid, kThreads, 0, b->ctx->stream>>>(v.dev(), b->probs.p, b->S.p, vsel, gate);
  SELF_LAUNCHED(b->ctx);
  return SELF_OK;
}

// grid of a table with capacity cap at level L (at least one block)
inline int level_grid(size_t cap, int L) { return (int)std::max<size_t>(1, cap >> (2 * L)); }

// inner iterations: graph = start (problems entering an inner solve) + graph_k x (apply, dss, update)
template <typename R>
int enqueue_inner(self_cgbatch* b, int L) {
  cudaStream_t st = b->ctx->stream;
  const TileView V = b->inner.dev();
  const int ge = level_grid(b->inner.cap_e, L), gv = level_grid(b->inner.cap_v, L);
  bk_start<R><<<gv, kThreads, 0, st>>>(V, b->probs.p, b->S.p, b->partial.p, b->ticket.p);
  SELF_LAUNCHED(b->ctx);
  for (int k = 0; k < b->graph_k; ++k) {
    bk_apply<R><<<ge, kThreads, 0, st>>>(V, b->probs.p, b->S.p, b->DT.p, b->partial.p, b->ticket.p);
    SELF_LAUNCHED(b->ctx);
    if (b->inner.cap_g > 0) {
      bk_dss<R><<<level_grid(b->inner.cap_g, L), kThreads, 0, st>>>(V, b->probs.p, b->S.p, V_Z, 0);
      SELF_LAUNCHED(b->ctx);
    }
    bk_update<R><<<gv, kThreads, 0, st>>>(V, b->probs.p, b->S.p, b->partial.p, b->inner.cap_v, b->ticket.p);
    SELF_LAUNCHED(b->ctx);
  }
  return SELF_OK;
}

// Compaction of view D (problems in phase ph) from the pool view, at grid level L
int enqueue_compact(self_cgbatch* b, self_cgbatch::View& D, int ph, int L) {
  cudaStream_t st = b->ctx->stream;
  const self_cgbatch::View& A = b->all;
  bk_compact_offsets<<<1, kScanThreads, 0, st>>>(A.eptr.p, A.gptr.p, A.vptr.p, b->S.p, b->cap, ph, D.eptr.p, D.gptr.p,
                                                 D.vptr.p, D.cnt.p);
  SELF_LAUNCHED(b->ctx);
  const size_t tiles = A.cap_e + A.cap_g + A.cap_v;
  const int grid = (int)std::max<size_t>(1, std::min<size_t>((tiles + kThreads - 1) / kThreads >> (2 * L), 4096));
  bk_compact_copy<<<grid, kThreads, 0, st>>>(A.dev(), A.gptr.p, b->S.p, ph, D.et.p, D.gt.p, D.vt.p, D.eptr.p,
                                             D.gptr.p, D.vptr.p);
  SELF_LAUNCHED(b->ctx);
  return SELF_OK;
}

// One tick on the device, enqueued (and captured into a graph by the callers): the outer step of the problems in
// phase 1 (FP32 form: x += the inner correction; FP64 residual r = b - A x and <r, r>), the outer decision
// (bk_decide), then the start of new inner solves and graph_k inner PCG iterations of the problems in phase 0.
// Both sets are compacted on the device, so the tick needs nothing from the host.
template <typename R>
int enqueue_tick(self_cgbatch* b, int L, const DecideArgs& da, cudaGraphConditionalHandle cond, int use_cond) {
  cudaStream_t st = b->ctx->stream;
  int rc;
  const auto& O = b->outer;
  const TileView VO = O.dev();
  if ((rc = enqueue_compact(b, b->outer, 1, L))) return rc;
  const int ge = level_grid(O.cap_e, L), gg = level_grid(O.cap_g, L), gv = level_grid(O.cap_v, L);
  if (sizeof(R) == 4) {  // x += u32 for problems whose inner solve ended
    bk_correct<<<gv, kThreads, 0, st>>>(VO, b->probs.p, b->S.p);
    SELF_LAUNCHED(b->ctx);
  }
  bk_apply_plain<double><<<ge, kThreads, 0, st>>>(VO, b->probs.p, b->S.p, b->DT.p, V_X, V_R, 1, 1);
  SELF_LAUNCHED(b->ctx);
  bk_dss<double><<<gg, kThreads, 0, st>>>(VO, b->probs.p, b->S.p, V_R, 1);
  SELF_LAUNCHED(b->ctx);
  bk_rr<<<gv, kThreads, 0, st>>>(VO, b->probs.p, b->S.p, b->partial.p, b->ticket.p, b->red.p);
  SELF_LAUNCHED(b->ctx);
  bk_decide<<<1, kThreads, 0, st>>>(b->S.p, b->red.p, b->cap, da, b->counters.p, cond, use_cond);
  SELF_LAUNCHED(b->ctx);
  if ((rc = enqueue_compact(b, b->inner, 0, L))) return rc;
  return enqueue_inner<R>(b, L);
}

DecideArgs decide_args(const self_solve_opts* o) {
  const bool fp32 = o->precision == SELF_PREC_FP32;
  DecideArgs a{};
  a.tol = o->tolerance;
  a.inner_tol = fp32 ? (o->inner_tolerance > 0 ? o->inner_tolerance : 1e-4) : o->tolerance;
  a.fp32 = fp32 ? 1 : 0;
  a.max_outer = fp32 ? (o->max_outer > 0 ? o->max_outer : 30) : 2;
  a.max_total = o->maxIters;
  // every loop body moves each running problem by at least one inner iteration or one refinement decision
  a.max_bodies = (unsigned int)std::min<long long>(2000000000LL, (long long)o->maxIters + 2LL * a.max_outer + 16);
  return a;
}

// Pool view upload (when the pool changed) and the smallest grid level covering its tiles.
int prepare(self_cgbatch* b, const self_solve_opts* o, int* level) {
  int rc;
  if ((rc = refresh(b))) return rc;
  std::vector<int> used;
  for (int p = 0; p < b->cap; ++p)
    if (b->slots[p].used) used.push_back(p);
  if ((rc = ensure_view(b, b->all, used))) return rc;
  int L = self_cgbatch::kLevels - 1;
  while (L > 0 && ((size_t)b->all.n_e > (size_t)level_grid(b->all.cap_e, L) ||
                   (size_t)b->all.n_g > (size_t)level_grid(b->all.cap_g, L) ||
                   (size_t)b->all.n_v > (size_t)level_grid(b->all.cap_v, L)))
    --L;
  *level = L;
  const DecideArgs a = decide_args(o);
  if (b->graph_args_set && std::memcmp(&a, &b->graph_args, sizeof(a)) != 0) drop_graphs(b);
  b->graph_args = a;
  b->graph_args_set = true;
  return SELF_OK;
}

// Tick graph of the given precision and level (captured once).
int tick_graph(self_cgbatch* b, bool fp32, int L, cudaGraphExec_t* out) {
  self_ctx* ctx = b->ctx;
  cudaGraphExec_t& G = b->tick_graphs[fp32 ? 1 : 0][L];
  if (!G) {
    cudaGraph_t g;
    const long long l0 = ctx->launches.load();
    SELF_CUDA_TRY(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    int rc = fp32 ? enqueue_tick<float>(b, L, b->graph_args, 0, 0) : enqueue_tick<double>(b, L, b->graph_args, 0, 0);
    cudaError_t ce = cudaStreamEndCapture(ctx->stream, &g);
    if (rc) return rc;
    if (ce != cudaSuccess) return set_error(ctx, SELF_ERR_CUDA, "batch graph capture: %s", cudaGetErrorString(ce));
    ce = cudaGraphInstantiate(&G, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return set_error(ctx, SELF_ERR_CUDA, "batch graph instantiate: %s", cudaGetErrorString(ce));
    b->tick_launches[fp32 ? 1 : 0][L] = ctx->launches.load() - l0;
    ctx->launches.fetch_sub(b->tick_launches[fp32 ? 1 : 0][L]);
  }
  *out = G;
  return SELF_OK;
}

// Persistent solve graph: the tick as the body of a conditional while node whose condition bk_decide clears when
// no problem is running (or the body budget is spent), so a whole batched solve is one graph launch.
int loop_graph(self_cgbatch* b, bool fp32, int L, cudaGraphExec_t* out) {
  self_ctx* ctx = b->ctx;
  cudaGraphExec_t& G = b->loop_graphs[fp32 ? 1 : 0][L];
  if (!G) {
    cudaGraph_t g = nullptr;
    SELF_CUDA_TRY(ctx, cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle cond;
    cudaError_t ce = cudaGraphConditionalHandleCreate(&cond, g, 1u, cudaGraphCondAssignDefault);
    if (ce != cudaSuccess) {
      cudaGraphDestroy(g);
      return set_error(ctx, SELF_ERR_CUDA, "conditional handle: %s", cudaGetErrorString(ce));
    }
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = cond;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    ce = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np);
    if (ce != cudaSuccess) {
      cudaGraphDestroy(g);
      return set_error(ctx, SELF_ERR_CUDA, "conditional node: %s", cudaGetErrorString(ce));
    }
    cudaGraph_t body = np.conditional.phGraph_out[0];
    const long long l0 = ctx->launches.load();
    ce = cudaStreamBeginCaptureToGraph(ctx->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (ce != cudaSuccess) {
      cudaGraphDestroy(g);
      return set_error(ctx, SELF_ERR_CUDA, "capture into the loop body: %s", cudaGetErrorString(ce));
    }
    int rc = fp32 ? enqueue_tick<float>(b, L, b->graph_args, cond, 1) : enqueue_tick<double>(b, L, b->graph_args, cond, 1);
    ce = cudaStreamEndCapture(ctx->stream, &body);
    ctx->launches.fetch_sub(ctx->launches.load() - l0);
    if (rc || ce != cudaSuccess) {
      cudaGraphDestroy(g);
      return rc ? rc : set_error(ctx, SELF_ERR_CUDA, "loop body capture: %s", cudaGetErrorString(ce));
    }
    ce = cudaGraphInstantiate(&G, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return set_error(ctx, SELF_ERR_CUDA, "loop graph instantiate: %s", cudaGetErrorString(ce));
  }
  *out = G;
  return SELF_OK;
}

// Enqueue one tick (no host synchronisation); the slot states are copied into hs by the next sync_states.
int tick_async(self_cgbatch* b, const self_solve_opts* o) {
  self_ctx* ctx = b->ctx;
  int rc, L;
  if ((rc = prepare(b, o, &L))) return rc;
  const bool fp32 = o->precision == SELF_PREC_FP32;
  cudaGraphExec_t G;
  if ((rc = tick_graph(b, fp32, L, &G))) return rc;
  SELF_CUDA_TRY(ctx, cudaGraphLaunch(G, ctx->stream));
  ctx->launches.fetch_add(b->tick_launches[fp32 ? 1 : 0][L]);
  return SELF_OK;
}

// Device slot states into hs (waits for the stream).
int sync_states(self_cgbatch* b) {
  self_ctx* ctx = b->ctx;
  SELF_CUDA_TRY(ctx, cudaMemcpyAsync(b->hs.data(), b->S.p, b->cap * sizeof(Scal), cudaMemcpyDeviceToHost, ctx->stream));
  SELF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return SELF_OK;
}

int tick(self_cgbatch* b, const self_solve_opts* o, int* nfinished) {
  int rc;
  if ((rc = tick_async(b, o)) || (rc = sync_states(b))) return rc;
  int fin = 0;
  for (int p = 0; p < b->cap; ++p) fin += b->slots[p].used && b->hs[p].phase == 2;
  if (nfinished) *nfinished = fin;
  return SELF_OK;
}

// Device copy of slot p's state (stream-ordered before the next tick)
int put_state(self_cgbatch* b, int p) {
  SELF_CUDA_TRY(b->ctx, cudaMemcpyAsync(b->S.p + p, &b->hs[p], sizeof(Scal), cudaMemcpyHostToDevice, b->ctx->stream));
  return SELF_OK;
}

int add_problem(self_cgbatch* b, const self_cg2d_desc* d, const double* source, int* slot_out) {
  self_ctx* ctx = b->ctx;
  selfgpu::cg::HostCompiled hc;
  int rc;
  if ((rc = selfgpu::cg::compile_host(ctx, d, hc))) return rc;
  int slot = -1;
  for (int p = 0; p < b->cap; ++p)
    if (!b->slots[p].used) {
      slot = p;
      break;
    }
  if (slot < 0) {
    slot = b->cap;
    if ((rc = ensure_cap(b, b->cap + 1))) return rc;
  }
  const int n = hc.n;
  if (n < 3 || n > 10) return set_error(b->ctx, SELF_ERR_UNSUPPORTED, "batched solver: degree %d outside 2..9", hc.N);
  if ((rc = set_dline(b->ctx, n, hc.D))) return rc;
  if (!b->haveD[hc.N]) {
    for (int k = 0; k < n * n; ++k) {
      b->hDT.d64[hc.N][k] = hc.D[k];
      b->hDT.d32[hc.N][k] = (float)hc.D[k];
    }
    b->haveD[hc.N] = true;
  }
  auto m = std::make_unique<self_cgbatch::Mem>();
  const size_t nl = hc.nl;
  std::vector<float> f32(hc.fac.begin(), hc.fac.end()), d32(hc.dinv.begin(), hc.dinv.end());
  if ((rc = put(ctx, m->fac64, hc.fac.data(), hc.fac.size())) || (rc = put(ctx, m->fac32, f32.data(), f32.size())) ||
      (rc = put(ctx, m->dinv64, hc.dinv.data(), nl)) || (rc = put(ctx, m->dinv32, d32.data(), nl)) ||
      (rc = put(ctx, m->src, hc.src.data(), nl)) || (rc = put(ctx, m->gptr, hc.gptr.data(), hc.gptr.size())) ||
      (rc = put(ctx, m->gidx, hc.gidx.data(), hc.gidx.size())) || (rc = put(ctx, m->gdir, hc.gdir.data(), hc.gdir.size())))
    return rc;
  if ((rc = zeros(ctx, m->f, nl)) || (rc = zeros(ctx, m->x, nl)) || (rc = zeros(ctx, m->r, nl)) ||
      (rc = zeros(ctx, m->v64, nl)) || (rc = zeros(ctx, m->w64, nl)) || (rc = zeros(ctx, m->z64, nl)) ||
      (rc = zeros(ctx, m->u32, nl)) || (rc = zeros(ctx, m->r32, nl)) || (rc = zeros(ctx, m->v32, nl)) ||
      (rc = zeros(ctx, m->w32, nl)) || (rc = zeros(ctx, m->z32, nl)) || (rc = zeros(ctx, m->v2_32, nl)) ||
      (rc = zeros(ctx, m->v2_64, nl)))
    return rc;
  Prob P;
  P.N = hc.N;
  P.n = n;
  P.nEl = hc.nEl;
  P.ngroups = hc.ngroups;
  P.nl = (long long)nl;
  P.fac32 = m->fac32.p;
  P.fac64 = m->fac64.p;
  P.dinv32 = m->dinv32.p;
  P.dinv64 = m->dinv64.p;
  P.src = m->src.p;
  P.gptr = m->gptr.p;
  P.gidx = m->gidx.p;
  P.gdir = m->gdir.p;
  P.f = m->f.p;
  P.x = m->x.p;
  P.r = m->r.p;
  P.v64 = m->v64.p;
  P.w64 = m->w64.p;
  P.z64 = m->z64.p;
  P.u32 = m->u32.p;
  P.r32 = m->r32.p;
  P.v32 = m->v32.p;
  P.w32 = m->w32.p;
  P.z32 = m->z32.p;
  P.v2_32 = m->v2_32.p;
  P.v2_64 = m->v2_64.p;
  if (source) {
    std::vector<double> f(nl);
    for (size_t k = 0; k < nl; ++k) f[k] = source[k] * hc.Jww[k];
    SELF_CUDA_TRY(ctx, cudaMemcpy(P.f, f.data(), nl * sizeof(double), cudaMemcpyHostToDevice));
  }
  self_cgbatch::Slot& S = b->slots[slot];
  S.used = true;
  S.bytes = (long long)(m->fac32.bytes() + m->dinv32.bytes() + 6 * nl * 4 + m->fac64.bytes() + m->dinv64.bytes() +
                        7 * nl * 8 + m->src.bytes() + m->gptr.bytes() + m->gidx.bytes() + m->gdir.bytes());
  b->bytes_in_use += S.bytes;
  S.mem = std::move(m);
  S.Jww = std::move(hc.Jww);
  S.dirnodes.clear();
  for (int g = 0; g < hc.ngroups; ++g)
    if (hc.gdir[g])
      for (int k = hc.gptr[g]; k < hc.gptr[g + 1]; ++k) S.dirnodes.push_back(hc.gidx[k]);
  S.src = std::move(hc.src);
  b->hp[slot] = P;
  Scal& sc = b->hs[slot];
  std::memset(&sc, 0, sizeof(sc));
  sc.phase = 1;
  sc.fresh = 1;
  b->dirty = true;
  *slot_out = slot;
  return put_state(b, slot);
}

}  // namespace

extern "C" {

int self_cgbatch_create(self_ctx* ctx, int nprob, const self_cg2d_desc* descs, self_cgbatch** out) {
  if (!ctx || nprob < 0 || (nprob > 0 && !descs) || !out) return SELF_ERR_INVALID;
  SELF_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  std::unique_ptr<self_cgbatch> b(new self_cgbatch());
  b->ctx = ctx;
  std::memset(b->epb, 0, sizeof(b->epb));
  std::memset(&b->hDT, 0, sizeof(b->hDT));
  int rc;
  if ((rc = ensure_cap(b.get(), std::max(nprob, 1)))) return rc;
  for (int p = 0; p < nprob; ++p) {
    int slot;
    if ((rc = add_problem(b.get(), &descs[p], nullptr, &slot))) return rc;
  }
  *out = b.release();
  return SELF_OK;
}

int self_cgbatch_destroy(self_cgbatch* b) {
  if (!b) return SELF_OK;
  cudaSetDevice(b->ctx->device);
  cudaStreamSynchronize(b->ctx->stream);
  delete b;
  return SELF_OK;
}

int self_cgbatch_add(self_cgbatch* b, const self_cg2d_desc* desc, const double* source, int* slot) {
  if (!b || !desc || !source || !slot) return SELF_ERR_INVALID;
  SELF_CUDA_TRY(b->ctx, cudaSetDevice(b->ctx->device));
  return add_problem(b, desc, source, slot);
}

int self_cgbatch_remove(self_cgbatch* b, int p) {
  if (!b || p < 0 || p >= b->cap || !b->slots[p].used) return SELF_ERR_INVALID;
  SELF_CUDA_TRY(b->ctx, cudaSetDevice(b->ctx->device));
  SELF_CUDA_TRY(b->ctx, cudaStreamSynchronize(b->ctx->stream));
  auto& S = b->slots[p];
  b->bytes_in_use -= S.bytes;
  S = self_cgbatch::Slot();
  std::memset(&b->hp[p], 0, sizeof(Prob));
  std::memset(&b->hs[p], 0, sizeof(Scal));
  b->hs[p].phase = 3;
  b->dirty = true;
  return put_state(b, p);
}

int self_cgbatch_footprint(const self_cg2d_desc* d, long long* bytes) {
  if (!d || !bytes) return SELF_ERR_INVALID;
  const long long nl = (long long)(d->N + 1) * (d->N + 1) * d->nEl;
  // FP32: 4 factors + diag + 6 vectors; FP64: 4 factors + diag + 7 vectors; src + groups
  *bytes = nl * (11 * 4 + 12 * 8 + 4 + 8) + 4096;
  return SELF_OK;
}

int self_cgbatch_set_source(self_cgbatch* b, int p, const double* source) {
  if (!b || p < 0 || p >= b->cap || !b->slots[p].used || !source) return SELF_ERR_INVALID;
  SELF_CUDA_TRY(b->ctx, cudaSetDevice(b->ctx->device));
  const auto& J = b->slots[p].Jww;
  std::vector<double> f(J.size());
  for (size_t k = 0; k < f.size(); ++k) f[k] = source[k] * J[k];
  SELF_CUDA_TRY(b->ctx, cudaMemcpy(b->hp[p].f, f.data(), f.size() * sizeof(double), cudaMemcpyHostToDevice));
  Scal& s = b->hs[p];
  std::memset(&s, 0, sizeof(s));
  s.phase = 1;
  s.fresh = 1;
  SELF_CUDA_TRY(b->ctx, cudaMemset(b->hp[p].x, 0, b->hp[p].nl * sizeof(double)));
  int rc = put_state(b, p);
  if (rc) return rc;
  SELF_CUDA_TRY(b->ctx, cudaStreamSynchronize(b->ctx->stream));
  return SELF_OK;
}

int self_cgbatch_problem_size(self_cgbatch* b, int p, long long* nl) {
  if (!b || p < 0 || p >= b->cap || !b->slots[p].used || !nl) return SELF_ERR_INVALID;
  *nl = b->hp[p].nl;
  return SELF_OK;
}

int self_cgbatch_get_solution(self_cgbatch* b, int p, double* solution) {
  if (!b || p < 0 || p >= b->cap || !b->slots[p].used || !solution) return SELF_ERR_INVALID;
  SELF_CUDA_TRY(b->ctx, cudaSetDevice(b->ctx->device));
  const size_t nl = (size_t)b->hp[p].nl;
  std::vector<double> x(nl);
  SELF_CUDA_TRY(b->ctx, cudaMemcpy(x.data(), b->hp[p].x, nl * sizeof(double), cudaMemcpyDeviceToHost));
  const auto& src = b->slots[p].src;
  for (size_t k = 0; k < nl; ++k) solution[k] = x[src[k]];  // UnMask
  for (int l : b->slots[p].dirnodes) solution[l] = 0.0;      // homogeneous Dirichlet values
  return SELF_OK;
}

int self_cgbatch_report(self_cgbatch* b, int p, self_solve_report* rep, int* finished) {
  if (!b || p < 0 || p >= b->cap || !b->slots[p].used || !rep) return SELF_ERR_INVALID;
  const Scal& s = b->hs[p];
  const double rel = s.r0 > 0 ? s.rr / s.r0 : 0.0;
  rep->ioerr = (s.phase == 2 && rel < 1e300 && (s.r0 == 0 || rel == rel)) ? 0 : -2;
  rep->iterations = s.total;
  rep->outer_iterations = s.outer;
  rep->r0 = s.r0;
  rep->rel_residual = rel;
  if (finished) *finished = s.phase == 2;
  return SELF_OK;
}

int self_cgbatch_step(self_cgbatch* b, const self_solve_opts* o, int* nfinished) {
  if (!b || !o || !(o->tolerance > 0) || o->maxIters < 1) return SELF_ERR_INVALID;
  SELF_CUDA_TRY(b->ctx, cudaSetDevice(b->ctx->device));
  return tick(b, o, nfinished);
}

long long self_cgbatch_bytes(const self_cgbatch* b) { return b ? b->bytes_in_use : 0; }

// Solve every problem in the batch from a zero initial guess: one launch of the persistent loop graph (ticks run
// on the device until every problem finished), then the slot states are read back once.
int self_cgbatch_solve(self_cgbatch* b, const self_solve_opts* o, self_solve_report* reports) {
  if (!b || !o || !(o->tolerance > 0) || o->maxIters < 1) return SELF_ERR_INVALID;
  self_ctx* ctx = b->ctx;
  SELF_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  int nused = 0;
  for (int p = 0; p < b->cap; ++p) {
    if (!b->slots[p].used) continue;
    ++nused;
    Scal& s = b->hs[p];
    std::memset(&s, 0, sizeof(s));
    s.phase = 1;
    s.fresh = 1;
    SELF_CUDA_TRY(ctx, cudaMemsetAsync(b->hp[p].x, 0, b->hp[p].nl * sizeof(double), ctx->stream));
  }
  int rc, L;
  SELF_CUDA_TRY(ctx, cudaMemcpyAsync(b->S.p, b->hs.data(), b->cap * sizeof(Scal), cudaMemcpyHostToDevice, ctx->stream));
  if (nused > 0) {
    if ((rc = prepare(b, o, &L))) return rc;
    const bool fp32 = o->precision == SELF_PREC_FP32;
    cudaGraphExec_t G;
    if ((rc = loop_graph(b, fp32, L, &G))) return rc;
    SELF_CUDA_TRY(ctx, cudaMemsetAsync(b->counters.p, 0, 2 * sizeof(unsigned int), ctx->stream));
    SELF_CUDA_TRY(ctx, cudaGraphLaunch(G, ctx->stream));
  }
  if ((rc = sync_states(b))) return rc;
  int k = 0;
  for (int p = 0; p < b->cap; ++p) {
    if (!b->slots[p].used) continue;
    int f;
    self_solve_report r;
    self_cgbatch_report(b, p, &r, &f);
    if (r.rel_residual >= o->tolerance || !f) r.ioerr = -1;
    if (reports) reports[k] = r;
    ++k;
  }
  return SELF_OK;
}

// Measure elements-per-CTA choices of the element operator for each (N, element-count bucket) present and
// keep the fastest; results are written to / read from a small JSON file when cache_path is given.
int self_cgbatch_autotune(self_cgbatch* b, const char* cache_path) {
  if (!b) return SELF_ERR_INVALID;
  self_ctx* ctx = b->ctx;
  SELF_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  bool present[10][4] = {};
  for (int p = 0; p < b->cap; ++p)
    if (b->slots[p].used) present[b->hp[p].N][bucket_of(b->hp[p].nEl)] = true;
  if (cache_path) {
    FILE* fp = fopen(cache_path, "r");
    if (fp) {
      char line[256];
      while (fgets(line, sizeof(line), fp)) {
        int N, bk, e;
        if (sscanf(line, " { \"N\": %d, \"bucket\": %d, \"epb\": %d", &N, &bk, &e) == 3 && N >= 2 && N <= 9 &&
            bk >= 0 && bk < 4 && e >= 1)
          b->epb[N][bk] = e;
      }
      fclose(fp);
    }
  }
  int rc;
  if ((rc = refresh(b))) return rc;
  std::vector<int> used;
  for (int p = 0; p < b->cap; ++p)
    if (b->slots[p].used) used.push_back(p);
  if ((rc = sync_states(b))) return rc;  // the device states are the live ones; restored below
  std::vector<Scal> hs(b->cap);
  for (auto& s : hs) {
    std::memset(&s, 0, sizeof(s));
    s.phase = 0;  // every problem "running" for the timing launches
  }
  SELF_CUDA_TRY(ctx, cudaMemcpy(b->S.p, hs.data(), hs.size() * sizeof(Scal), cudaMemcpyHostToDevice));
  for (int N = 2; N <= 9; ++N)
    for (int bk = 0; bk < 4; ++bk) {
      if (!present[N][bk] || b->epb[N][bk] > 0) continue;
      const int r = max_epb_rt(N);
      int best = default_tile_elems(N);
      double best_ms = 1e30;
      // element tiles of 1, 2, 4, ... 32 node rounds (FP64 body) and 1, 2, 4, 8 line rounds (FP32 body), each a
      // multiple of the node round
      std::vector<int> cand;
      for (int e = r; e <= 32 * r; e *= 2) cand.push_back(e);
      for (int k = 0; k < 4; ++k) cand.push_back(std::max(r, ((line_round_elems_rt(N) << k) / r) * r));
      std::sort(cand.begin(), cand.end());
      cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
      for (int e : cand) {
        if ((rc = upload_view(b, b->tune, used, N, bk, e))) return rc;
        for (int w = 0; w < 2; ++w)
          if ((rc = k_apply_plain<float>(b, b->tune, V_V, V_Z, 0, 0))) return rc;
        double ms = 0;
        if ((rc = self_ctx_timer_start(ctx))) return rc;
        for (int r = 0; r < 10; ++r)
          if ((rc = k_apply_plain<float>(b, b->tune, V_V, V_Z, 0, 0))) return rc;
        if ((rc = self_ctx_timer_stop(ctx, &ms))) return rc;
        if (ms < best_ms) {
          best_ms = ms;
          best = e;
        }
      }
      b->epb[N][bk] = best;
    }
  b->dirty = true;
  if ((rc = refresh(b))) return rc;
  SELF_CUDA_TRY(ctx, cudaMemcpy(b->S.p, b->hs.data(), b->cap * sizeof(Scal), cudaMemcpyHostToDevice));
  if (cache_path) {
    FILE* fp = fopen(cache_path, "w");
    if (fp) {
      fprintf(fp, "[\n");
      bool first = true;
      for (int N = 2; N <= 9; ++N)
        for (int bk = 0; bk < 4; ++bk)
          if (b->epb[N][bk] > 0) {
            fprintf(fp, "%s  { \"N\": %d, \"bucket\": %d, \"epb\": %d }", first ? "" : ",\n", N, bk, b->epb[N][bk]);
            first = false;
          }
      fprintf(fp, "\n]\n");
      fclose(fp);
    }
  }
  return SELF_OK;
}

int self_cgbatch_tuning(self_cgbatch* b, int N, int bucket, int* epb) {
  if (!b || N < 2 || N > 9 || bucket < 0 || bucket > 3 || !epb) return SELF_ERR_INVALID;
  *epb = b->epb[N][bucket] > 0 ? b->epb[N][bucket] : default_tile_elems(N);
  return SELF_OK;
}

}  // extern "C"
