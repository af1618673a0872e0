// CGSEM 2-D matrix-free operator, direct-stiffness summation, masks and Krylov solvers on sm_103a.
//
// Replaces CGsemElliptic_2D's MatrixAction / Residual / DotProduct / Solve (CGsemElliptic_2D_Class.f90
// :617-1207) and the GMRES(m) of IterativeSolvers_Class.f90 :493-652 (as used on element-local vectors
// by Stommel_Class.f90 :1161-1322).
//
// Vectors are element-local "L-vectors" (Fortran u(0:N,0:N,1:nEl)), kept MASKED as in the reference:
// a node shared by several elements holds its value in one primary copy, the other copies are zero, and
// Dirichlet nodes are zero in every Krylov vector.  Shared-node topology is compiled once on the host into
//   src[l]           local index of the primary copy of local node l (UnMask = gather x[src[l]]);
//   groups (CSR)     one group per shared edge node (2 copies, primary first) and per mesh corner node
//                    (its copies in node->element list order), plus single-copy groups for Dirichlet nodes.
//                    GlobalSum followed by Mask = sum the group in list order, write the sum to the primary
//                    copy and zero to the others (Dirichlet groups: zero to all) -- no atomics, the
//                    summation order of the reference.
// The element operator uses per-node factors folded on the host:
//   G11 = k w_i w_j (dydp^2+dxdp^2)/J, G12 = -k w_i w_j (dyds dydp + dxds dxdp)/J, G22 = k w_i w_j (dxds^2+dyds^2)/J,
//   M = lambda J w_i w_j, and for the advection-diffusion operator B1 = w_i w_j (vx dydp - vy dxdp),
//   B2 = w_i w_j (vy dxds - vx dyds):
//   Lu = -( D_s^T (G11 us + G12 up) + D_p^T (G12 us + G22 up) ) - M u - (B1 us + B2 up),  us = D_s u, up = D_p u,
// which is FluxDivergence (:854-926) with CalculateGradient (:791-850) re-associated, plus the mass and
// advection terms of the documented operators.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <limits>
#include <unordered_map>
#include <type_traits>
#include <vector>

#include "cg2d_api.hpp"
#include "internal.hpp"
#include "line_ops.cuh"

using namespace selfgpu;

namespace selfgpu {
namespace cg {

// ---------------------------------------------------------------------------------- element operator
template <int N1, typename R>
struct CGConst {
  R D[N1 * N1];  // collocation derivative matrix, column major
};

template <int N1>
constexpr int cg_epb() {
  return (N1 * N1 >= 256) ? 1 : (256 / (N1 * N1));
}

// out = [alpha*f*Jww] - Lu(x gathered through src), computed per element.  nf = 4 (Helmholtz) or 6 (adv-diff).
template <int N1, typename R, int NF>
__global__ void __launch_bounds__(256) cg_apply_local(const R* __restrict__ x, const int* __restrict__ src,
                                                      const R* __restrict__ fac, const R* __restrict__ rhs,
                                                      R* __restrict__ out, int nEl, CGConst<N1, R> Cg) {
  constexpr int NN = N1 * N1;
  constexpr int EPB = cg_epb<N1>();
  __shared__ R D[N1 * N1];
  __shared__ R su[EPB][NN];
  __shared__ R s1[EPB][NN];
  __shared__ R s2[EPB][NN];
  const int tid = threadIdx.x, le = threadIdx.y;
  const int e = blockIdx.x * EPB + le;
  for (int t = tid + NN * le; t < N1 * N1; t += NN * EPB) D[t] = Cg.D[t];
  const bool active = e < nEl;
  const int i = tid % N1, j = tid / N1;
  const size_t l = (size_t)e * NN + tid;
  R u = 0;
  if (active) {
    u = x[src[l]];
    su[le][tid] = u;
  }
  __syncthreads();
  R us = 0, up = 0, G11 = 0, G12 = 0, G22 = 0, M = 0;
  if (active) {
#pragma unroll
    for (int m = 0; m < N1; ++m) {
      us += D[i + N1 * m] * su[le][m + N1 * j];
      up += D[j + N1 * m] * su[le][i + N1 * m];
    }
    const R* fe = fac + (size_t)e * NF * NN;
    G11 = fe[tid];
    G12 = fe[NN + tid];
    G22 = fe[2 * NN + tid];
    M = fe[3 * NN + tid];
    s1[le][tid] = G11 * us + G12 * up;
    s2[le][tid] = G12 * us + G22 * up;
  }
  __syncthreads();
  if (active) {
    R a = 0, b = 0;
#pragma unroll
    for (int m = 0; m < N1; ++m) {
      a += D[m + N1 * i] * s1[le][m + N1 * j];  // (D^T F1)(i, j)
      b += D[m + N1 * j] * s2[le][i + N1 * m];  // (D^T F2)(i, j)
    }
    R Lu = -(a + b) - M * u;
    if (NF == 6) {
      const R* fe = fac + (size_t)e * NF * NN;
      Lu -= fe[4 * NN + tid] * us + fe[5 * NN + tid] * up;
    }
    out[l] = rhs ? (rhs[l] - Lu) : Lu;
  }
}

// GlobalSum + Mask over the shared-node groups: the two-copy groups as pairs, the others as CSR groups.
constexpr int kDssPairsPerThread = 8;

template <typename R>
__global__ void cg_dss_mask_pairs(R* __restrict__ v, const int2* __restrict__ pairs, int npairs,
                                  const int* __restrict__ gptr, const int* __restrict__ gidx,
                                  const unsigned char* __restrict__ gdir, int ngroups) {
  // the first ceil(npairs / kDssPairsPerThread) threads sum kDssPairsPerThread pairs each (pairs t, t + P, ...;
  // all loads before the stores, so each thread keeps several independent loads in flight); the rest take the
  // CSR groups
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int P = (npairs + kDssPairsPerThread - 1) / kDssPairsPerThread;
  if (t < P) {
    int2 p[kDssPairsPerThread];
    R a[kDssPairsPerThread], b[kDssPairsPerThread];
#pragma unroll
    for (int q = 0; q < kDssPairsPerThread; ++q) {
      const int k = t + q * P;
      if (k < npairs) {
        p[q] = pairs[k];
        a[q] = v[p[q].x];
        b[q] = v[p[q].y];
      }
    }
#pragma unroll
    for (int q = 0; q < kDssPairsPerThread; ++q) {
      if (t + q * P < npairs) {
        R s = 0;
        s += a[q];
        s += b[q];
        v[p[q].x] = s;
        v[p[q].y] = 0;
      }
    }
    return;
  }
  const int g = t - P;
  if (g >= ngroups) return;
  const int a = gptr[g], b = gptr[g + 1];
  if (gdir[g]) {
    for (int k = a; k < b; ++k) v[gidx[k]] = 0;
    return;
  }
  R s = 0;
  for (int k = a; k < b; ++k) s += v[gidx[k]];
  v[gidx[a]] = s;
  for (int k = a + 1; k < b; ++k) v[gidx[k]] = 0;
}

// ---------------------------------------------------------------------------------- reductions
constexpr int kRedThreads = 256;

template <typename T>
__device__ __forceinline__ T block_sum(T v) {
  __shared__ T sh[kRedThreads / 32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, ln = threadIdx.x & 31;
  if (ln == 0) sh[w] = v;
  __syncthreads();
  T r = 0;
  if (w == 0) {
    r = (ln < kRedThreads / 32) ? sh[ln] : T(0);
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  }
  __syncthreads();
  return r;  // valid in thread 0
}

// partial[k * nblk + blockIdx] = sum a_k * b_k (up to 2 dot products in one pass), FP64 accumulation
template <typename R>
__global__ void __launch_bounds__(kRedThreads) dot2_partials(const R* __restrict__ a0, const R* __restrict__ b0,
                                                             const R* __restrict__ a1, const R* __restrict__ b1,
                                                             size_t n, double* __restrict__ partial) {
  double s0 = 0, s1 = 0;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    s0 += (double)a0[k] * (double)b0[k];
    if (a1) s1 += (double)a1[k] * (double)b1[k];
  }
  s0 = block_sum(s0);
  if (threadIdx.x == 0) partial[blockIdx.x] = s0;
  if (a1) {
    s1 = block_sum(s1);
    if (threadIdx.x == 0) partial[gridDim.x + blockIdx.x] = s1;
  }
}

// deterministic final sum of nblk partials per slot, into out[slot]
__global__ void __launch_bounds__(kRedThreads) reduce_partials(const double* __restrict__ partial, int nblk,
                                                               int nslots, double* __restrict__ out) {
  for (int s = 0; s < nslots; ++s) {
    double v = 0;
    for (int k = threadIdx.x; k < nblk; k += blockDim.x) v += partial[(size_t)s * nblk + k];
    v = block_sum(v);
    if (threadIdx.x == 0) out[s] = v;
  }
}

// ---------------------------------------------------------------------------------- CG scalar logic
// Device scalar state of one GMRES cycle.
struct GMScalars {
  double r0, rc, tol;  // r0: ||r0|| of the whole solve (the stop test is relative to it)
  int i, nr, done, breakdown;  // i: steps of the cycle so far; nr: columns in the solve
};

// Device scalar state of one (P)CG solve.
struct CGScalars {
  double num, den, vz, rr, r0, tol;
  int iter, done, ioerr, maxIters;
  int bodies, pad;  // loop-graph bodies run in this solve (the device-side loop's bound and launch count)
  double* resi;         // residual history (resi[iter] = ||r||), or null
  double alpha, beta;   // step lengths of the current iteration, formed once by the last block of the kernel
  float alpha32, beta32;  // before (no per-thread FP64 division); FP32 copies for the FP32 kernels
};

// ---------------------------------------------------------------------------------- fused (P)CG iteration
// One iteration is three launches, captured in a CUDA graph of several iterations:
//   pcg_apply_fused (FP32: _f32, FP64: _eo line forms): v_new = w + beta v_old (beta = num/den, v_new = w on the
//                     first iteration), z = L(v_new) per element (before the direct-stiffness sum), partial sums
//                     of <v_new, z>;
//   cg_dss_mask_pairs: z = Mask(GlobalSum(z)) (pairs of two-copy groups, CSR for the rest; folding the group sums
//                     into the update kernel, one node per thread, measured slower: dependent scattered loads);
//   pcg_update_fused (_vec: 16-byte node groups): a = num/<v,z>, u += a v, r -= a z, w = dinv r, partial sums of
//                     <r,w> and <r,r>, and the end-of-iteration scalar update (den = num, num = <r,w>, ||r||, stop
//                     tests).
// <v, Mask(GlobalSum(Lv))> equals the element-local sum of v(src[l]) * (Lv)_l because v is zero on Dirichlet
// nodes and on non-primary copies.  The grid-wide sums are deterministic: every block writes its partial, and the
// last block to finish (atomic ticket) adds the partials in block order and updates the scalars.

// Sum over a 256-thread block of one value per thread: warp sums in the working precision R, the 8 warp sums in
// FP64 (result in thread 0).  FP32 kernels keep the narrow FP64 pipe out of the per-node work.
template <typename R>
__device__ __forceinline__ double block_sum_mixed(R v) {
  __shared__ double sh[kRedThreads / 32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, ln = threadIdx.x & 31;
  if (ln == 0) sh[w] = (double)v;
  __syncthreads();
  double r = 0;
  if (w == 0) {
    r = (ln < kRedThreads / 32) ? sh[ln] : 0.0;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  }
  __syncthreads();
  return r;
}

// Grid-wide sums of NS per-thread values (1-D blocks of kRedThreads threads): returns true in the last block to
// finish, with the sums (block order, fixed tree order inside each block) in thread 0's tot.
template <int NS, typename R>
__device__ __forceinline__ bool grid_sums_last(const R (&v)[NS], double* __restrict__ partial,
                                               unsigned int* __restrict__ ticket, double (&tot)[NS]) {
  __shared__ bool s_last;
  const int nb = gridDim.x;
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    const double b = block_sum_mixed<R>(v[s]);
    if (threadIdx.x == 0) partial[(size_t)s * nb + blockIdx.x] = b;
  }
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(ticket, 1u) == (unsigned)(nb - 1);
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    double a = 0.0;
    for (int k = threadIdx.x; k < nb; k += blockDim.x) a += __ldcg(&partial[(size_t)s * nb + k]);
    tot[s] = block_sum_mixed<double>(a);
  }
  if (threadIdx.x == 0) *ticket = 0u;
  return true;
}

// Element groups of EPB elements, grid-stride over the groups, P groups per pass (1-D blocks of 256 threads:
// thread t works on node t % NN of element t / NN of each group; threads beyond EPB * NN only join the
// reductions).  With P = 2 (FP32) every thread has two independent chains of loads in flight.
template <int N1, typename R, int NF>
__global__ void __launch_bounds__(kRedThreads) pcg_apply_fused(const R* __restrict__ w, const R* __restrict__ vold,
                                                               R* __restrict__ vnew, const int* __restrict__ src,
                                                               const R* __restrict__ fac, R* __restrict__ z, int nEl,
                                                               CGConst<N1, R> Cg, CGScalars* S,
                                                               double* __restrict__ partial,
                                                               unsigned int* __restrict__ ticket) {
  if (S->done) return;
  constexpr int NN = N1 * N1;
  constexpr int EPB = cg_epb<N1>();
  constexpr int P = sizeof(R) == 4 ? 2 : 1;
  static_assert(EPB * NN <= kRedThreads, "one element group per block pass");
  __shared__ R D[N1 * N1];
  __shared__ R su[P][EPB][NN];
  __shared__ R s1[P][EPB][NN];
  __shared__ R s2[P][EPB][NN];
  const int tid = threadIdx.x % NN, le = threadIdx.x / NN;
  for (int t = threadIdx.x; t < N1 * N1; t += kRedThreads) D[t] = Cg.D[t];
  const bool first = S->iter == 0;
  const R beta = first ? R(0) : (sizeof(R) == 4 ? (R)S->beta32 : (R)S->beta);
  const int i = tid % N1, j = tid / N1;
  const int ngroups = (nEl + EPB - 1) / EPB;
  R pa = 0;
  for (int g0 = blockIdx.x * P; g0 < ngroups; g0 += gridDim.x * P) {
    // every independent load of the P nodes first (index, own w and v, folded factors), then the gathers
    bool active[P];
    size_t l[P];
    int e[P];
    R u[P], G11[P], G12[P], G22[P], M[P], B1[P], B2[P];
#pragma unroll
    for (int q = 0; q < P; ++q) {
      e[q] = (g0 + q) * EPB + le;
      active[q] = le < EPB && g0 + q < ngroups && e[q] < nEl;
      l[q] = (size_t)e[q] * NN + tid;
      u[q] = G11[q] = G12[q] = G22[q] = M[q] = B1[q] = B2[q] = R(0);
    }
    int sl[P];
    R wl[P], vl[P];
#pragma unroll
    for (int q = 0; q < P; ++q) {
      if (!active[q]) continue;
      sl[q] = src[l[q]];
      wl[q] = w[l[q]];
      vl[q] = first ? R(0) : vold[l[q]];
      const R* fe = fac + (size_t)e[q] * NF * NN;
      G11[q] = fe[tid];
      G12[q] = fe[NN + tid];
      G22[q] = fe[2 * NN + tid];
      M[q] = fe[3 * NN + tid];
      if (NF == 6) {
        B1[q] = fe[4 * NN + tid];
        B2[q] = fe[5 * NN + tid];
      }
    }
#pragma unroll
    for (int q = 0; q < P; ++q) {
      if (!active[q]) continue;
      const R ws = w[sl[q]], vs = first ? R(0) : vold[sl[q]];
      u[q] = first ? ws : ws + beta * vs;
      vnew[l[q]] = first ? wl[q] : wl[q] + beta * vl[q];
    }
    __syncthreads();  // D loaded / previous pass done with the scratch arrays
#pragma unroll
    for (int q = 0; q < P; ++q)
      if (active[q]) su[q][le][tid] = u[q];
    __syncthreads();
    R us[P], up[P];
#pragma unroll
    for (int q = 0; q < P; ++q) {
      us[q] = up[q] = R(0);
      if (!active[q]) continue;
#pragma unroll
      for (int m = 0; m < N1; ++m) {
        us[q] += D[i + N1 * m] * su[q][le][m + N1 * j];
        up[q] += D[j + N1 * m] * su[q][le][i + N1 * m];
      }
      s1[q][le][tid] = G11[q] * us[q] + G12[q] * up[q];
      s2[q][le][tid] = G12[q] * us[q] + G22[q] * up[q];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < P; ++q) {
      if (!active[q]) continue;
      R a = 0, b = 0;
#pragma unroll
      for (int m = 0; m < N1; ++m) {
        a += D[m + N1 * i] * s1[q][le][m + N1 * j];
        b += D[m + N1 * j] * s2[q][le][i + N1 * m];
      }
      R Lu = -(a + b) - M[q] * u[q];
      if (NF == 6) Lu -= B1[q] * us[q] + B2[q] * up[q];
      z[l[q]] = Lu;
      pa += u[q] * Lu;
    }
  }
  const R acc[1] = {pa};
  double tot[1];
  if (grid_sums_last<1, R>(acc, partial, ticket, tot) && threadIdx.x == 0) {
    S->vz = tot[0];
    S->alpha = S->num / tot[0];
    S->alpha32 = (float)S->alpha;
  }
}

// FP32 form of pcg_apply_fused, one thread per grid line: thread (e, t) of a block pass holds line t of element e
// (the N1 nodes u(., t)) in registers and forms (line_op_f32)
//   us(., t) = D u(., t)                       row pass, D entries as constant-bank FMA operands;
//   up(c, .) = D u(c, .)                       column pass: the same thread as column c, u(c, .) read back from a
//                                              per-line padded buffer (row stride N1 + 1: bank-conflict free for
//                                              the row-major write and the column read);
//   F1, F2 at its row nodes, (D^T F1)(., t) in registers, (D^T F2)(c, .) in the column pass, both summed into Lu.
// A warp holds whole elements when 32 % N1 == 0, and the transposes then need warp barriers only.  The arithmetic
// is that of pcg_apply_fused in another summation order.
template <int N1>
constexpr int line_epb() {
  return kRedThreads / N1;  // elements per block pass
}

template <int N1, int NF>
__global__ void __launch_bounds__(kRedThreads) pcg_apply_fused_f32(const float* __restrict__ w,
                                                                   const float* __restrict__ vold,
                                                                   float* __restrict__ vnew, const int* __restrict__ src,
                                                                   const float* __restrict__ fac, float* __restrict__ z,
                                                                   int nEl, CGConst<N1, float> Cg, CGScalars* S,
                                                                   double* __restrict__ partial,
                                                                   unsigned int* __restrict__ ticket) {
  if (S->done) return;
  constexpr int NN = N1 * N1;
  constexpr int EPL = line_epb<N1>();
  constexpr int LS = N1 + 1;  // padded line in the transpose buffers
  __shared__ float X[EPL * N1 * LS];
  __shared__ float Y[EPL * N1 * LS];
  const int le = threadIdx.x / N1, t = threadIdx.x - le * N1;  // element in the pass, line index
  const bool first = S->iter == 0;
  const float beta = first ? 0.f : S->beta32;
  const int ngroups = (nEl + EPL - 1) / EPL;
  float pa = 0.f;
  for (int g = blockIdx.x; g < ngroups; g += gridDim.x) {
    const int e = g * EPL + le;
    const bool active = le < EPL && e < nEl;
    const size_t l0 = (size_t)e * NN + (size_t)N1 * t;  // row t: nodes (i, t), i = 0..N1-1
    const float* fe = fac + (size_t)e * NF * NN + (size_t)N1 * t;
    float u[N1], Lu[N1];
    if (active) {
#pragma unroll
      for (int f = 0; f < 4; ++f) prefetch_l2(fe + f * NN);  // the factor lines are read two barriers later
      int sl[N1];
      float wl[N1], vl[N1], vn[N1];
      load_line<N1>(src + l0, sl);
      load_line<N1>(w + l0, wl);
      if (first) {
#pragma unroll
        for (int i = 0; i < N1; ++i) vl[i] = 0.f;
      } else {
        load_line<N1>(vold + l0, vl);
      }
#pragma unroll
      for (int i = 0; i < N1; ++i) {
        vn[i] = first ? wl[i] : wl[i] + beta * vl[i];
        u[i] = sl[i] == (int)(l0 + i) ? vn[i] : (first ? w[sl[i]] : w[sl[i]] + beta * vold[sl[i]]);
      }
      store_line<N1>(vnew + l0, vn);
    }
    auto fl = [&](int f, float (&G)[N1]) { load_line<N1>(fe + f * NN, G); };
    line_op_f32<N1, NF>(Cg.D, fl, active, le < EPL ? le : 0, t, X, Y, u, Lu);
    if (active) {
      store_line<N1>(z + l0, Lu);
#pragma unroll
      for (int i = 0; i < N1; ++i) pa += u[i] * Lu[i];
    }
    line_sync<N1>();  // the next pass reuses X and Y
  }
  const float acc[1] = {pa};
  double tot[1];
  if (grid_sums_last<1, float>(acc, partial, ticket, tot) && threadIdx.x == 0) {
    S->vz = tot[0];
    S->alpha = S->num / tot[0];
    S->alpha32 = (float)S->alpha;
  }
}

// Lu on line t (nodes (i, t), i = 0..N1-1) of element le of a block pass, from u(., t) in registers: the line-
// oriented operator of pcg_apply_fused_f32 in FP64 with even-odd contractions.  Every thread of the block calls it
// (threads without a line pass active = false and only join the barriers); fe = the element's factors + N1 t;
// X, Y = the block's padded transpose buffers (row stride N1 + 1: 64-bit accesses of a half warp fall in distinct
// bank pairs for the row-major writes and the column reads).  On return X and Y are free.
template <int N1, int NF>
__device__ __forceinline__ void line_op_f64(const EOPair<N1>& T, const double* __restrict__ fe, bool active, int le,
                                            int t, double* X, double* Y, const double (&u)[N1], double (&Lu)[N1]) {
  constexpr int NN = N1 * N1, LS = N1 + 1;
  double* Xl = X + (size_t)(le * N1 + t) * LS;
  double* Yl = Y + (size_t)(le * N1 + t) * LS;
  double us[N1], up[N1], a[N1];
  if (active) {
    eo_matvec<N1>(T.D, u, us);  // (D u)(., t)
#pragma unroll
    for (int i = 0; i < N1; ++i) Xl[i] = u[i];
  }
  __syncthreads();
  if (active) {  // column pass: column c = t, up(c, .) = D u(c, .)
    double uc[N1], yc[N1];
#pragma unroll
    for (int m = 0; m < N1; ++m) uc[m] = X[(size_t)(le * N1 + m) * LS + t];
    eo_matvec<N1>(T.D, uc, yc);
#pragma unroll
    for (int j = 0; j < N1; ++j) Y[(size_t)(le * N1 + j) * LS + t] = yc[j];
  }
  __syncthreads();
  if (active) {
    double G11[N1], G12[N1], G22[N1], F1[N1];
    load_line<N1>(fe, G11);
    load_line<N1>(fe + NN, G12);
    load_line<N1>(fe + 2 * NN, G22);
#pragma unroll
    for (int i = 0; i < N1; ++i) {
      up[i] = Yl[i];
      F1[i] = G11[i] * us[i] + G12[i] * up[i];
      Xl[i] = G12[i] * us[i] + G22[i] * up[i];  // F2(i, t)
    }
    eo_matvec<N1>(T.Dt, F1, a);  // (D^T F1)(., t)
  }
  __syncthreads();
  if (active) {  // column pass: (D^T F2)(c, .)
    double fc[N1], yc[N1];
#pragma unroll
    for (int m = 0; m < N1; ++m) fc[m] = X[(size_t)(le * N1 + m) * LS + t];
    eo_matvec<N1>(T.Dt, fc, yc);
#pragma unroll
    for (int j = 0; j < N1; ++j) Y[(size_t)(le * N1 + j) * LS + t] = yc[j];
  }
  __syncthreads();
  if (active) {
    double M[N1];
    load_line<N1>(fe + 3 * NN, M);
#pragma unroll
    for (int i = 0; i < N1; ++i) Lu[i] = -(a[i] + Yl[i]) - M[i] * u[i];
    if constexpr (NF == 6) {
      double B1[N1], B2[N1];
      load_line<N1>(fe + 4 * NN, B1);
      load_line<N1>(fe + 5 * NN, B2);
#pragma unroll
      for (int i = 0; i < N1; ++i) Lu[i] -= B1[i] * us[i] + B2[i] * up[i];
    }
  }
}

template <int N1>
__device__ __forceinline__ void eo_copy_tables(const EOPair<N1>& src, EOPair<N1>& dst) {
  constexpr int NC = sizeof(EOPair<N1>) / sizeof(double);
  const double* s = reinterpret_cast<const double*>(&src);
  double* d = reinterpret_cast<double*>(&dst);
  for (int k = threadIdx.x; k < NC; k += blockDim.x) d[k] = s[k];
}

// FP64 fused PCG apply (pcg_apply_fused's work and outputs) with the even-odd line operator.
template <int N1, int NF>
__global__ void __launch_bounds__(kRedThreads, 2) pcg_apply_fused_eo(const double* __restrict__ w,
                                                                     const double* __restrict__ vold,
                                                                     double* __restrict__ vnew,
                                                                     const int* __restrict__ src,
                                                                     const double* __restrict__ fac,
                                                                     double* __restrict__ z, int nEl, EOPair<N1> Tg,
                                                                     CGScalars* S, double* __restrict__ partial,
                                                                     unsigned int* __restrict__ ticket) {
  if (S->done) return;
  constexpr int NN = N1 * N1;
  constexpr int EPL = line_epb<N1>();
  constexpr int LS = N1 + 1;
  __shared__ EOPair<N1> T;
  __shared__ double X[EPL * N1 * LS];
  __shared__ double Y[EPL * N1 * LS];
  eo_copy_tables<N1>(Tg, T);
  __syncthreads();
  const int le = threadIdx.x / N1, t = threadIdx.x - le * N1;
  const bool first = S->iter == 0;
  const double beta = first ? 0.0 : S->beta;
  const int ngroups = (nEl + EPL - 1) / EPL;
  double pa = 0.0;
  for (int g = blockIdx.x; g < ngroups; g += gridDim.x) {
    const int e = g * EPL + le;
    const bool active = le < EPL && e < nEl;
    const size_t l0 = (size_t)e * NN + (size_t)N1 * t;
    double u[N1], Lu[N1];
    if (active) {
      int sl[N1];
      double wl[N1], vn[N1];
      load_line<N1>(src + l0, sl);
      load_line<N1>(w + l0, wl);
      if (first) {
#pragma unroll
        for (int i = 0; i < N1; ++i) vn[i] = wl[i];
      } else {
        double vl[N1];
        load_line<N1>(vold + l0, vl);
#pragma unroll
        for (int i = 0; i < N1; ++i) vn[i] = wl[i] + beta * vl[i];
      }
#pragma unroll
      for (int i = 0; i < N1; ++i)
        u[i] = sl[i] == (int)(l0 + i) ? vn[i] : (first ? w[sl[i]] : w[sl[i]] + beta * vold[sl[i]]);
      store_line<N1>(vnew + l0, vn);
    }
    line_op_f64<N1, NF>(T, fac + (size_t)(active ? e : 0) * NF * NN + (size_t)N1 * t, active, le, t, X, Y, u, Lu);
    if (active) {
      store_line<N1>(z + l0, Lu);
#pragma unroll
      for (int i = 0; i < N1; ++i) pa += u[i] * Lu[i];
    }
  }
  const double acc[1] = {pa};
  double tot[1];
  if (grid_sums_last<1, double>(acc, partial, ticket, tot) && threadIdx.x == 0) {
    S->vz = tot[0];
    S->alpha = S->num / tot[0];
    S->alpha32 = (float)S->alpha;
  }
}

// FP64 local apply (cg_apply_local's work: out = [rhs] - L(x gathered through src)) with the even-odd line operator.
template <int N1, int NF>
__global__ void __launch_bounds__(kRedThreads, 2) cg_apply_local_eo(const double* __restrict__ x,
                                                                    const int* __restrict__ src,
                                                                    const double* __restrict__ fac,
                                                                    const double* __restrict__ rhs,
                                                                    double* __restrict__ out, int nEl,
                                                                    EOPair<N1> Tg) {
  constexpr int NN = N1 * N1;
  constexpr int EPL = line_epb<N1>();
  constexpr int LS = N1 + 1;
  __shared__ EOPair<N1> T;
  __shared__ double X[EPL * N1 * LS];
  __shared__ double Y[EPL * N1 * LS];
  eo_copy_tables<N1>(Tg, T);
  __syncthreads();
  const int le = threadIdx.x / N1, t = threadIdx.x - le * N1;
  const int e = blockIdx.x * EPL + le;
  const bool active = le < EPL && e < nEl;
  const size_t l0 = (size_t)e * NN + (size_t)N1 * t;
  double u[N1], Lu[N1];
  if (active) {
    int sl[N1];
    load_line<N1>(src + l0, sl);
#pragma unroll
    for (int i = 0; i < N1; ++i) u[i] = x[sl[i]];
  }
  line_op_f64<N1, NF>(T, fac + (size_t)(active ? e : 0) * NF * NN + (size_t)N1 * t, active, le, t, X, Y, u, Lu);
  if (active) {
    if (rhs) {
      double rl[N1];
      load_line<N1>(rhs + l0, rl);
#pragma unroll
      for (int i = 0; i < N1; ++i) Lu[i] = rl[i] - Lu[i];
    }
    store_line<N1>(out + l0, Lu);
  }
}

// End-of-iteration scalar step (one thread): den = num, num = <r, w>, beta, ||r|| and the stop tests.
__device__ __forceinline__ void pcg_end_iteration(CGScalars* S, double rw, double rr) {
  const double rn = sqrt(rr);
  S->den = S->num;
  S->num = rw;
  S->beta = S->num / S->den;
  S->beta32 = (float)S->beta;
  S->iter += 1;
  if (S->resi) S->resi[S->iter] = rn;
  S->rr = rn;
  if (!(rn == rn) || isinf(rn)) {  // non-finite residual
    S->done = 1;
    S->ioerr = -7;
  } else if (rn / S->r0 < S->tol) {
    S->done = 1;
    S->ioerr = 0;
  } else if (S->iter >= S->maxIters) {
    S->done = 1;
    S->ioerr = -1;
  }
}

template <typename R>
__global__ void __launch_bounds__(kRedThreads) pcg_update_fused(R* __restrict__ u, R* __restrict__ r,
                                                                R* __restrict__ w, const R* __restrict__ v,
                                                                const R* __restrict__ z, const R* __restrict__ dinv,
                                                                size_t n, CGScalars* S, double* __restrict__ partial,
                                                                unsigned int* __restrict__ ticket) {
  if (S->done) return;
  const R a = sizeof(R) == 4 ? (R)S->alpha32 : (R)S->alpha;
  R prw = 0, prr = 0;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  constexpr int U = 4;  // four independent nodes per pass: their loads are all in flight together
  for (; k + (U - 1) * stride < n; k += U * stride) {
    R uu[U], vv[U], rr[U], zz[U], dd[U];
#pragma unroll
    for (int q = 0; q < U; ++q) {
      const size_t x = k + q * stride;
      uu[q] = u[x];
      vv[q] = v[x];
      rr[q] = r[x];
      zz[q] = z[x];
      dd[q] = dinv ? dinv[x] : R(1);
    }
#pragma unroll
    for (int q = 0; q < U; ++q) {
      const size_t x = k + q * stride;
      u[x] = uu[q] + a * vv[q];
      const R rk = rr[q] - a * zz[q];
      r[x] = rk;
      const R wk = dinv ? rk * dd[q] : rk;
      if (w) w[x] = wk;
      prw += rk * wk;
      prr += rk * rk;
    }
  }
  for (; k < n; k += stride) {
    u[k] += a * v[k];
    const R rk = r[k] - a * z[k];
    r[k] = rk;
    const R wk = dinv ? rk * dinv[k] : rk;
    if (w) w[k] = wk;
    prw += rk * wk;
    prr += rk * rk;
  }
  const R acc[2] = {prw, prr};
  double tot[2];
  if (grid_sums_last<2, R>(acc, partial, ticket, tot) && threadIdx.x == 0) pcg_end_iteration(S, tot[0], tot[1]);
}

// pcg_update_fused over 16-byte groups of consecutive nodes (float4: 4 FP32 nodes, double2: 2 FP64 nodes; the
// L-vector length is a multiple of the group when (N+1)^2 nEl is, otherwise the scalar kernel runs).
template <typename R, typename V>
__global__ void __launch_bounds__(kRedThreads) pcg_update_fused_vec(V* __restrict__ u, V* __restrict__ r,
                                                                    V* __restrict__ w, const V* __restrict__ v,
                                                                    const V* __restrict__ z,
                                                                    const V* __restrict__ dinv, size_t nv,
                                                                    CGScalars* S, double* __restrict__ partial,
                                                                    unsigned int* __restrict__ ticket) {
  static_assert(sizeof(V) == 16 && sizeof(V) % sizeof(R) == 0, "16-byte groups");
  constexpr int L = sizeof(V) / sizeof(R);
  if (S->done) return;
  const R a = sizeof(R) == 4 ? (R)S->alpha32 : (R)S->alpha;
  R prw = 0, prr = 0;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  constexpr int U = 1;  // groups per thread and pass: 1 measured 3.7 % faster per FP32 PCG iteration than 2, 4
  for (; k < nv; k += U * stride) {
    V uu[U], vv[U], rr[U], zz[U], dd[U];
    bool ok[U];
#pragma unroll
    for (int q = 0; q < U; ++q) {
      const size_t x = k + q * stride;
      ok[q] = x < nv;
      if (!ok[q]) continue;
      uu[q] = u[x];
      vv[q] = v[x];
      rr[q] = r[x];
      zz[q] = z[x];
      if (dinv) dd[q] = dinv[x];
    }
#pragma unroll
    for (int q = 0; q < U; ++q) {
      if (!ok[q]) continue;
      const size_t x = k + q * stride;
      R us[L], vs[L], rs[L], zs[L], ds[L], uo[L], ro[L], wo[L];
      memcpy(us, &uu[q], 16);
      memcpy(vs, &vv[q], 16);
      memcpy(rs, &rr[q], 16);
      memcpy(zs, &zz[q], 16);
      if (dinv) memcpy(ds, &dd[q], 16);
#pragma unroll
      for (int c = 0; c < L; ++c) {
        uo[c] = us[c] + a * vs[c];
        ro[c] = rs[c] - a * zs[c];
        wo[c] = dinv ? ro[c] * ds[c] : ro[c];
        prw += ro[c] * wo[c];
        prr += ro[c] * ro[c];
      }
      V t;
      memcpy(&t, uo, 16);
      u[x] = t;
      memcpy(&t, ro, 16);
      r[x] = t;
      if (w) {
        memcpy(&t, wo, 16);
        w[x] = t;
      }
    }
  }
  const R acc[2] = {prw, prr};
  double tot[2];
  if (grid_sums_last<2, R>(acc, partial, ticket, tot) && threadIdx.x == 0) pcg_end_iteration(S, tot[0], tot[1]);
}

// w = dinv r and num = <r, w> before the first iteration
template <typename R>
__global__ void __launch_bounds__(kRedThreads) pcg_start_fused(const R* __restrict__ r, const R* __restrict__ dinv,
                                                               R* __restrict__ w, size_t n, CGScalars* S,
                                                               double* __restrict__ partial,
                                                               unsigned int* __restrict__ ticket) {
  if (S->done) return;
  R pa = 0;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const R wk = dinv ? r[k] * dinv[k] : r[k];
    w[k] = wk;
    pa += r[k] * wk;
  }
  const R acc[1] = {pa};
  double tot[1];
  if (grid_sums_last<1, R>(acc, partial, ticket, tot) && threadIdx.x == 0) S->num = tot[0];
}

#include "pc_linear.cuh"
#include "tc_apply.cuh"
#include "compact.cuh"

// ---------------------------------------------------------------------------------- generic vector ops
template <typename R>
__global__ void axpby(R* __restrict__ y, const R* __restrict__ x, R a, R b, size_t n) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    y[k] = a * x[k] + b * y[k];
}

template <typename R>
__global__ void scale_copy(R* __restrict__ y, const R* __restrict__ x, const double* __restrict__ s, int inv,
                           size_t n) {
  const double f = inv ? 1.0 / s[0] : s[0];
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    y[k] = (R)(f * (double)x[k]);
}

// MGS step: y -= h * x (h = hk[0]) and out = <x_next, y> (or <y, y> when x_next is null), the grid-wide sum
// closed by the last block (ticket)
template <typename R>
__global__ void __launch_bounds__(kRedThreads) mgs_axpy_dot_fused(R* __restrict__ y, const R* __restrict__ x,
                                                                  const double* __restrict__ hk,
                                                                  const R* __restrict__ xn, size_t n,
                                                                  double* __restrict__ partial,
                                                                  unsigned int* __restrict__ ticket,
                                                                  double* __restrict__ out) {
  const R h = (R)hk[0];
  R s0 = 0;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const R yk = y[k] - h * x[k];
    y[k] = yk;
    s0 += xn ? xn[k] * yk : yk * yk;
  }
  const R acc[1] = {s0};
  double tot[1];
  if (grid_sums_last<1, R>(acc, partial, ticket, tot) && threadIdx.x == 0) out[0] = tot[0];
}

// x += sum_k V_k y_k
// ---------------------------------------------------------------------------------- on-chip modified Gram-Schmidt
// One cooperative launch per Arnoldi step (one block per SM, all resident): each block keeps its chunk of w in
// shared memory for the whole step, so the i + 1 projections stream only the basis vectors (each read twice: the
// dot of projection k and the axpy of projection k, fused with the next dot) instead of w, v_k and v_{k+1} and a
// write of w per projection; the step ends by writing v_{i+1} = w / ||w|| (gmres_next_basis) from shared memory.
// The MGS order is the reference's: h(k) = <v_k, w> with w already reduced by v_0 .. v_{k-1}.  Grid-wide sums are
// deterministic (every block adds the block partials in block order) and every barrier wait is bounded.
constexpr int kMgsThreads = 1024;
constexpr long long kMgsMaxPolls = 1LL << 22;  // polls of the barrier generation word; a round ends within µs

__device__ __forceinline__ double block_sum_mgs(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int wid = threadIdx.x >> 5, ln = threadIdx.x & 31;
  if (ln == 0) sh[wid] = v;
  __syncthreads();
  double r = 0.0;
  if (wid == 0) {
    r = ln < (int)(blockDim.x >> 5) ? sh[ln] : 0.0;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  }
  __syncthreads();
  return r;  // valid in thread 0
}

// Sum of v over the grid into *tot (every thread); false after a barrier time-out (err set, the caller returns).
// part: 2 x gridDim.x partials (alternating rounds), bar: {arrivals, generation}.
__device__ __forceinline__ bool mgs_allreduce(double v, double* __restrict__ part, int round, unsigned int* bar,
                                              int* err, double* sh, double* tot) {
  __shared__ int s_ok;
  const double b = block_sum_mgs(v, sh);
  const unsigned int nb = gridDim.x;
  double* P = part + (size_t)(round & 1) * nb;
  if (threadIdx.x == 0) {
    P[blockIdx.x] = b;
    __threadfence();
    volatile unsigned int* gen = bar + 1;
    const unsigned int g = *gen;  // this round's generation: it moves only after every block arrived
    bool ok = true;
    if (atomicAdd(bar, 1u) == nb - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      long long polls = 0;
      while (*gen == g && ++polls < kMgsMaxPolls) {
      }
      ok = *gen != g;
    }
    __threadfence();
    if (!ok) atomicExch(err, 1);
    s_ok = ok && *((volatile int*)err) == 0;
  }
  __syncthreads();
  if (!s_ok) return false;
  double a = 0.0;
  for (unsigned int k = threadIdx.x; k < nb; k += blockDim.x) a += __ldcg(&P[k]);
  const double t = block_sum_mgs(a, sh);
  if (threadIdx.x == 0) sh[32] = t;
  __syncthreads();
  *tot = sh[32];
  __syncthreads();  // sh is reused by the next sum
  return true;
}

// the stream element of mgs_onchip: 16-byte vectors of FP32 values; FP64 values one by one (measured: double2 made
// the FP64 step 15 % slower, float4 the FP32 step 32 % faster than single values)
template <typename R>
struct MgsVec;
template <>
struct MgsVec<float> {
  using T = float4;
  static constexpr int N = 4;
};
template <>
struct MgsVec<double> {
  using T = double;
  static constexpr int N = 1;
};

// MGS of w against V[0..i] and v_{i+1} = w / ||w||: H[k] = h(k, i) for k <= i, H[i + 1] = ||w||^2.  Block b owns
// nodes [b chunk, (b + 1) chunk) of the L-vectors.
template <typename R>
__global__ void __launch_bounds__(kMgsThreads, 1) mgs_onchip(const R* __restrict__ w, R* __restrict__ V, size_t nl,
                                                            int i, int chunk, double* __restrict__ H,
                                                            double* __restrict__ part, unsigned int* bar, int* err) {
  using VT = typename MgsVec<R>::T;
  constexpr int EV = MgsVec<R>::N;
  extern __shared__ __align__(16) unsigned char mgs_smem[];
  R* ws = reinterpret_cast<R*>(mgs_smem);
  VT* wv = reinterpret_cast<VT*>(mgs_smem);
  __shared__ double sh[33];
  const size_t c0 = (size_t)blockIdx.x * chunk;  // chunk is a multiple of 4: c0 starts a 16-byte vector
  const int n = c0 < nl ? (int)(nl - c0 < (size_t)chunk ? nl - c0 : (size_t)chunk) : 0;
  const int nv = n / EV;  // whole vectors; the tail (the last block only) goes node by node
  // a thread's products are summed in R (FP32 vectors: no per-node FP64 conversions on GB300's narrow FP64 pipe),
  // the block and grid sums in FP64, as in mgs_axpy_dot_fused
  R acc = 0;
  double h = 0.0;
  {
    const VT* wg = reinterpret_cast<const VT*>(w + c0);
    const VT* v0 = reinterpret_cast<const VT*>(V + c0);
#pragma unroll 2
    for (int q = threadIdx.x; q < nv; q += blockDim.x) {
      const VT x = wg[q], a = v0[q];
      wv[q] = x;
      const R* xs = reinterpret_cast<const R*>(&x);
      const R* as = reinterpret_cast<const R*>(&a);
#pragma unroll
      for (int c = 0; c < EV; ++c) acc += as[c] * xs[c];
    }
    for (int q = nv * EV + threadIdx.x; q < n; q += blockDim.x) {
      const R x = w[c0 + q];
      ws[q] = x;
      acc += V[c0 + q] * x;
    }
  }
  if (!mgs_allreduce((double)acc, part, 0, bar, err, sh, &h)) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) H[0] = h;
  for (int k = 0; k <= i; ++k) {
    const R* vk = V + (size_t)k * nl + c0;
    const R* vn = V + (size_t)(k + 1) * nl + c0;
    const VT* vkv = reinterpret_cast<const VT*>(vk);
    const VT* vnv = reinterpret_cast<const VT*>(vn);
    const R hk = (R)h;
    const bool last = k == i;
    acc = 0;
#pragma unroll 2
    for (int q = threadIdx.x; q < nv; q += blockDim.x) {
      VT y = wv[q];
      const VT a = vkv[q];
      VT b = a;
      if (!last) b = vnv[q];
      R* ys = reinterpret_cast<R*>(&y);
      const R* as = reinterpret_cast<const R*>(&a);
      const R* bs = reinterpret_cast<const R*>(&b);
#pragma unroll
      for (int c = 0; c < EV; ++c) {
        ys[c] = ys[c] - hk * as[c];
        acc += last ? ys[c] * ys[c] : bs[c] * ys[c];
      }
      wv[q] = y;
    }
    for (int q = nv * EV + threadIdx.x; q < n; q += blockDim.x) {
      const R y = ws[q] - hk * vk[q];
      ws[q] = y;
      acc += last ? y * y : vn[q] * y;
    }
    if (!mgs_allreduce((double)acc, part, k + 1, bar, err, sh, &h)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) H[k + 1] = h;
  }
  // v_{i+1} = w / ||w||, zero on a lucky breakdown (the rule of gmres_givens / gmres_next_basis)
  const bool zero = fabs(sqrt(h)) <= 2.220446049250313e-16;
  const double f = zero ? 0.0 : 1.0 / sqrt(h);
  R* vo = V + (size_t)(i + 1) * nl + c0;
  for (int q = threadIdx.x; q < n; q += blockDim.x) vo[q] = zero ? (R)0 : (R)(f * (double)ws[q]);
}

template <typename R>
__global__ void gmres_update(R* __restrict__ x, const R* __restrict__ V, const double* __restrict__ y, int nr,
                             size_t n, const R* __restrict__ dinv) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    double s = 0;
    for (int j = 0; j < nr; ++j) s += (double)V[(size_t)j * n + k] * y[j];
    x[k] += dinv ? (R)(s * (double)dinv[k]) : (R)s;
  }
}

// y = x * d elementwise
template <typename R>
__global__ void scale_by(R* __restrict__ y, const R* __restrict__ x, const R* __restrict__ d, size_t n) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    y[k] = x[k] * d[k];
}

template <typename R, typename S>
__global__ void convert(R* __restrict__ y, const S* __restrict__ x, size_t n) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    y[k] = (R)x[k];
}

}  // namespace cg
}  // namespace selfgpu

// ====================================================================================== handle
using namespace selfgpu::cg;

namespace {

template <typename T>
int upload(self_ctx* ctx, DevBuf<T>& b, const std::vector<T>& host) {
  if (b.alloc(host.size()) != cudaSuccess) return set_error(ctx, SELF_ERR_ALLOC, "device allocation failed");
  if (!host.empty())
    SELF_CUDA_TRY(ctx, cudaMemcpy(b.p, host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice));
  return SELF_OK;
}

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

inline int grid_for(const self_ctx* ctx, size_t n) {
  size_t want = (n + kRedThreads - 1) / kRedThreads;
  size_t cap = (size_t)std::max(1, ctx->num_sms) * 8;  // 8 CTAs of 256 threads per SM, grid-stride loops
  return (int)std::max<size_t>(1, std::min(want, cap));
}

}  // namespace

namespace selfgpu {
namespace cg {

// Operator data on the device in precision R.
// Buffers a captured PCG iteration graph was built on.
struct PcgGraphKey {
  const void *u, *r, *v, *v2, *w, *z, *dinv, *fac;
  int tc;         // tensor-core form of the FP32 apply
  int host_loop;  // captured as a plain graph repeated from the host (else a conditional-while loop)
  bool operator==(const PcgGraphKey& o) const {
    return u == o.u && r == o.r && v == o.v && v2 == o.v2 && w == o.w && z == o.z && dinv == o.dinv &&
           fac == o.fac && tc == o.tc && host_loop == o.host_loop;
  }
};

template <typename R>
struct OpData {
  DevBuf<R> fac;   // NF * n^2 per element
  DevBuf<R> rhs_scale;  // J w_i w_j per node (load vector of the residual)
  DevBuf<R> dinv;  // 1 / assembled diagonal (masked positions 1)
  std::vector<R> D;
};

}  // namespace cg
}  // namespace selfgpu

struct self_cg2d {
  self_ctx* ctx = nullptr;
  int N = 0, n = 0, nEl = 0, nEdges = 0, nNodes = 0, op = 0, nf = 4;
  size_t nl = 0;
  double lambda = 0, vx = 0, vy = 0;
  DevBuf<int> src, gptr, gidx;
  DevBuf<unsigned char> gdir;
  int ngroups = 0;
  DevBuf<int2> dss_pairs;                  // two-copy groups (primary, secondary)
  DevBuf<int> dss_gptr, dss_gidx;          // the other groups
  DevBuf<unsigned char> dss_gdir;
  int dss_npairs = 0, dss_nrest = 0;
  std::vector<int> h_src, h_gptr, h_gidx;
  std::vector<unsigned char> h_gdir;
  selfgpu::cg::OpData<double> op64;
  selfgpu::cg::OpData<float> op32;
  bool have32 = false;
  // work vectors (FP64)
  DevBuf<double> u, r, v, w, z, f, t, partial, red, resi;
  DevBuf<selfgpu::cg::CGScalars> S;
  // FP32 work vectors for the inner solves
  DevBuf<float> u32, r32, v32, w32, z32;
  DevBuf<double> gm_V, gm_y;  // GMRES basis (m+1) * nl, y
  DevBuf<float> gm_V32;
  DevBuf<double> gm_H, gm_rho, gm_c, gm_s, gm_bhat;
  DevBuf<double> mgs_part;          // on-chip MGS: 2 x SMs block partials
  DevBuf<unsigned int> mgs_bar;     // {arrivals, generation}
  DevBuf<int> mgs_err;              // barrier time-out flag
  DevBuf<selfgpu::cg::GMScalars> GS;
  std::vector<double> h_J, h_w;
  std::vector<double> h_fac, h_dinv;
  bool affine = false;               // every element affine (see build_factors)
  std::vector<double> h_kw, h_ec;    // then: k w_i w_j per node, (c11, c12, c22, lambda J) per element
  bool upload_dev = true;  // false: compile the host arrays only (used by the batched solver)
  int nblk = 0;
  // fused (P)CG: second direction buffer, block ticket of the grid-wide sums, one captured iteration graph per
  // (precision, preconditioner)
  DevBuf<double> v2;
  DevBuf<float> v2_32;
  DevBuf<unsigned int> ticket;
  cudaGraphExec_t pcg_graph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  selfgpu::cg::PcgGraphKey pcg_key[2][2] = {};
  long long pcg_graph_launches = 0;  // kernels in a captured PCG graph
  int apply_grid = 0;                // blocks of the fused apply (grid-stride over element groups)
  int tc = 0;                        // FP32 apply at N = 7 on the tensor cores (set per solve from the options)
  // FP32 inner PCG on the compact node layout (one value per unknown; built on first use, when the shared-node
  // groups are those of a conforming mesh: see compact_build)
  struct Compact {
    bool tried = false, ok = false;
    int M = 0, nInt = 0, nE2 = 0, nE1 = 0, nC = 0, ng = 0, ngp = 0, nz = 0;
    int fp64 = -1;  // FP64 solves on the layout: 1 when the even-odd FP64 line operator applies (N1 >= 6)
    DevBuf<int4> desc;
    DevBuf<int> coff, cl;
    DevBuf<float> fac;  // the FP32 element factors line-interleaved by pass group (compact.cuh factor_index)
    bool affine = false;  // affine elements: kw (k w_i w_j per node, line-interleaved) and ec per element instead
    DevBuf<float> kw;
    DevBuf<float4> ec;
    template <typename R>
    struct Vecs {  // Krylov vectors, contribution space and captured solve graphs of one precision
      DevBuf<R> dinv, u, r, v, v2, w, zc;
      cudaGraphExec_t graph[2] = {nullptr, nullptr};
      selfgpu::cg::PcgGraphKey key[2] = {};
      long long graph_launches = 0;
    };
    Vecs<float> f32;
    Vecs<double> f64;  // allocated on the first FP64 solve
  } cpt;
  // linear-FEM preconditioner (SELF_SOLVE_PCG_LINEAR): node positions kept from create; the linear mesh's topology,
  // sub-quad factors and work vectors are built on first use
  struct PcLinear {
    std::vector<double> x, y;
    bool built = false;
    int ngroups = 0, nUnique = 0, nDirichlet = 0;
    bool lift = false;  // the linear mesh has Dirichlet nodes the spectral mesh does not
    int nodes_mode = -1;  // SELF_PC_NODES_* the operands were built for
    DevBuf<int> src, gptr, gidx;
    DevBuf<unsigned char> gdir, lprim, dlift;
    DevBuf<int2> dss_pairs;  // the groups in the pair + CSR form of cg_dss_mask_pairs
    DevBuf<int> dss_gptr, dss_gidx;
    DevBuf<unsigned char> dss_gdir;
    int dss_npairs = 0, dss_nrest = 0;
    DevBuf<double> fac64, rl, ul, vl, vl2, zl, rd;
    DevBuf<float> fac32, rl32, ul32, vl32, vl2_32, zl32, rd32;
    DevBuf<selfgpu::cg::CGScalars> SL;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    selfgpu::cg::PcgGraphKey key[2] = {};
    int key_iters[2] = {-1, -1};
    long long graph_launches = 0;
  } pcl;
  ~self_cg2d() {
    for (auto& row : pcg_graph)
      for (auto& g : row)
        if (g) cudaGraphExecDestroy(g);
    for (auto& g : pcl.graph)
      if (g) cudaGraphExecDestroy(g);
    for (auto& g : cpt.f32.graph)
      if (g) cudaGraphExecDestroy(g);
    for (auto& g : cpt.f64.graph)
      if (g) cudaGraphExecDestroy(g);
  }
};

namespace {

// the even-odd tables of D and D^T (FP64), or false when D is not centro-antisymmetric or N1 < 6 (where the
// even-odd form saves no FP64 operation: 16 of 16 per line at N1 = 4, 20 of 25 at N1 = 5, and the node-per-thread
// kernel keeps more warps resident)
template <int N1, typename R>
bool eo_pair(const std::vector<R>& D, EOPair<N1>& T) {
  if constexpr (sizeof(R) != 8 || N1 < 6) {
    return false;
  } else {
    return eo_table<N1>(D.data(), false, T.D) && eo_table<N1>(D.data(), true, T.Dt);
  }
}

template <int N1, typename R, int NF>
void launch_apply_t(self_cg2d* h, const R* x, const R* fac, const R* rhs, R* out, const std::vector<R>& D) {
  if constexpr (sizeof(R) == 8 && N1 >= 6) {
    EOPair<N1> T;
    if (eo_pair<N1>(D, T)) {
      constexpr int EPL = line_epb<N1>();
      cg_apply_local_eo<N1, NF><<<(h->nEl + EPL - 1) / EPL, kRedThreads, 0, h->ctx->stream>>>(x, h->src.p, fac, rhs,
                                                                                             out, h->nEl, T);
      return;
    }
  }
  CGConst<N1, R> C;
  for (int k = 0; k < N1 * N1; ++k) C.D[k] = D[k];
  constexpr int EPB = cg_epb<N1>();
  dim3 blk(N1 * N1, EPB);
  cg_apply_local<N1, R, NF><<<(h->nEl + EPB - 1) / EPB, blk, 0, h->ctx->stream>>>(x, h->src.p, fac, rhs, out,
                                                                                 h->nEl, C);
}

template <typename R>
int launch_apply(self_cg2d* h, const R* x, const R* rhs, R* out, const selfgpu::cg::OpData<R>& od) {
  const R* fac = od.fac.p;
  const bool adv = h->nf == 6;
#define SELF_CG_CASE(NV)                                                       \
  case NV:                                                                     \
    if (adv)                                                                   \
      launch_apply_t<NV, R, 6>(h, x, fac, rhs, out, od.D);                     \
    else                                                                       \
      launch_apply_t<NV, R, 4>(h, x, fac, rhs, out, od.D);                     \
    break;
  switch (h->n) {
    SELF_CG_CASE(3)
    SELF_CG_CASE(4)
    SELF_CG_CASE(5)
    SELF_CG_CASE(6)
    SELF_CG_CASE(7)
    SELF_CG_CASE(8)
    SELF_CG_CASE(9)
    SELF_CG_CASE(10)
    default:
      return set_error(h->ctx, SELF_ERR_UNSUPPORTED, "CG degree %d", h->N);
  }
#undef SELF_CG_CASE
  SELF_LAUNCHED(h->ctx);
  return SELF_OK;
}

template <typename R>
int launch_dss(self_cg2d* h, R* v) {
  if (h->ngroups == 0) return SELF_OK;
  const int nt = (h->dss_npairs + kDssPairsPerThread - 1) / kDssPairsPerThread + h->dss_nrest;
  cg_dss_mask_pairs<R><<<(nt + 255) / 256, 256, 0, h->ctx->stream>>>(v, h->dss_pairs.p, h->dss_npairs,
                                                                     h->dss_gptr.p, h->dss_gidx.p, h->dss_gdir.p,
                                                                     h->dss_nrest);
  SELF_LAUNCHED(h->ctx);
  return SELF_OK;
}

template <int N1, typename R, int NF>
void launch_apply_fused_t(self_cg2d* h, const R* w, const R* vold, R* vnew, const R* fac, R* z,
                          const std::vector<R>& D) {
  CGConst<N1, R> C;
  for (int k = 0; k < N1 * N1; ++k) C.D[k] = D[k];
  EOPair<N1> T;
  const bool eo = eo_pair<N1>(D, T);  // FP64 with a centro-antisymmetric D: the even-odd line kernel
  // one wave of resident blocks (at most apply_grid, for which the partial sums are sized)
  static int resident[3][11][2] = {};  // per kernel, degree and operator: blocks per SM (0 = not queried)
  const int kind = sizeof(R) == 4 ? 0 : (eo ? 2 : 1);
  int& nb = resident[kind][N1][NF == 6];
  if (nb == 0) {
    int q = 0;
    cudaError_t ce;
    if constexpr (sizeof(R) == 4)
      ce = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&q, pcg_apply_fused_f32<N1, NF>, kRedThreads, 0);
    else if constexpr (N1 >= 6)
      ce = eo ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&q, pcg_apply_fused_eo<N1, NF>, kRedThreads, 0)
              : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&q, pcg_apply_fused<N1, R, NF>, kRedThreads, 0);
    else
      ce = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&q, pcg_apply_fused<N1, R, NF>, kRedThreads, 0);
    if (ce != cudaSuccess) q = 4;
    nb = std::max(1, q);
  }
  const int epb = (sizeof(R) == 4 || eo) ? line_epb<N1>() : cg_epb<N1>();
  const int groups = (h->nEl + epb - 1) / epb;
  const int grid = std::max(1, std::min({h->apply_grid, nb * std::max(1, h->ctx->num_sms), groups}));
  if constexpr (sizeof(R) == 4 && N1 == 8) {
    if (h->tc) {  // tensor-core contractions (tcgen05, compensated TF32), 32 elements per tile
      const int smem = (int)sizeof(tc::Smem);
      // set for the current device on every launch (a process may drive several devices; the call is cheap)
      cudaFuncSetAttribute(pcg_apply_tc<NF>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
      // 4 blocks per SM: the shared-memory and register limits, and 4 x 128 TMEM columns fill the SM's 512
      const int q = 4;
      const int tgroups = (h->nEl + tc::kTileElems - 1) / tc::kTileElems;
      const int tgrid = std::max(1, std::min({h->apply_grid, q * std::max(1, h->ctx->num_sms), tgroups}));
      pcg_apply_tc<NF><<<tgrid, kRedThreads, smem, h->ctx->stream>>>(w, vold, vnew, h->src.p, fac, z, h->nEl, C,
                                                                      h->S.p, h->partial.p, h->ticket.p);
      return;
    }
  }
  if constexpr (sizeof(R) == 4) {
    pcg_apply_fused_f32<N1, NF><<<grid, kRedThreads, 0, h->ctx->stream>>>(
        w, vold, vnew, h->src.p, fac, z, h->nEl, C, h->S.p, h->partial.p, h->ticket.p);
  } else if (eo) {
    if constexpr (N1 >= 6)
      pcg_apply_fused_eo<N1, NF><<<grid, kRedThreads, 0, h->ctx->stream>>>(
          w, vold, vnew, h->src.p, fac, z, h->nEl, T, h->S.p, h->partial.p, h->ticket.p);
  } else {
    pcg_apply_fused<N1, R, NF><<<grid, kRedThreads, 0, h->ctx->stream>>>(
        w, vold, vnew, h->src.p, fac, z, h->nEl, C, h->S.p, h->partial.p, h->ticket.p);
  }
}

template <typename R>
int launch_apply_fused(self_cg2d* h, const R* w, const R* vold, R* vnew, R* z, const selfgpu::cg::OpData<R>& od) {
  const R* fac = od.fac.p;
  const bool adv = h->nf == 6;
#define SELF_CG_CASE(NV)                                                   \
  case NV:                                                                 \
    if (adv)                                                               \
      launch_apply_fused_t<NV, R, 6>(h, w, vold, vnew, fac, z, od.D);      \
    else                                                                   \
      launch_apply_fused_t<NV, R, 4>(h, w, vold, vnew, fac, z, od.D);      \
    break;
  switch (h->n) {
    SELF_CG_CASE(3)
    SELF_CG_CASE(4)
    SELF_CG_CASE(5)
    SELF_CG_CASE(6)
    SELF_CG_CASE(7)
    SELF_CG_CASE(8)
    SELF_CG_CASE(9)
    SELF_CG_CASE(10)
    default:
      return set_error(h->ctx, SELF_ERR_UNSUPPORTED, "CG degree %d", h->N);
  }
#undef SELF_CG_CASE
  SELF_LAUNCHED(h->ctx);
  return SELF_OK;
}

// Linear-FEM preconditioner operator: one wave of resident blocks, grid-stride over element groups.
template <int N1, typename R>
void launch_q1_t(self_cg2d* h, const R* w, const R* vold, R* vnew, const int* src, const R* rd, const R* fac, R* z,
                 CGScalars* SL) {
  static int resident[2][11] = {};  // per precision and degree: blocks per SM (0 = not queried)
  int& nb = resident[sizeof(R) == 4][N1];
  if (nb == 0) {
    int q = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&q, q1_apply_fused<N1, R>, kRedThreads, 0) != cudaSuccess) q = 4;
    nb = std::max(1, q);
  }
  const int groups = (h->nEl + cg_epb<N1>() - 1) / cg_epb<N1>();
  const int grid = std::max(1, std::min({h->apply_grid, nb * std::max(1, h->ctx->num_sms), groups}));
  q1_apply_fused<N1, R><<<grid, kRedThreads, 0, h->ctx->stream>>>(w, vold, vnew, src, rd, fac, z, h->nEl, h->S.p,
                                                                 SL, h->partial.p, h->ticket.p);
}

template <typename R>
int launch_q1(self_cg2d* h, const R* w, const R* vold, R* vnew, const int* src, const R* rd, const R* fac, R* z,
              CGScalars* SL) {
  switch (h->n) {
    case 3: launch_q1_t<3, R>(h, w, vold, vnew, src, rd, fac, z, SL); break;
    case 4: launch_q1_t<4, R>(h, w, vold, vnew, src, rd, fac, z, SL); break;
    case 5: launch_q1_t<5, R>(h, w, vold, vnew, src, rd, fac, z, SL); break;
    case 6: launch_q1_t<6, R>(h, w, vold, vnew, src, rd, fac, z, SL); break;
    case 7: launch_q1_t<7, R>(h, w, vold, vnew, src, rd, fac, z, SL); break;
    case 8: launch_q1_t<8, R>(h, w, vold, vnew, src, rd, fac, z, SL); break;
    case 9: launch_q1_t<9, R>(h, w, vold, vnew, src, rd, fac, z, SL); break;
    case 10: launch_q1_t<10, R>(h, w, vold, vnew, src, rd, fac, z, SL); break;
    default:
      return set_error(h->ctx, SELF_ERR_UNSUPPORTED, "CG degree %d", h->N);
  }
  SELF_LAUNCHED(h->ctx);
  return SELF_OK;
}

// Operands of one application of the linear-FEM preconditioner in precision R.
template <typename R>
struct PcRun {
  const R* fac;
  const int *src, *gptr, *gidx;  // the linear mesh's primary-copy gather and groups
  const unsigned char *gdir, *lprim, *dlift;
  int ngroups, iters;
  const int2* pairs;  // the groups in the pair + CSR form
  const int *pgptr, *pgidx;
  const unsigned char* pgdir;
  int npairs, nrest;
  R *rl, *ul, *vl, *vl2, *zl, *rd;  // rd: Dirichlet lift, null when the linear mesh needs none
  CGScalars* SL;
};

// preconditioner%Solve on the device: u_l from r (spectral masked L-vector), `iters` inner CG iterations at most
template <typename R>
int pc_linear_apply(self_cg2d* h, const R* r, const PcRun<R>& pc) {
  cudaStream_t st = h->ctx->stream;
  pcl_start<R><<<h->nblk, kRedThreads, 0, st>>>(r, h->src.p, pc.lprim, pc.dlift, pc.rl, pc.ul, pc.rd, h->nl, h->S.p,
                                                pc.SL, h->partial.p, h->ticket.p);
  SELF_LAUNCHED(h->ctx);
  for (int it = 0; it < pc.iters; ++it) {
    R* lo = (it % 2 == 0) ? pc.vl : pc.vl2;
    R* ln = (it % 2 == 0) ? pc.vl2 : pc.vl;
    int rc = launch_q1<R>(h, pc.rl, lo, ln, pc.src, pc.rd, pc.fac, pc.zl, pc.SL);
    if (rc) return rc;
    if (pc.ngroups > 0) {
      const int nt = (pc.npairs + kDssPairsPerThread - 1) / kDssPairsPerThread + pc.nrest;
      cg_dss_mask_pairs<R><<<(nt + 255) / 256, 256, 0, st>>>(pc.zl, pc.pairs, pc.npairs, pc.pgptr, pc.pgidx,
                                                             pc.pgdir, pc.nrest);
      SELF_LAUNCHED(h->ctx);
    }
    using V = typename std::conditional<sizeof(R) == 4, float4, double2>::type;
    constexpr int L = sizeof(V) / sizeof(R);
    // FP32 only: the double2 form measured 39.6 against 36.8 us per launch for the scalar FP64 kernel
    if (sizeof(R) == 4 && h->nl % L == 0 && aligned16(pc.ul) && aligned16(pc.rl) && aligned16(ln) &&
        aligned16(pc.zl)) {
      pcl_update_vec<R, V><<<h->nblk, kRedThreads, 0, st>>>(
          reinterpret_cast<V*>(pc.ul), reinterpret_cast<V*>(pc.rl), reinterpret_cast<const V*>(ln),
          reinterpret_cast<const V*>(pc.zl), h->nl / L, h->S.p, pc.SL, h->partial.p, h->ticket.p);
    } else {
      pcl_update<R><<<h->nblk, kRedThreads, 0, st>>>(pc.ul, pc.rl, ln, pc.zl, h->nl, h->S.p, pc.SL, h->partial.p,
                                                     h->ticket.p);
    }
    SELF_LAUNCHED(h->ctx);
  }
  return SELF_OK;
}

// MatrixAction: out = Mask(GlobalSum(L(UnMask(x))))
template <typename R>
int matrix_action(self_cg2d* h, const R* x, R* out, const selfgpu::cg::OpData<R>& od) {
  int rc = launch_apply<R>(h, x, nullptr, out, od);
  if (rc) return rc;
  return launch_dss<R>(h, out);
}

// red[0..slots) = dot products (FP64 accumulation)
template <typename R>
int dots(self_cg2d* h, const R* a0, const R* b0, const R* a1, const R* b1, double* red) {
  cudaStream_t st = h->ctx->stream;
  dot2_partials<R><<<h->nblk, kRedThreads, 0, st>>>(a0, b0, a1, b1, h->nl, h->partial.p);
  SELF_LAUNCHED(h->ctx);
  reduce_partials<<<1, kRedThreads, 0, st>>>(h->partial.p, h->nblk, a1 ? 2 : 1, red);
  SELF_LAUNCHED(h->ctx);
  return SELF_OK;
}

int read_scalar(self_cg2d* h, const double* dptr, double* out) {
  SELF_CUDA_TRY(h->ctx, cudaMemcpyAsync(out, dptr, sizeof(double), cudaMemcpyDeviceToHost, h->ctx->stream));
  SELF_CUDA_TRY(h->ctx, cudaStreamSynchronize(h->ctx->stream));
  return SELF_OK;
}

template <typename R>
int residual(self_cg2d* h, const R* f, const R* sol, R* r, const selfgpu::cg::OpData<R>& od) {
  int rc = launch_apply<R>(h, sol, f, r, od);  // r = f*Jww - L(unmask(sol))
  if (rc) return rc;
  return launch_dss<R>(h, r);
}

}  // namespace

namespace selfgpu {
namespace cg {


// (P)CG iterations on the device from the current residual; returns ioerr and fills iters/resi.
// abs_stop: the reference's early return when ||r0|| < TOL (CGsemElliptic_2D_Class.f90:1160-1162); the inner
// solves of the iterative refinement use a purely relative stop.
// The whole solve is one launch of a graph whose conditional while node repeats a body of kGraphIters fused
// iterations (three launches each, two on the compact layout; the direction buffers alternate) until the device
// scalars report the stop; the host reads the scalar block once, after the solve.
constexpr int kGraphIters = 16;  // even: the current direction is back in `v` after every body


// With pc (linear-FEM preconditioner) every outer iteration starts with the inner solve u_l = M^-1 r and
// w, num = <r, w> (pc_num); the graph then holds kGraphItersPC outer iterations of 3 * pc->iters + 5 launches.
constexpr int kGraphItersPC = 2;

// Last kernel of a loop-graph body: repeat the body while the solve runs, at most maxIters / per_graph + 2 bodies.
__global__ void pcg_loop_cond(CGScalars* S, cudaGraphConditionalHandle cond, int per_graph) {
  const int b = ++S->bodies;
  cudaGraphSetConditional(cond, (!S->done && b < S->maxIters / per_graph + 2) ? 1u : 0u);
}

// The whole (P)CG solve as one graph: a conditional while node whose body is per_graph iterations, enqueued by
// body(k), and pcg_loop_cond; the device decides when to stop (no host round trip between iterations).
// glaunches = the kernels of one body (taken back out of the context's launch counter: replay_until_done counts
// them per body run).
template <class Body>
int capture_iterations(self_cg2d* h, cudaGraphExec_t& G, long long& glaunches, int per_graph, Body body) {
  self_ctx* ctx = h->ctx;
  cudaStream_t st = ctx->stream;
  if (ctx->host_loop) {  // a plain graph of per_graph iterations, repeated from the host by replay_until_done
    cudaGraph_t g;
    int rc = SELF_OK;
    const long long l0 = ctx->launches.load();
    SELF_CUDA_TRY(ctx, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < per_graph && !rc; ++k) rc = body(k);
    cudaError_t ce = cudaStreamEndCapture(st, &g);
    glaunches = ctx->launches.load() - l0;
    ctx->launches.fetch_sub(glaunches);
    if (ce == cudaSuccess && rc) cudaGraphDestroy(g);
    if (rc) return rc;
    if (ce != cudaSuccess) return set_error(ctx, SELF_ERR_CUDA, "PCG graph capture: %s", cudaGetErrorString(ce));
    ce = cudaGraphInstantiate(&G, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return set_error(ctx, SELF_ERR_CUDA, "PCG graph instantiate: %s", cudaGetErrorString(ce));
    return SELF_OK;
  }
  cudaGraph_t g = nullptr;
  SELF_CUDA_TRY(ctx, cudaGraphCreate(&g, 0));
  cudaGraphConditionalHandle cond;
  cudaError_t ce = cudaGraphConditionalHandleCreate(&cond, g, 1u, cudaGraphCondAssignDefault);
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = cond;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  if (ce == cudaSuccess) ce = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np);
  if (ce != cudaSuccess) {
    cudaGraphDestroy(g);
    return set_error(ctx, SELF_ERR_CUDA, "PCG loop graph: %s", cudaGetErrorString(ce));
  }
  cudaGraph_t bodyg = np.conditional.phGraph_out[0];
  const long long l0 = ctx->launches.load();
  ce = cudaStreamBeginCaptureToGraph(st, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
  if (ce != cudaSuccess) {
    cudaGraphDestroy(g);
    return set_error(ctx, SELF_ERR_CUDA, "PCG loop body capture: %s", cudaGetErrorString(ce));
  }
  int rc = SELF_OK;
  for (int k = 0; k < per_graph && !rc; ++k) rc = body(k);
  if (!rc) {
    pcg_loop_cond<<<1, 1, 0, st>>>(h->S.p, cond, per_graph);
    ctx->launches.fetch_add(1);
  }
  const cudaError_t le = rc ? cudaSuccess : cudaGetLastError();
  ce = cudaStreamEndCapture(st, &bodyg);
  glaunches = ctx->launches.load() - l0;
  ctx->launches.fetch_sub(glaunches);
  if (rc || le != cudaSuccess || ce != cudaSuccess) {
    cudaGraphDestroy(g);
    if (rc) return rc;
    return set_error(ctx, SELF_ERR_CUDA, "PCG loop body capture: %s",
                     cudaGetErrorString(le != cudaSuccess ? le : ce));
  }
  ce = cudaGraphInstantiate(&G, g, 0);
  cudaGraphDestroy(g);
  if (ce != cudaSuccess) return set_error(ctx, SELF_ERR_CUDA, "PCG graph instantiate: %s", cudaGetErrorString(ce));
  return SELF_OK;
}

// One launch of the loop graph G runs the solve to its stop; hs holds the scalars afterwards.  Host-looped form
// (self_ctx_host_loop): G repeated, one synchronisation per launch, at most maxIters / per_graph + 2 launches.
int replay_until_done(self_cg2d* h, cudaGraphExec_t G, long long glaunches, CGScalars& hs, int per_graph = 1) {
  self_ctx* ctx = h->ctx;
  cudaStream_t st = ctx->stream;
  if (ctx->host_loop) {
    const long long max_launches = (long long)hs.maxIters / per_graph + 2;
    for (long long gl = 0; gl < max_launches; ++gl) {
      SELF_CUDA_TRY(ctx, cudaGraphLaunch(G, st));
      ctx->launches.fetch_add(glaunches);
      SELF_CUDA_TRY(ctx, cudaMemcpyAsync(&hs, h->S.p, sizeof(hs), cudaMemcpyDeviceToHost, st));
      SELF_CUDA_TRY(ctx, cudaStreamSynchronize(st));
      if (hs.done) break;
    }
    return SELF_OK;
  }
  SELF_CUDA_TRY(ctx, cudaGraphLaunch(G, st));
  SELF_CUDA_TRY(ctx, cudaMemcpyAsync(&hs, h->S.p, sizeof(hs), cudaMemcpyDeviceToHost, st));
  SELF_CUDA_TRY(ctx, cudaStreamSynchronize(st));
  ctx->launches.fetch_add((long long)hs.bodies * glaunches);
  return SELF_OK;
}

template <typename R>
int pcg_device(self_cg2d* h, R* u, R* r, R* v, R* w, R* z, const R* dinv, int maxIters, double tol, double r0,
               double* resi_dev, int* iters, double* rel, const OpData<R>& od, bool abs_stop = true,
               const PcRun<R>* pc = nullptr) {
  self_ctx* ctx = h->ctx;
  cudaStream_t st = ctx->stream;
  R* v2 = (sizeof(R) == 4) ? reinterpret_cast<R*>(h->v2_32.p) : reinterpret_cast<R*>(h->v2.p);
  if (!v2) return set_error(ctx, SELF_ERR_INVALID, "PCG direction buffer missing");
  CGScalars hs{};
  hs.r0 = r0;
  hs.tol = tol;
  hs.maxIters = maxIters;
  hs.iter = 0;
  hs.done = (abs_stop && r0 < tol) || maxIters <= 0 || r0 == 0.0;
  hs.ioerr = hs.done ? 0 : -2;
  hs.resi = resi_dev;
  SELF_CUDA_TRY(ctx, cudaMemcpyAsync(h->S.p, &hs, sizeof(hs), cudaMemcpyHostToDevice, st));
  // a solve that stopped on a device time-out may have left blocks outside the grid sum: start from a clean ticket
  SELF_CUDA_TRY(ctx, cudaMemsetAsync(h->ticket.p, 0, sizeof(unsigned int), st));
  if (!hs.done) {
    if (!pc) {
      pcg_start_fused<R><<<h->nblk, kRedThreads, 0, st>>>(r, dinv, w, h->nl, h->S.p, h->partial.p, h->ticket.p);
      SELF_LAUNCHED(ctx);
    }
    const int prec = sizeof(R) == 4 ? 1 : 0;
    PcgGraphKey key{u, r, v, v2, w, z, dinv, od.fac.p, h->tc, ctx->host_loop};
    if (pc) key = PcgGraphKey{u, r, v, v2, w, z, pc->ul, pc->fac, h->tc, ctx->host_loop};
    cudaGraphExec_t& G = pc ? h->pcl.graph[prec] : h->pcg_graph[prec][dinv ? 1 : 0];
    PcgGraphKey& gk = pc ? h->pcl.key[prec] : h->pcg_key[prec][dinv ? 1 : 0];
    long long& glaunches = pc ? h->pcl.graph_launches : h->pcg_graph_launches;
    const int per_graph = pc ? kGraphItersPC : kGraphIters;
    if (G && (!(gk == key) || (pc && h->pcl.key_iters[prec] != pc->iters))) {
      cudaGraphExecDestroy(G);
      G = nullptr;
    }
    if (!G) {
      const int rc = capture_iterations(h, G, glaunches, per_graph, [&](int k) -> int {
        int rc = SELF_OK;
        R* vold = (k % 2 == 0) ? v : v2;
        R* vnew = (k % 2 == 0) ? v2 : v;
        if (pc) {
          rc = pc_linear_apply<R>(h, r, *pc);
          if (!rc) {
            pc_num<R><<<h->nblk, kRedThreads, 0, st>>>(r, pc->ul, h->src.p, pc->src, w, h->nl, h->S.p,
                                                       h->partial.p, h->ticket.p);
            SELF_LAUNCHED(ctx);
          }
        }
        if (!rc) rc = launch_apply_fused<R>(h, w, vold, vnew, z, od);
        if (!rc) rc = launch_dss<R>(h, z);
        if (!rc) {
          R* wo = pc ? nullptr : w;
          const R* di = pc ? nullptr : dinv;
          using V = typename std::conditional<sizeof(R) == 4, float4, double2>::type;
          constexpr int L = sizeof(V) / sizeof(R);
          if (h->nl % L == 0 && aligned16(u) && aligned16(r) && aligned16(w) && aligned16(vnew) && aligned16(z) &&
              aligned16(dinv)) {
            pcg_update_fused_vec<R, V><<<h->nblk, kRedThreads, 0, st>>>(
                reinterpret_cast<V*>(u), reinterpret_cast<V*>(r), reinterpret_cast<V*>(wo),
                reinterpret_cast<const V*>(vnew), reinterpret_cast<const V*>(z), reinterpret_cast<const V*>(di),
                h->nl / L, h->S.p, h->partial.p, h->ticket.p);
          } else {
            pcg_update_fused<R><<<h->nblk, kRedThreads, 0, st>>>(u, r, wo, vnew, z, di, h->nl, h->S.p, h->partial.p,
                                                                h->ticket.p);
          }
          SELF_LAUNCHED(ctx);
        }
        return rc;
      });
      if (rc) return rc;
      gk = key;
      if (pc) h->pcl.key_iters[prec] = pc->iters;
    }
    if (const int rc = replay_until_done(h, G, glaunches, hs, per_graph)) return rc;
  }
  SELF_CUDA_TRY(ctx, cudaMemcpyAsync(&hs, h->S.p, sizeof(hs), cudaMemcpyDeviceToHost, st));
  SELF_CUDA_TRY(ctx, cudaStreamSynchronize(st));
  *iters = hs.iter;
  *rel = hs.iter > 0 ? hs.rr / r0 : 0.0;
  if (!hs.done) hs.ioerr = -1;
  return hs.ioerr;
}

// (P)CG on the compact layout (r holds the right-hand side, u the zero initial guess): two launches per iteration
// (pcg_apply_compact_f32 / _f64, pcg_update_compact), the solve one launch of a loop graph.
template <int N1>
CompactView compact_view(self_cg2d* h) {
  auto& Cp = h->cpt;
  return CompactView{Cp.desc.p, Cp.coff.p, Cp.nInt, Cp.nE2, Cp.nE1, Cp.nC, Cp.ngp, h->nEl};
}

inline self_cg2d::Compact::Vecs<float>& cvecs(self_cg2d* h, const float*) { return h->cpt.f32; }
inline self_cg2d::Compact::Vecs<double>& cvecs(self_cg2d* h, const double*) { return h->cpt.f64; }

template <int N1, int NF>
int launch_compact_apply_t(self_cg2d* h, const float* w, const float* vold, float* vnew) {
  CGConst<N1, float> Cg;
  for (int k = 0; k < N1 * N1; ++k) Cg.D[k] = h->op32.D[k];
  const bool aff = NF == 4 && h->cpt.affine;
  static int resident[11][3] = {};
  int& nb = resident[N1][aff ? 2 : (NF == 6)];
  if (nb == 0) {
    int q = 0;
    const cudaError_t ce = aff ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                                     &q, pcg_apply_compact_f32<N1, NF, NF == 4>, kRedThreads, 0)
                               : cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                                     &q, pcg_apply_compact_f32<N1, NF, false>, kRedThreads, 0);
    nb = std::max(1, ce == cudaSuccess ? q : 3);
  }
  const int groups = (h->nEl + line_epb<N1>() - 1) / line_epb<N1>();
  const int grid = std::max(1, std::min({h->apply_grid, nb * std::max(1, h->ctx->num_sms), groups}));
  AffineOp<N1> A{h->cpt.kw.p, h->cpt.ec.p, {}};
  for (int j = 0; j < N1; ++j)
    for (int i = 0; i < N1; ++i) A.ww[i + N1 * j] = (float)(h->h_w[i] * h->h_w[j]);
  float* zc = h->cpt.f32.zc.p;
  if (aff)
    pcg_apply_compact_f32<N1, NF, NF == 4><<<grid, kRedThreads, 0, h->ctx->stream>>>(
        w, vold, vnew, compact_view<N1>(h), h->cpt.fac.p, A, zc, Cg, h->S.p, h->partial.p, h->ticket.p);
  else
    pcg_apply_compact_f32<N1, NF, false><<<grid, kRedThreads, 0, h->ctx->stream>>>(
        w, vold, vnew, compact_view<N1>(h), h->cpt.fac.p, A, zc, Cg, h->S.p, h->partial.p, h->ticket.p);
  SELF_LAUNCHED(h->ctx);
  return SELF_OK;
}

template <int N1, int NF>
int launch_compact_apply_t(self_cg2d* h, const double* w, const double* vold, double* vnew) {
  if constexpr (N1 >= 6) {
    EOPair<N1> T;
    if (!eo_pair<N1>(h->op64.D, T)) return set_error(h->ctx, SELF_ERR_UNSUPPORTED, "FP64 compact apply: no even-odd D");
    static int resident[11][2] = {};
    int& nb = resident[N1][NF == 6];
    if (nb == 0) {
      int q = 0;
      const cudaError_t ce =
          cudaOccupancyMaxActiveBlocksPerMultiprocessor(&q, pcg_apply_compact_f64<N1, NF>, kRedThreads, 0);
      nb = std::max(1, ce == cudaSuccess ? q : 2);
    }
    const int groups = (h->nEl + line_epb<N1>() - 1) / line_epb<N1>();
    const int grid = std::max(1, std::min({h->apply_grid, nb * std::max(1, h->ctx->num_sms), groups}));
    pcg_apply_compact_f64<N1, NF><<<grid, kRedThreads, 0, h->ctx->stream>>>(
        w, vold, vnew, compact_view<N1>(h), h->op64.fac.p, h->cpt.f64.zc.p, T, h->S.p, h->partial.p, h->ticket.p);
    SELF_LAUNCHED(h->ctx);
    return SELF_OK;
  } else {
    return set_error(h->ctx, SELF_ERR_UNSUPPORTED, "FP64 compact apply: degree %d", N1 - 1);
  }
}

template <int N1, typename R>
int launch_compact_update_t(self_cg2d* h, const R* vnew, bool jac) {
  auto& Cp = h->cpt;
  auto& Vc = cvecs(h, vnew);
  static int nbu[11] = {};  // resident blocks per SM: one full wave, grid-stride over the node groups
  if (nbu[N1] == 0) {
    int q = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&q, pcg_update_compact<N1, R>, kRedThreads, 0) !=
        cudaSuccess)
      q = 4;
    nbu[N1] = std::max(1, q);
  }
  const int groups = (Cp.ngp / 4 + kRedThreads - 1) / kRedThreads;
  const int grid = std::max(1, std::min({h->nblk, nbu[N1] * std::max(1, h->ctx->num_sms), groups}));
  pcg_update_compact<N1, R><<<grid, kRedThreads, 0, h->ctx->stream>>>(
      Vc.u.p, Vc.r.p, Vc.w.p, vnew, Vc.zc.p, jac ? Vc.dinv.p : nullptr, compact_view<N1>(h), h->S.p, h->partial.p,
      h->ticket.p);
  SELF_LAUNCHED(h->ctx);
  return SELF_OK;
}

template <int N1>
int launch_compact_assemble_t(self_cg2d* h, double* out) {
  auto& Cp = h->cpt;
  compact_assemble<N1, float><<<h->nblk, kRedThreads, 0, h->ctx->stream>>>(out, Cp.f32.zc.p, Cp.cl.p, Cp.ng,
                                                                          compact_view<N1>(h));
  SELF_LAUNCHED(h->ctx);
  return SELF_OK;
}

// the compact kernels by degree: apply (op = 0), update (1), assemble the FP32 output into a masked FP64 L-vector (2)
template <typename R>
int compact_dispatch(self_cg2d* h, int op, const R* w, const R* vold, R* vnew, bool jac, double* out) {
  const bool adv = h->nf == 6;
#define SELF_CG_CASE(NV)                                                                                 \
  case NV:                                                                                               \
    if (op == 0)                                                                                         \
      return adv ? launch_compact_apply_t<NV, 6>(h, w, vold, vnew) : launch_compact_apply_t<NV, 4>(h, w, vold, vnew); \
    if (op == 1) return launch_compact_update_t<NV, R>(h, vnew, jac);                                   \
    return launch_compact_assemble_t<NV>(h, out);
  switch (h->n) {
    SELF_CG_CASE(3)
    SELF_CG_CASE(4)
    SELF_CG_CASE(5)
    SELF_CG_CASE(6)
    SELF_CG_CASE(7)
    SELF_CG_CASE(8)
    SELF_CG_CASE(9)
    SELF_CG_CASE(10)
    default:
      return set_error(h->ctx, SELF_ERR_UNSUPPORTED, "CG degree %d", h->N);
  }
#undef SELF_CG_CASE
}

int launch_compact_apply(self_cg2d* h, const float* w, const float* vold, float* vnew) {
  return compact_dispatch<float>(h, 0, w, vold, vnew, false, nullptr);
}
int launch_compact_assemble(self_cg2d* h, double* out) {
  return compact_dispatch<float>(h, 2, nullptr, nullptr, nullptr, false, out);
}
// one PCG iteration on the compact layout: apply, then update
template <typename R>
int launch_compact(self_cg2d* h, const R* w, const R* vold, R* vnew, bool jac) {
  int rc = compact_dispatch<R>(h, 0, w, vold, vnew, jac, nullptr);
  return rc ? rc : compact_dispatch<R>(h, 1, w, vold, vnew, jac, nullptr);
}

// The FP64 vectors of the compact layout (first FP64 solve), with the Jacobi diagonal gathered from the FP64
// element-local one.  False when the FP64 compact apply does not apply (no even-odd line operator: N < 5).
int compact_fp64_ready(self_cg2d* h, bool* ready) {
  auto& Cp = h->cpt;
  *ready = false;
  if (!Cp.ok) return SELF_OK;
  if (Cp.fp64 < 0) {
    bool eo = false;
    switch (h->n) {
      case 6: { EOPair<6> T; eo = eo_pair<6>(h->op64.D, T); break; }
      case 7: { EOPair<7> T; eo = eo_pair<7>(h->op64.D, T); break; }
      case 8: { EOPair<8> T; eo = eo_pair<8>(h->op64.D, T); break; }
      case 9: { EOPair<9> T; eo = eo_pair<9>(h->op64.D, T); break; }
      case 10: { EOPair<10> T; eo = eo_pair<10>(h->op64.D, T); break; }
      default: break;
    }
    Cp.fp64 = eo ? 1 : 0;
  }
  if (!Cp.fp64) return SELF_OK;
  auto& V = Cp.f64;
  self_ctx* ctx = h->ctx;
  if (!V.u.p) {
    const size_t ngp = Cp.ngp;
    for (DevBuf<double>* b : {&V.dinv, &V.u, &V.r, &V.v, &V.v2, &V.w}) {
      if (b->alloc(ngp) != cudaSuccess) return set_error(ctx, SELF_ERR_ALLOC, "device allocation of %zu doubles", ngp);
      SELF_CUDA_TRY(ctx, cudaMemsetAsync(b->p, 0, ngp * sizeof(double), ctx->stream));
    }
    if (V.zc.alloc(Cp.nz) != cudaSuccess)
      return set_error(ctx, SELF_ERR_ALLOC, "device allocation of %d doubles", Cp.nz);
    compact_gather<double><<<h->nblk, kRedThreads, 0, ctx->stream>>>(V.dinv.p, h->op64.dinv.p, Cp.cl.p, Cp.ng, Cp.ngp);
    SELF_LAUNCHED(ctx);
  }
  *ready = true;
  return SELF_OK;
}

template <typename R>
int pcg_device_compact(self_cg2d* h, bool jac, int maxIters, double tol, double r0, double* resi_dev, bool abs_stop,
                       int* iters, double* rel) {
  self_ctx* ctx = h->ctx;
  cudaStream_t st = ctx->stream;
  auto& Cp = h->cpt;
  auto& Vc = cvecs(h, (const R*)nullptr);
  CGScalars hs{};
  hs.r0 = r0;
  hs.tol = tol;
  hs.maxIters = maxIters;
  hs.done = (abs_stop && r0 < tol) || maxIters <= 0 || r0 == 0.0;
  hs.ioerr = hs.done ? 0 : -2;
  hs.resi = resi_dev;
  SELF_CUDA_TRY(ctx, cudaMemcpyAsync(h->S.p, &hs, sizeof(hs), cudaMemcpyHostToDevice, st));
  SELF_CUDA_TRY(ctx, cudaMemsetAsync(h->ticket.p, 0, sizeof(unsigned int), st));
  if (!hs.done) {
    const R* dinv = jac ? Vc.dinv.p : nullptr;
    pcg_start_fused<R><<<h->nblk, kRedThreads, 0, st>>>(Vc.r.p, dinv, Vc.w.p, Cp.ngp, h->S.p, h->partial.p,
                                                        h->ticket.p);
    SELF_LAUNCHED(ctx);
    cudaGraphExec_t& G = Vc.graph[jac ? 1 : 0];
    const PcgGraphKey key{Vc.u.p, Vc.r.p, Vc.v.p, Vc.v2.p, Vc.w.p, Vc.zc.p, dinv, nullptr, 0, ctx->host_loop};
    if (G && !(Vc.key[jac ? 1 : 0] == key)) {
      cudaGraphExecDestroy(G);
      G = nullptr;
    }
    if (!G) {
      const int rc = capture_iterations(h, G, Vc.graph_launches, kGraphIters, [&](int k) {
        return launch_compact<R>(h, Vc.w.p, k % 2 == 0 ? Vc.v.p : Vc.v2.p, k % 2 == 0 ? Vc.v2.p : Vc.v.p, jac);
      });
      if (rc) return rc;
      Vc.key[jac ? 1 : 0] = key;
    }
    if (const int rc = replay_until_done(h, G, Vc.graph_launches, hs, kGraphIters)) return rc;
  }
  SELF_CUDA_TRY(ctx, cudaMemcpyAsync(&hs, h->S.p, sizeof(hs), cudaMemcpyDeviceToHost, st));
  SELF_CUDA_TRY(ctx, cudaStreamSynchronize(st));
  *iters = hs.iter;
  *rel = hs.iter > 0 ? hs.rr / r0 : 0.0;
  if (!hs.done) hs.ioerr = -1;
  return hs.ioerr;
}

}  // namespace cg
}  // namespace selfgpu


// ---------------------------------------------------------------------------------- GMRES scalars
namespace selfgpu {
namespace cg {

// After the Arnoldi step i (0-based): H(:, i) holds h(1..i+2, i+1) of the reference (hnext = h(i+2,i+1)).
// Applies the previous Givens rotations to the new column, forms the new rotation, updates bhat and
// the residual estimate (IterativeSolvers_Class.f90:560-600), all in FP64.
__global__ void gmres_givens(const double* __restrict__ hcol, int i, int m, double* rho, double* c, double* s,
                             double* bhat, GMScalars* G, double* resi, int l) {
  if (G->done) return;  // the cycle already stopped: later steps of the enqueued cycle change nothing
  // hcol[0..i] = h(1..i+1, i+1) ; hcol[i+1] = ||w||^2
  const double hn = sqrt(hcol[i + 1]);
  double* R = rho + (size_t)i * m;  // column i of rho (rho(k, i+1) at R[k])
  G->i = i + 1;                     // Arnoldi steps of this cycle so far (the reference's l counts them)
  const double aeps = 2.220446049250313e-16;
  if (fabs(hn) <= aeps) {  // AlmostEqual(h(i+1,i), 0): lucky breakdown, column i stays out of the solve
    G->nr = i;
    G->breakdown = 1;
    G->done = 1;
    return;
  }
  G->nr = i + 1;
  R[0] = hcol[0];
  for (int k = 1; k <= i; ++k) {
    const double g = c[k - 1] * R[k - 1] + s[k - 1] * hcol[k];
    R[k] = -s[k - 1] * R[k - 1] + c[k - 1] * hcol[k];
    R[k - 1] = g;
  }
  const double d = sqrt(R[i] * R[i] + hn * hn);
  c[i] = R[i] / d;
  s[i] = hn / d;
  R[i] = c[i] * R[i] + s[i] * hn;
  bhat[i + 1] = -s[i] * bhat[i];
  bhat[i] = c[i] * bhat[i];
  G->rc = fabs(bhat[i + 1]);
  if (resi && l > 0) resi[l] = G->rc;
  if (!(G->rc == G->rc) || isinf(G->rc)) {  // non-finite recurrence: stop the cycle, the host reports it
    G->done = 1;
    return;
  }
  if (G->rc / G->r0 <= G->tol) G->done = 1;
}

// v_{i+1} = w / sqrt(hsq), or zero once the cycle stopped on a breakdown (no division by ~0)
template <typename R>
__global__ void gmres_next_basis(R* __restrict__ y, const R* __restrict__ w, const double* __restrict__ hsq,
                                 const GMScalars* __restrict__ G, size_t n) {
  const bool zero = G->breakdown != 0;
  const double f = zero ? 0.0 : 1.0 / sqrt(hsq[0]);
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    y[k] = zero ? (R)0 : (R)(f * (double)w[k]);
}

// back substitution of the triangular system (rho y = bhat) for nr columns
__global__ void gmres_backsolve(const double* __restrict__ rho, const double* __restrict__ bhat, int m,
                                const GMScalars* __restrict__ G, double* y) {
  const int nr = G->nr;
  auto RHO = [&](int k, int j) { return rho[(size_t)j * m + k]; };
  y[nr - 1] = bhat[nr - 1] / RHO(nr - 1, nr - 1);
  for (int k = nr - 2; k >= 0; --k) {
    double t = bhat[k];
    for (int j = k + 1; j < nr; ++j) t -= RHO(k, j) * y[j];
    y[k] = t / RHO(k, k);
  }
}

__global__ void sqrt_scalar(const double* __restrict__ a, double* __restrict__ b) { b[0] = sqrt(a[0]); }

}  // namespace cg
}  // namespace selfgpu

namespace {

using namespace selfgpu::cg;

// Shared-node topology: groups and primary-copy gather indices (CGsemElliptic_2D_Class.f90 :350-787)
// The direct-stiffness groups as cg_dss_mask_pairs reads them: two-copy non-Dirichlet groups as (primary,
// secondary) pairs, the others as CSR groups (same group order and summation order as the group list).
int upload_dss(self_ctx* ctx, const std::vector<int>& gptr, const std::vector<int>& gidx,
               const std::vector<unsigned char>& gdir, int ngroups, DevBuf<int2>& dpairs, DevBuf<int>& dgptr,
               DevBuf<int>& dgidx, DevBuf<unsigned char>& dgdir, int& npairs, int& nrest) {
  std::vector<int2> pairs;
  std::vector<int> rptr(1, 0), ridx;
  std::vector<unsigned char> rdir;
  for (int g = 0; g < ngroups; ++g) {
    const int a = gptr[g], b = gptr[g + 1];
    if (b - a == 2 && !gdir[g]) {
      pairs.push_back(make_int2(gidx[a], gidx[a + 1]));
    } else {
      for (int k = a; k < b; ++k) ridx.push_back(gidx[k]);
      rptr.push_back((int)ridx.size());
      rdir.push_back(gdir[g]);
    }
  }
  npairs = (int)pairs.size();
  nrest = (int)rdir.size();
  int rc;
  if (!pairs.empty() && (rc = upload(ctx, dpairs, pairs))) return rc;
  if ((rc = upload(ctx, dgptr, rptr))) return rc;
  if (!ridx.empty() && (rc = upload(ctx, dgidx, ridx))) return rc;
  if (!rdir.empty() && (rc = upload(ctx, dgdir, rdir))) return rc;
  return SELF_OK;
}

int compile_topology(self_cg2d* h, const self_cg2d_desc* d) {
  const int n = h->n, N = h->N;
  const size_t NN = (size_t)n * n;
  auto side_node = [&](int side, int k, int& i, int& j) {
    switch (side) {
      case 1: i = k; j = 0; break;
      case 2: i = N; j = k; break;
      case 3: i = k; j = N; break;
      default: i = 0; j = k; break;
    }
  };
  auto corner = [&](int c, int& i, int& j) {
    static const int ci[4] = {0, 1, 1, 0}, cj[4] = {0, 0, 1, 1};
    i = ci[c - 1] * N;
    j = cj[c - 1] * N;
  };
  auto lid = [&](int e1based, int i, int j) { return (int)((size_t)(e1based - 1) * NN + i + (size_t)n * j); };
  h->h_src.resize(h->nl);
  for (size_t k = 0; k < h->nl; ++k) h->h_src[k] = (int)k;
  h->h_gptr.assign(1, 0);
  h->h_gidx.clear();
  h->h_gdir.clear();
  for (int k = 0; k < d->nEdges; ++k) {
    const int* E = d->edges + 6 * k;
    if (E[0] < 1 || E[0] > d->nEl || E[1] < 1 || E[1] > 4)
      return set_error(h->ctx, SELF_ERR_INVALID, "edge %d: bad primary element/side", k + 1);
    if (E[2] > 0) {
      if (E[2] > d->nEl || std::abs(E[3]) < 1 || std::abs(E[3]) > 4 || (E[5] != 1 && E[5] != -1))
        return set_error(h->ctx, SELF_ERR_INVALID, "edge %d: bad secondary element/side", k + 1);
      int nn = E[4];
      for (int m = 1; m <= N - 1; ++m, nn += E[5]) {
        if (nn < 1 || nn > N - 1) return set_error(h->ctx, SELF_ERR_INVALID, "edge %d: bad start/inc", k + 1);
        int i1, j1, i2, j2;
        side_node(E[1], m, i1, j1);
        side_node(std::abs(E[3]), nn, i2, j2);
        int a = lid(E[0], i1, j1), b = lid(E[2], i2, j2);
        h->h_gidx.push_back(a);
        h->h_gidx.push_back(b);
        h->h_gptr.push_back((int)h->h_gidx.size());
        h->h_gdir.push_back(0);
        h->h_src[b] = a;
      }
    } else if (E[2] == SELF_DIRICHLET) {
      for (int m = 1; m <= N - 1; ++m) {
        int i1, j1;
        side_node(E[1], m, i1, j1);
        h->h_gidx.push_back(lid(E[0], i1, j1));
        h->h_gptr.push_back((int)h->h_gidx.size());
        h->h_gdir.push_back(1);
      }
    }
  }
  for (int nd = 0; nd < d->nNodes; ++nd) {
    const int a = d->n2e_ptr[nd], b = d->n2e_ptr[nd + 1];
    if (b <= a) continue;
    const bool dir = d->nodeType[nd] == SELF_DIRICHLET;
    int first = -1;
    for (int c = a; c < b; ++c) {
      if (d->n2e_elem[c] < 1 || d->n2e_elem[c] > d->nEl || d->n2e_local[c] < 1 || d->n2e_local[c] > 4)
        return set_error(h->ctx, SELF_ERR_INVALID, "node %d: bad element list", nd + 1);
      int i, j;
      corner(d->n2e_local[c], i, j);
      int l = lid(d->n2e_elem[c], i, j);
      h->h_gidx.push_back(l);
      if (first < 0) first = l;
      if (!dir) h->h_src[l] = first;
    }
    h->h_gptr.push_back((int)h->h_gidx.size());
    h->h_gdir.push_back(dir ? 1 : 0);
  }
  h->ngroups = (int)h->h_gdir.size();
  if (!h->upload_dev) return SELF_OK;
  int rc;
  if ((rc = upload(h->ctx, h->src, h->h_src))) return rc;
  if ((rc = upload(h->ctx, h->gptr, h->h_gptr))) return rc;
  if ((rc = upload(h->ctx, h->gidx, h->h_gidx))) return rc;
  if ((rc = upload(h->ctx, h->gdir, h->h_gdir))) return rc;
  return upload_dss(h->ctx, h->h_gptr, h->h_gidx, h->h_gdir, h->ngroups, h->dss_pairs, h->dss_gptr, h->dss_gidx,
                    h->dss_gdir, h->dss_npairs, h->dss_nrest);
}

// Folded element factors, Jacobi diagonal; FP64 master copy, FP32 copy for the inner solves.
int build_factors(self_cg2d* h, const self_cg2d_desc* d, std::vector<double>& Jww) {
  const int n = h->n;
  const size_t NN = (size_t)n * n;
  const int nf = h->nf;
  std::vector<double> fac((size_t)nf * NN * h->nEl), diag(h->nl);
  Jww.resize(h->nl);
  const double* D = d->dmat;
  const double* w = d->qweight;
  for (int e = 0; e < h->nEl; ++e)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const size_t id = (size_t)e * NN + i + (size_t)n * j;
        const double J = d->J[id];
        if (!(J != 0.0)) return set_error(h->ctx, SELF_ERR_INVALID, "zero Jacobian in element %d", e + 1);
        const double k = d->fluxCoeff[id], ww = w[i] * w[j];
        const double xs = d->dxds[id], xp = d->dxdp[id], ys = d->dyds[id], yp = d->dydp[id];
        double* fe = &fac[(size_t)e * nf * NN];
        const size_t t = i + (size_t)n * j;
        fe[t] = k * ww * (yp * yp + xp * xp) / J;
        fe[NN + t] = -k * ww * (ys * yp + xs * xp) / J;
        fe[2 * NN + t] = k * ww * (xs * xs + ys * ys) / J;
        fe[3 * NN + t] = h->lambda * J * ww;
        if (nf == 6) {
          fe[4 * NN + t] = ww * (h->vx * yp - h->vy * xp);
          fe[5 * NN + t] = ww * (h->vy * xs - h->vx * ys);
        }
        Jww[id] = J * w[i] * w[j];
      }
  // local diagonal (operator applied to unit vectors, closed form)
  for (int e = 0; e < h->nEl; ++e) {
    const double* fe = &fac[(size_t)e * nf * NN];
    for (int b = 0; b < n; ++b)
      for (int a = 0; a < n; ++a) {
        double s1 = 0, s2 = 0;
        for (int m = 0; m < n; ++m) {
          s1 += D[m + a * n] * D[m + a * n] * fe[m + (size_t)n * b];
          s2 += D[m + b * n] * D[m + b * n] * fe[2 * NN + a + (size_t)n * m];
        }
        const size_t t = a + (size_t)n * b;
        double v = -(s1 + s2 + 2.0 * D[a + a * n] * D[b + b * n] * fe[NN + t]) - fe[3 * NN + t];
        if (nf == 6) v -= fe[4 * NN + t] * D[a + a * n] + fe[5 * NN + t] * D[b + b * n];
        diag[(size_t)e * NN + t] = v;
      }
  }
  // assemble over the groups: primary copy gets the sum, masked copies get 1
  std::vector<double> dinv(h->nl);
  for (size_t k = 0; k < h->nl; ++k) dinv[k] = 1.0 / diag[k];
  for (int g = 0; g < h->ngroups; ++g) {
    const int a = h->h_gptr[g], b = h->h_gptr[g + 1];
    double s = 0;
    for (int k = a; k < b; ++k) s += diag[h->h_gidx[k]];
    for (int k = a; k < b; ++k) dinv[h->h_gidx[k]] = 1.0;
    if (!h->h_gdir[g]) dinv[h->h_gidx[a]] = 1.0 / s;
  }
  h->h_fac = fac;
  h->h_dinv = dinv;
  if (!h->upload_dev) return SELF_OK;
  // affine elements (metric terms and J the same at every node of the element to 1e-9 relative, far below the
  // FP32 rounding of the factors; the metric terms of a straight-sided element differ from node to node only by
  // the rounding of the derivative sums): the Helmholtz factors split into k w_i w_j per node and four numbers per
  // element, which the compact FP32 apply streams instead
  h->affine = nf == 4;
  for (int e = 0; e < h->nEl && h->affine; ++e) {
    const size_t b = (size_t)e * NN;
    auto geo = [&](size_t id, double* c) {
      const double xs = d->dxds[id], xp = d->dxdp[id], ys = d->dyds[id], yp = d->dydp[id], J = d->J[id];
      c[0] = (yp * yp + xp * xp) / J;
      c[1] = -(ys * yp + xs * xp) / J;
      c[2] = (xs * xs + ys * ys) / J;
      c[3] = J;
    };
    double c0[4];
    geo(b, c0);
    const double sc = std::max(std::fabs(c0[0]), std::fabs(c0[2]));
    for (size_t t = 0; t < NN && h->affine; ++t) {
      double c[4];
      geo(b + t, c);
      for (int q = 0; q < 3; ++q)
        if (std::fabs(c[q] - c0[q]) > 1e-9 * sc) h->affine = false;
      if (std::fabs(c[3] - c0[3]) > 1e-9 * std::fabs(c0[3])) h->affine = false;
    }
    if (h->affine) {
      h->h_ec.insert(h->h_ec.end(), {c0[0], c0[1], c0[2], h->lambda * c0[3]});
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) h->h_kw.push_back(d->fluxCoeff[b + i + (size_t)n * j] * w[i] * w[j]);
    }
  }
  if (!h->affine) {
    std::vector<double>().swap(h->h_ec);
    std::vector<double>().swap(h->h_kw);
  }
  int rc;
  if ((rc = upload(h->ctx, h->op64.fac, fac))) return rc;
  if ((rc = upload(h->ctx, h->op64.dinv, dinv))) return rc;
  h->op64.D.assign(D, D + NN);
  std::vector<float> f32(fac.begin(), fac.end()), di32(dinv.begin(), dinv.end());
  if ((rc = upload(h->ctx, h->op32.fac, f32))) return rc;
  if ((rc = upload(h->ctx, h->op32.dinv, di32))) return rc;
  h->op32.D.assign(D, D + NN);
  h->have32 = true;
  return SELF_OK;
}

// compact.cuh's layout functions for a run-time degree (host side of the compact build)
int compact_interior_index(int n, int e, int ii, int jj, int nEl) {
  switch (n) {
    case 3: return interior_index<3>(e, ii, jj, nEl);
    case 4: return interior_index<4>(e, ii, jj, nEl);
    case 5: return interior_index<5>(e, ii, jj, nEl);
    case 6: return interior_index<6>(e, ii, jj, nEl);
    case 7: return interior_index<7>(e, ii, jj, nEl);
    case 8: return interior_index<8>(e, ii, jj, nEl);
    case 9: return interior_index<9>(e, ii, jj, nEl);
    default: return interior_index<10>(e, ii, jj, nEl);
  }
}
size_t compact_factor_index(int n, int nf, int g, int f, int i, int line) {
  switch (n) {
    case 3: return factor_index<3>(nf, g, f, i, line);
    case 4: return factor_index<4>(nf, g, f, i, line);
    case 5: return factor_index<5>(nf, g, f, i, line);
    case 6: return factor_index<6>(nf, g, f, i, line);
    case 7: return factor_index<7>(nf, g, f, i, line);
    case 8: return factor_index<8>(nf, g, f, i, line);
    case 9: return factor_index<9>(nf, g, f, i, line);
    default: return factor_index<10>(nf, g, f, i, line);
  }
}

// Compact node layout of the FP32 inner PCG (compact.cuh): entity numbering, element descriptors, the compact ->
// element-local map and the Jacobi diagonal, from the shared-node groups.  Leaves cpt.ok false (the element-local
// form is used) when the groups are not those of a conforming mesh: an interior node shared or masked, a side whose
// nodes are partly Dirichlet or shared with several sides in different orders, an edge shared by more than two
// sides, or sizes beyond 32-bit indexing.
int compact_build(self_cg2d* h) {
  auto& C = h->cpt;
  C.tried = true;
  C.ok = false;
  const int n = h->n, N = h->N, M = n - 2, nEl = h->nEl;
  const size_t NN = (size_t)n * n, nl = h->nl;
  if (M < 1 || nl >= ((size_t)1 << 28) || !h->have32) return SELF_OK;
  const std::vector<int>& src = h->h_src;
  std::vector<unsigned char> mask(nl, 0);
  std::vector<int> gof(nl, -1), gpos(nl, -1);
  for (int g = 0; g < h->ngroups; ++g)
    for (int k = h->h_gptr[g]; k < h->h_gptr[g + 1]; ++k) {
      const int l = h->h_gidx[k];
      gof[l] = g;
      gpos[l] = k - h->h_gptr[g];
      if (h->h_gdir[g]) mask[l] = 1;
    }
  auto lid = [&](int e, int i, int j) { return (int)((size_t)e * NN + i + (size_t)n * j); };
  auto side_lid = [&](int e, int s, int m) {  // side s: 0 south (j = 0), 1 east (i = N), 2 north (j = N), 3 west
    switch (s) {
      case 0: return lid(e, m, 0);
      case 1: return lid(e, N, m);
      case 2: return lid(e, m, N);
      default: return lid(e, 0, m);
    }
  };
  auto side_of = [&](int l, int& e, int& s, int& m) {  // side and position of a node inside a side (not a corner)
    e = (int)(l / NN);
    const int t = (int)(l - (size_t)e * NN), i = t % n, j = t / n;
    const bool ib = i == 0 || i == N, jb = j == 0 || j == N;
    if (ib == jb) return false;
    if (j == 0) { s = 0; m = i; }
    else if (i == N) { s = 1; m = j; }
    else if (j == N) { s = 2; m = i; }
    else { s = 3; m = j; }
    return true;
  };
  for (int e = 0; e < nEl; ++e)
    for (int j = 1; j < N; ++j)
      for (int i = 1; i < N; ++i) {
        const int l = lid(e, i, j);
        if (mask[l] || src[l] != l || gof[l] >= 0) return SELF_OK;
      }
  // sides: the primary side (its nodes are their own primary copies) and the orientation of the others
  std::vector<int> skey(4 * (size_t)nEl, -1), nsec(4 * (size_t)nEl, 0);
  std::vector<unsigned char> sflip(4 * (size_t)nEl, 0), sslot(4 * (size_t)nEl, 0);
  for (int e = 0; e < nEl; ++e)
    for (int s = 0; s < 4; ++s) {
      int nm = 0;
      for (int m = 1; m < N; ++m) nm += mask[side_lid(e, s, m)];
      if (nm == N - 1) continue;  // Dirichlet side
      if (nm) return SELF_OK;
      int pe = -1, ps = -1, flip = 0;
      for (int m = 1; m < N; ++m) {
        int qe, qs, qm;
        if (!side_of(src[side_lid(e, s, m)], qe, qs, qm)) return SELF_OK;
        if (m == 1) {
          pe = qe;
          ps = qs;
          if (qm == 1) flip = 0;
          else if (qm == N - 1) flip = 1;
          else return SELF_OK;
        } else if (qe != pe || qs != ps || qm != (flip ? N - m : m)) {
          return SELF_OK;
        }
      }
      const int key = pe * 4 + ps, me = e * 4 + s;
      if (key == me) {
        if (flip) return SELF_OK;
      } else {
        sslot[me] = 1;
        if (++nsec[key] > 1) return SELF_OK;
      }
      skey[me] = key;
      sflip[me] = (unsigned char)flip;
    }
  for (int me = 0; me < 4 * nEl; ++me)
    if (skey[me] >= 0 && skey[skey[me]] != skey[me]) return SELF_OK;  // a secondary side's primary is not a side
  std::vector<int> eid(4 * (size_t)nEl, -1);
  int nE2 = 0, nE1 = 0;
  for (int k = 0; k < 4 * nEl; ++k)
    if (skey[k] == k && nsec[k] == 1) eid[k] = nE2++;
  for (int k = 0; k < 4 * nEl; ++k)
    if (skey[k] == k && nsec[k] == 0) eid[k] = nE2 + nE1++;
  // corners, numbered in order of first appearance; slots in the order of the copies in the shared-node group
  static const int ci[4] = {0, 1, 1, 0}, cj[4] = {0, 0, 1, 1};  // SW, SE, NE, NW
  std::vector<int> corner_of(nl, -1), cprim, coff(1, 0);
  std::vector<int4> desc(3 * (size_t)nEl);
  for (int e = 0; e < nEl; ++e) {
    int code[4], cc[4], fs[4];
    for (int s = 0; s < 4; ++s) {
      const int me = e * 4 + s;
      code[s] = skey[me] < 0 ? -1 : (eid[skey[me]] << 2) | (sslot[me] << 1) | sflip[me];
    }
    for (int c = 0; c < 4; ++c) {
      const int l = lid(e, ci[c] * N, cj[c] * N);
      cc[c] = -1;
      fs[c] = 0;
      if (mask[l]) continue;
      const int p = src[l];
      const int pt = (int)(p % NN), pi = pt % n, pj = pt / n;
      if (!((pi == 0 || pi == N) && (pj == 0 || pj == N))) return SELF_OK;
      if (gof[l] != gof[p] || (gof[p] >= 0 && gpos[p] != 0)) return SELF_OK;
      if (corner_of[p] < 0) {
        corner_of[p] = (int)cprim.size();
        cprim.push_back(p);
        const int g = gof[p];
        coff.push_back(coff.back() + (g >= 0 ? h->h_gptr[g + 1] - h->h_gptr[g] : 1));
      }
      const int id = corner_of[p];
      cc[c] = (id << 1) | (l == p ? 1 : 0);
      fs[c] = coff[id] + (gof[l] >= 0 ? gpos[l] : 0);
    }
    desc[3 * (size_t)e] = make_int4(code[0], code[1], code[2], code[3]);
    desc[3 * (size_t)e + 1] = make_int4(cc[0], cc[1], cc[2], cc[3]);
    desc[3 * (size_t)e + 2] = make_int4(fs[0], fs[1], fs[2], fs[3]);
  }
  const int nC = (int)cprim.size();
  const size_t nInt = (size_t)nEl * M * M, nEM = (size_t)(nE2 + nE1) * M;
  const size_t ng = nInt + nEM + nC, ngp = (ng + 3) / 4 * 4, nz = nInt + 2 * nEM + (size_t)coff.back();
  if (nz >= ((size_t)1 << 30) || ((size_t)(nE2 + nE1) << 2) >= ((size_t)1 << 30)) return SELF_OK;
  std::vector<int> cl(ng);
  for (int e = 0; e < nEl; ++e)
    for (int j = 1; j < N; ++j)
      for (int i = 1; i < N; ++i) cl[compact_interior_index(n, e, i - 1, j - 1, nEl)] = lid(e, i, j);
  // the FP32 factors line-interleaved by pass group (factor_index), the last group padded with zeros
  const int nf = h->nf, epl = kRedThreads / n, ngrp = (nEl + epl - 1) / epl;
  std::vector<float> facT(h->affine ? 0 : (size_t)ngrp * nf * n * epl * n, 0.f);
  for (int e = 0; e < nEl && !h->affine; ++e)
    for (int f = 0; f < nf; ++f)
      for (int t = 0; t < n; ++t)
        for (int i = 0; i < n; ++i)
          facT[compact_factor_index(n, nf, e / epl, f, i, (e % epl) * n + t)] =
              (float)h->h_fac[(size_t)e * nf * NN + (size_t)f * NN + (size_t)t * n + i];
  for (int k = 0; k < 4 * nEl; ++k)
    if (eid[k] >= 0)
      for (int m = 1; m < N; ++m) cl[nInt + (size_t)eid[k] * M + (m - 1)] = side_lid(k / 4, k % 4, m);
  for (int c = 0; c < nC; ++c) cl[nInt + nEM + c] = cprim[c];
  std::vector<float> dinv(ngp, 0.f);
  for (size_t k = 0; k < ng; ++k) dinv[k] = (float)h->h_dinv[cl[k]];
  self_ctx* ctx = h->ctx;
  int rc;
  if ((rc = upload(ctx, C.desc, desc)) || (rc = upload(ctx, C.coff, coff)) || (rc = upload(ctx, C.cl, cl)) ||
      (rc = upload(ctx, C.f32.dinv, dinv)))
    return rc;
  C.affine = h->affine;
  if (C.affine) {  // one streamed value per node (k w_i w_j, line-interleaved) and four per element
    std::vector<float> kwT((size_t)ngrp * n * epl * n, 0.f);
    std::vector<float4> ec(nEl);
    for (int e = 0; e < nEl; ++e) {
      for (int t = 0; t < n; ++t)
        for (int i = 0; i < n; ++i)
          kwT[compact_factor_index(n, 1, e / epl, 0, i, (e % epl) * n + t)] =
              (float)h->h_kw[(size_t)e * NN + (size_t)t * n + i];
      ec[e] = make_float4((float)h->h_ec[4 * (size_t)e], (float)h->h_ec[4 * (size_t)e + 1],
                          (float)h->h_ec[4 * (size_t)e + 2], (float)h->h_ec[4 * (size_t)e + 3]);
    }
    if ((rc = upload(ctx, C.kw, kwT)) || (rc = upload(ctx, C.ec, ec))) return rc;
    std::vector<double>().swap(h->h_kw);  // on the device now; the compact build runs once per handle
    std::vector<double>().swap(h->h_ec);
  } else if ((rc = upload(ctx, C.fac, facT))) {
    return rc;
  }
  for (DevBuf<float>* b : {&C.f32.u, &C.f32.r, &C.f32.v, &C.f32.v2, &C.f32.w}) {
    if (b->alloc(ngp) != cudaSuccess) return set_error(ctx, SELF_ERR_ALLOC, "device allocation of %zu floats", ngp);
    SELF_CUDA_TRY(ctx, cudaMemsetAsync(b->p, 0, ngp * sizeof(float), ctx->stream));
  }
  if (C.f32.zc.alloc(nz) != cudaSuccess)
    return set_error(ctx, SELF_ERR_ALLOC, "device allocation of %zu floats", nz);
  C.M = M;
  C.nInt = (int)nInt;
  C.nE2 = nE2;
  C.nE1 = nE1;
  C.nC = nC;
  C.ng = (int)ng;
  C.ngp = (int)ngp;
  C.nz = (int)nz;
  C.ok = true;
  return SELF_OK;
}

int ensure(self_ctx* ctx, DevBuf<double>& b, size_t n) {
  if (b.n >= n) return SELF_OK;
  if (b.alloc(n) != cudaSuccess) return set_error(ctx, SELF_ERR_ALLOC, "device allocation of %zu doubles", n);
  return SELF_OK;
}
int ensuref(self_ctx* ctx, DevBuf<float>& b, size_t n) {
  if (b.n >= n) return SELF_OK;
  if (b.alloc(n) != cudaSuccess) return set_error(ctx, SELF_ERR_ALLOC, "device allocation of %zu floats", n);
  return SELF_OK;
}

}  // namespace

extern "C" {

int self_cg2d_create(self_ctx* ctx, const self_cg2d_desc* d, self_cg2d** out) {
  if (!ctx || !d || !out) return SELF_ERR_INVALID;
  SELF_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  if (d->N < 2 || d->N > 9) return set_error(ctx, SELF_ERR_UNSUPPORTED, "CG degree %d outside 2..9", d->N);
  if (d->nEl < 1) return set_error(ctx, SELF_ERR_INVALID, "empty mesh");
  if (d->op != 0 && d->op != 1) return set_error(ctx, SELF_ERR_INVALID, "operator %d", d->op);
  std::unique_ptr<self_cg2d> h(new self_cg2d());
  h->ctx = ctx;
  h->N = d->N;
  h->n = d->N + 1;
  h->nEl = d->nEl;
  h->nEdges = d->nEdges;
  h->nNodes = d->nNodes;
  h->op = d->op;
  h->nf = d->op == 1 ? 6 : 4;
  h->lambda = d->lambda;
  h->vx = d->vx;
  h->vy = d->vy;
  h->nl = (size_t)h->n * h->n * h->nEl;
  int rc = compile_topology(h.get(), d);
  if (rc) return rc;
  if (d->x && d->y) {  // kept for the linear-FEM preconditioner, built on first use
    h->pcl.x.assign(d->x, d->x + h->nl);
    h->pcl.y.assign(d->y, d->y + h->nl);
  }
  std::vector<double> Jww;
  if ((rc = build_factors(h.get(), d, Jww))) return rc;
  h->h_J.assign(d->J, d->J + h->nl);
  h->h_w.assign(d->qweight, d->qweight + h->n);
  h->nblk = grid_for(ctx, h->nl);
  const int epb = (h->n * h->n >= 256) ? 1 : 256 / (h->n * h->n);
  const size_t groups = ((size_t)h->nEl + epb - 1) / epb;
  h->apply_grid = (int)std::max<size_t>(1, std::min(groups, (size_t)std::max(1, ctx->num_sms) * 8));
  if ((rc = ensure(ctx, h->partial, (size_t)2 * std::max(h->nblk, h->apply_grid)))) return rc;
  if (h->ticket.alloc(1) != cudaSuccess) return set_error(ctx, SELF_ERR_ALLOC, "device allocation failed");
  SELF_CUDA_TRY(ctx, cudaMemset(h->ticket.p, 0, sizeof(unsigned int)));
  if ((rc = ensure(ctx, h->red, 8))) return rc;
  if (h->S.alloc(1) != cudaSuccess) return set_error(ctx, SELF_ERR_ALLOC, "device allocation failed");
  if ((rc = ensure(ctx, h->t, h->nl))) return rc;
  *out = h.release();
  return SELF_OK;
}

int self_cg2d_destroy(self_cg2d* h) {
  if (!h) return SELF_OK;
  cudaSetDevice(h->ctx->device);
  cudaStreamSynchronize(h->ctx->stream);
  delete h;
  return SELF_OK;
}

// MatrixAction: Au = Mask(GlobalSum(L(UnMask(u)))).  u is read only (the reference leaves u masked).
int self_cg2d_matrix_action_f32(self_cg2d* h, const double* u, double* Au, int form) {
  if (!h || !u || !Au) return SELF_ERR_INVALID;
  self_ctx* ctx = h->ctx;
  SELF_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  if (form < SELF_F32_LOCAL || form > SELF_F32_COMPACT) return set_error(ctx, SELF_ERR_INVALID, "FP32 form %d", form);
  if (form == SELF_F32_TENSOR_CORES && h->N != 7)
    return set_error(ctx, SELF_ERR_UNSUPPORTED, "tensor-core FP32 operator: N = 7 only (N = %d)", h->N);
  const size_t nl = h->nl;
  int rc;
  if ((rc = ensure(ctx, h->r, nl)) || (rc = ensure(ctx, h->z, nl))) return rc;
  SELF_CUDA_TRY(ctx, cudaMemcpyAsync(h->r.p, u, nl * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  CGScalars hs{};  // first iteration of the fused apply: v = w, z = L(unmask(w)), alpha from num = 1
  hs.num = 1.0;
  SELF_CUDA_TRY(ctx, cudaMemcpyAsync(h->S.p, &hs, sizeof(hs), cudaMemcpyHostToDevice, ctx->stream));
  if (form == SELF_F32_COMPACT) {
    if (!h->cpt.tried && (rc = compact_build(h))) return rc;
    auto& Cp = h->cpt;
    if (!Cp.ok) return set_error(ctx, SELF_ERR_UNSUPPORTED, "compact layout: mesh not covered");
    compact_gather<float><<<h->nblk, kRedThreads, 0, ctx->stream>>>(Cp.f32.w.p, h->r.p, Cp.cl.p, Cp.ng, Cp.ngp);
    SELF_LAUNCHED(ctx);
    if ((rc = launch_compact_apply(h, Cp.f32.w.p, Cp.f32.v2.p, Cp.f32.v.p))) return rc;
    SELF_CUDA_TRY(ctx, cudaMemsetAsync(h->z.p, 0, nl * sizeof(double), ctx->stream));
    if ((rc = launch_compact_assemble(h, h->z.p))) return rc;
  } else {
    if ((rc = ensuref(ctx, h->w32, nl)) || (rc = ensuref(ctx, h->v32, nl)) || (rc = ensuref(ctx, h->v2_32, nl)) ||
        (rc = ensuref(ctx, h->z32, nl)))
      return rc;
    convert<float, double><<<h->nblk, kRedThreads, 0, ctx->stream>>>(h->w32.p, h->r.p, nl);
    SELF_LAUNCHED(ctx);
    h->tc = form == SELF_F32_TENSOR_CORES ? 1 : 0;
    rc = launch_apply_fused<float>(h, h->w32.p, h->v2_32.p, h->v32.p, h->z32.p, h->op32);
    h->tc = 0;
    if (rc || (rc = launch_dss<float>(h, h->z32.p))) return rc;
    convert<double, float><<<h->nblk, kRedThreads, 0, ctx->stream>>>(h->z.p, h->z32.p, nl);
    SELF_LAUNCHED(ctx);
  }
  CGScalars out{};
  SELF_CUDA_TRY(ctx, cudaMemcpyAsync(&out, h->S.p, sizeof(out), cudaMemcpyDeviceToHost, ctx->stream));
  SELF_CUDA_TRY(ctx, cudaMemcpyAsync(Au, h->z.p, nl * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  SELF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (out.ioerr == SELF_ERR_TIMEOUT) return set_error(ctx, SELF_ERR_TIMEOUT, "tensor-core barrier wait ran out");
  return SELF_OK;
}

int self_cg2d_matrix_action(self_cg2d* h, const double* u, double* Au) {
  if (!h || !u || !Au) return SELF_ERR_INVALID;
  self_ctx* ctx = h->ctx;
  SELF_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  int rc;
  if ((rc = ensure(ctx, h->v, h->nl)) || (rc = ensure(ctx, h->z, h->nl))) return rc;
  SELF_CUDA_TRY(ctx, cudaMemcpyAsync(h->v.p, u, h->nl * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  if ((rc = matrix_action<double>(h, h->v.p, h->z.p, h->op64))) return rc;
  SELF_CUDA_TRY(ctx, cudaMemcpyAsync(Au, h->z.p, h->nl * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  SELF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return SELF_OK;
}

}  // extern "C"

namespace selfgpu {
namespace cg {

// Mask: zero non-primary copies and Dirichlet nodes
template <typename R>
__global__ void cg_mask(R* __restrict__ v, const int* __restrict__ gptr, const int* __restrict__ gidx,
                        const unsigned char* __restrict__ gdir, int ngroups) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ngroups) return;
  const int a = gptr[g], b = gptr[g + 1];
  for (int k = gdir[g] ? a : a + 1; k < b; ++k) v[gidx[k]] = 0;
}

// UnMask: out[l] = in[src[l]]
template <typename R>
__global__ void cg_unmask(R* __restrict__ out, const R* __restrict__ in, const int* __restrict__ src, size_t n) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    out[k] = in[src[k]];
}

}  // namespace cg
}  // namespace selfgpu

namespace {

std::vector<double> make_load(const self_cg2d* h, const double* source) {
  std::vector<double> f(h->nl);
  const int n = h->n;
  const size_t NN = (size_t)n * n;
  for (size_t e = 0; e < (size_t)h->nEl; ++e)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const size_t id = e * NN + i + (size_t)n * j;
        f[id] = source[id] * h->h_J[id] * h->h_w[i] * h->h_w[j];  // source*J*ws(iS)*wp(iP)
      }
  return f;
}

int upload_vec(self_cg2d* h, DevBuf<double>& b, const double* host) {
  int rc = ensure(h->ctx, b, h->nl);
  if (rc) return rc;
  SELF_CUDA_TRY(h->ctx, cudaMemcpyAsync(b.p, host, h->nl * sizeof(double), cudaMemcpyHostToDevice, h->ctx->stream));
  return SELF_OK;
}

int download_vec(self_cg2d* h, double* host, const double* dev) {
  SELF_CUDA_TRY(h->ctx, cudaMemcpyAsync(host, dev, h->nl * sizeof(double), cudaMemcpyDeviceToHost, h->ctx->stream));
  SELF_CUDA_TRY(h->ctx, cudaStreamSynchronize(h->ctx->stream));
  return SELF_OK;
}

template <typename R>
int mask_dev(self_cg2d* h, R* v) {
  if (!h->ngroups) return SELF_OK;
  cg_mask<R><<<(h->ngroups + 255) / 256, 256, 0, h->ctx->stream>>>(v, h->gptr.p, h->gidx.p, h->gdir.p, h->ngroups);
  SELF_LAUNCHED(h->ctx);
  return SELF_OK;
}

template <typename R>
int unmask_dev(self_cg2d* h, R* out, const R* in) {
  cg_unmask<R><<<h->nblk, kRedThreads, 0, h->ctx->stream>>>(out, in, h->src.p, h->nl);
  SELF_LAUNCHED(h->ctx);
  return SELF_OK;
}

// AlmostEqual (CommonRoutines.f90:58-96): |a-b| <= eps, or eps relative to either value when neither is 0.
bool almost_equal(double a, double b) {
  const double eps = std::numeric_limits<double>::epsilon();
  if (a == 0.0 || b == 0.0) return std::fabs(a - b) <= eps;
  return std::fabs(a - b) <= eps * std::fabs(a) || std::fabs(a - b) <= eps * std::fabs(b);
}

// Node identification of ConstructLinearMeshFromOther (QuadMeshClass.f90:1899-1952): local node l takes the ID of
// the first earlier local node at the same position (AlmostEqual in x and y), else a new ID.  A hash grid of cell
// size 1e-9 x the mesh extent (far above AlmostEqual's ~1e-16 relative tolerance) limits the search to the 3 x 3
// neighbouring cells; the result is that of the reference's all-pairs search.
int linear_node_ids(const std::vector<double>& x, const std::vector<double>& y, std::vector<int>& uid) {
  const size_t n = x.size();
  double x0 = x[0], x1 = x[0], y0 = y[0], y1 = y[0];
  for (size_t k = 1; k < n; ++k) {
    x0 = std::min(x0, x[k]);
    x1 = std::max(x1, x[k]);
    y0 = std::min(y0, y[k]);
    y1 = std::max(y1, y[k]);
  }
  const double h = std::max({x1 - x0, y1 - y0, 1e-300}) * 1e-9;
  auto cell = [&](double v, double o) { return (long long)std::floor((v - o) / h); };
  auto key = [](long long a, long long b) {
    return (unsigned long long)a * 0x9E3779B97F4A7C15ull ^ (unsigned long long)b;
  };
  std::unordered_map<unsigned long long, int> head;  // cell -> latest node in it (list through `next`)
  head.reserve(n);
  std::vector<int> next(n, -1);
  uid.assign(n, -1);
  int nu = 0;
  for (size_t i = 0; i < n; ++i) {
    const long long cx = cell(x[i], x0), cy = cell(y[i], y0);
    int best = -1;
    for (long long dx = -1; dx <= 1; ++dx)
      for (long long dy = -1; dy <= 1; ++dy) {
        auto it = head.find(key(cx + dx, cy + dy));
        if (it == head.end()) continue;
        for (int j = it->second; j >= 0; j = next[j])
          if ((best < 0 || j < best) && almost_equal(x[i], x[j]) && almost_equal(y[i], y[j])) best = j;
      }
    uid[i] = best >= 0 ? uid[best] : nu++;
    auto it = head.find(key(cx, cy));
    if (it == head.end()) {
      head.emplace(key(cx, cy), (int)i);
    } else {
      next[i] = it->second;
      it->second = (int)i;
    }
  }
  return nu;
}

// Linear-FEM preconditioner operands, built on first use:
//  * the linear mesh's topology in the L-vector layout: node IDs by position (above); its Dirichlet set = the
//    nodes of sub-quad sides no other sub-quad shares (ConstructEdges gives them NO_NORMAL_FLOW, which
//    CGsemPreconditioner_2D Build turns into DIRICHLET), plus the spectral mesh's own Dirichlet nodes; src (copy
//    -> primary copy, the lowest local index, i.e. the first linear element of the node's list), groups (all
//    copies of a shared or Dirichlet node in element order), lprim (primary copies of non-Dirichlet nodes) and
//    dlift (copies Dirichlet here but not in the spectral mesh: the Dirichlet lift);
//  * the element stencils: per GLL sub-quad (bilinear element through its four corner nodes,
//    CGsemPreconditioner_2D's fluxCoeff = 1, Gauss-Lobatto weights 1) the folded metric factors at corner (a, b)
//      dx/ds = (x(si+1, pj+b) - x(si, pj+b)) / 2,  dx/dp = (x(si+a, pj+1) - x(si+a, pj)) / 2  (and y alike),
//      G11 = (yp^2 + xp^2) / J,  G12 = -(ys yp + xs xp) / J,  G22 = (xs^2 + ys^2) / J,  J = xs yp - xp ys,
//    (the transfinite metrics of a straight-sided element at its corners, MappedGeometryClass_2D GenerateMetrics
//    :611-710 on ConstructLinearMeshFromOther's straight side curves), the sub-quad operator formed from them
//    and summed into the element's 9-point stencil;
//  * work vectors in the precision asked for.
int pcl_ensure(self_cg2d* h, bool fp32, int nodes_mode) {
  auto& P = h->pcl;
  self_ctx* ctx = h->ctx;
  if (P.x.empty())
    return set_error(ctx, SELF_ERR_INVALID, "linear-FEM preconditioner: the descriptor gave no node positions (x, y)");
  if (nodes_mode != SELF_PC_NODES_POSITION && nodes_mode != SELF_PC_NODES_CONNECTIVITY)
    return set_error(ctx, SELF_ERR_INVALID, "preconditioner node identification %d", nodes_mode);
  int rc;
  const int N = h->N, n = h->n;
  const size_t NN = (size_t)n * n, nl = h->nl;
  if (P.built && P.nodes_mode != nodes_mode) {  // rebuild the topology; graphs hold the old group count
    P.built = false;
    for (auto& g : P.graph)
      if (g) {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
  }
  if (!P.built) {
    std::vector<int> uid;
    int nu = 0;
    if (nodes_mode == SELF_PC_NODES_POSITION) {
      nu = linear_node_ids(P.x, P.y, uid);
    } else {  // the spectral mesh's groups, numbered in first-appearance order
      std::vector<int> rep(nl);
      for (size_t l = 0; l < nl; ++l) rep[l] = (int)l;
      for (int g = 0; g < h->ngroups; ++g)
        for (int k = h->h_gptr[g]; k < h->h_gptr[g + 1]; ++k) rep[h->h_gidx[k]] = h->h_gidx[h->h_gptr[g]];
      std::vector<int> id_of(nl, -1);
      uid.assign(nl, 0);
      for (size_t l = 0; l < nl; ++l) {
        int& v = id_of[rep[l]];
        if (v < 0) v = nu++;
        uid[l] = v;
      }
    }
    std::vector<unsigned char> dir(nu, 0);
    for (int g = 0; g < h->ngroups; ++g)
      if (h->h_gdir[g])
        for (int k = h->h_gptr[g]; k < h->h_gptr[g + 1]; ++k) dir[uid[h->h_gidx[k]]] = 1;
    // sub-quad sides on the spectral elements' sides (sub-quad sides inside an element are always shared)
    std::unordered_map<unsigned long long, int> sides;
    sides.reserve((size_t)h->nEl * 4 * N);
    auto side_key = [](int a, int b) {
      return ((unsigned long long)std::min(a, b) << 32) | (unsigned long long)std::max(a, b);
    };
    auto side_node = [&](int side, int k, int& i, int& j) {
      switch (side) {
        case 0: i = k; j = 0; break;
        case 1: i = N; j = k; break;
        case 2: i = k; j = N; break;
        default: i = 0; j = k; break;
      }
    };
    for (int pass = 0; pass < 2; ++pass)
      for (int e = 0; e < h->nEl; ++e)
        for (int side = 0; side < 4; ++side)
          for (int m = 0; m < N; ++m) {
            int i0, j0, i1, j1;
            side_node(side, m, i0, j0);
            side_node(side, m + 1, i1, j1);
            const int a = uid[(size_t)e * NN + i0 + (size_t)n * j0], b = uid[(size_t)e * NN + i1 + (size_t)n * j1];
            if (pass == 0) {
              sides[side_key(a, b)] += 1;
            } else if (sides[side_key(a, b)] == 1) {
              dir[a] = 1;
              dir[b] = 1;
            }
          }
    // copies of every node, in local-index (= element) order
    std::vector<int> first(nu, -1), ptr(nu + 1, 0);
    for (size_t l = 0; l < nl; ++l) {
      ptr[uid[l] + 1]++;
      if (first[uid[l]] < 0) first[uid[l]] = (int)l;
    }
    for (int u = 0; u < nu; ++u) ptr[u + 1] += ptr[u];
    std::vector<int> lst(nl), pos(ptr.begin(), ptr.end() - 1);
    for (size_t l = 0; l < nl; ++l) lst[pos[uid[l]]++] = (int)l;
    std::vector<int> src(nl), gptr(1, 0), gidx;
    std::vector<unsigned char> gdir, lprim(nl, 0), sdir(nl, 0), dlift(nl, 0);
    for (int g = 0; g < h->ngroups; ++g)
      if (h->h_gdir[g])
        for (int k = h->h_gptr[g]; k < h->h_gptr[g + 1]; ++k) sdir[h->h_gidx[k]] = 1;
    P.lift = false;
    for (size_t l = 0; l < nl; ++l) {
      const int u = uid[l];
      src[l] = dir[u] ? (int)l : first[u];
      lprim[l] = (!dir[u] && first[u] == (int)l) ? 1 : 0;
      dlift[l] = (dir[u] && !sdir[l]) ? 1 : 0;
      P.lift = P.lift || dlift[l];
    }
    int nd = 0;
    for (int u = 0; u < nu; ++u) {
      nd += dir[u];
      if (ptr[u + 1] - ptr[u] < 2 && !dir[u]) continue;
      for (int k = ptr[u]; k < ptr[u + 1]; ++k) gidx.push_back(lst[k]);
      gptr.push_back((int)gidx.size());
      gdir.push_back(dir[u]);
    }
    P.ngroups = (int)gdir.size();
    P.nodes_mode = nodes_mode;
    P.nUnique = nu;
    P.nDirichlet = nd;
    // the element's 9-point stencil: every sub-quad's 4 x 4 operator (FluxDivergence on the sub-quad applied to
    // its 4 unit corner vectors) added into the rows of its corner nodes; kept: self, E, N, NE, NW per node
    std::vector<double> fac((size_t)kQ1Slots * NN * h->nEl, 0.0);
    std::vector<double> st(NN * 9);
    for (int e = 0; e < h->nEl; ++e) {
      const double* X = &P.x[(size_t)e * NN];
      const double* Y = &P.y[(size_t)e * NN];
      std::fill(st.begin(), st.end(), 0.0);
      for (int pj = 0; pj < N; ++pj)
        for (int si = 0; si < N; ++si) {
          double G11[4], G12[4], G22[4];
          for (int b = 0; b < 2; ++b)
            for (int a = 0; a < 2; ++a) {
              const double xs = 0.5 * (X[(si + 1) + n * (pj + b)] - X[si + n * (pj + b)]);
              const double ys = 0.5 * (Y[(si + 1) + n * (pj + b)] - Y[si + n * (pj + b)]);
              const double xp = 0.5 * (X[(si + a) + n * (pj + 1)] - X[(si + a) + n * pj]);
              const double yp = 0.5 * (Y[(si + a) + n * (pj + 1)] - Y[(si + a) + n * pj]);
              const double J = xs * yp - xp * ys;
              if (!(J != 0.0) || !std::isfinite(J))
                return set_error(ctx, SELF_ERR_INVALID, "degenerate GLL sub-quad in element %d", e + 1);
              const int c = a + 2 * b;
              G11[c] = (yp * yp + xp * xp) / J;
              G12[c] = -(ys * yp + xs * xp) / J;
              G22[c] = (xs * xs + ys * ys) / J;
            }
          for (int beta = 0; beta < 4; ++beta) {
            double u[4] = {0, 0, 0, 0}, F1[4], F2[4];
            u[beta] = 1.0;
            for (int c = 0; c < 4; ++c) {
              const int a = c & 1, b = c >> 1;
              const double us = 0.5 * (u[1 + 2 * b] - u[2 * b]);
              const double up = 0.5 * (u[a + 2] - u[a]);
              F1[c] = G11[c] * us + G12[c] * up;
              F2[c] = G12[c] * us + G22[c] * up;
            }
            for (int al = 0; al < 4; ++al) {
              const int a = al & 1, b = al >> 1;
              const double d1 = (a ? 0.5 : -0.5) * (F1[2 * b] + F1[1 + 2 * b]);
              const double d2 = (b ? 0.5 : -0.5) * (F2[a] + F2[a + 2]);
              const int di = (beta & 1) - a, dj = (beta >> 1) - b;
              st[(size_t)((si + a) + n * (pj + b)) * 9 + (di + 1) + 3 * (dj + 1)] += -(d1 + d2);
            }
          }
        }
      double* fe = &fac[(size_t)e * kQ1Slots * NN];
      for (size_t t = 0; t < NN; ++t) {
        const double* c9 = &st[t * 9];
        fe[kQ1Self * NN + t] = c9[4];  // (0, 0)
        fe[kQ1E * NN + t] = c9[5];     // (1, 0)
        fe[kQ1N * NN + t] = c9[7];     // (0, 1)
        fe[kQ1NE * NN + t] = c9[8];    // (1, 1)
        fe[kQ1NW * NN + t] = c9[6];    // (-1, 1)
      }
    }
    if ((rc = upload(ctx, P.fac64, fac))) return rc;
    std::vector<float> f32(fac.begin(), fac.end());
    if ((rc = upload(ctx, P.fac32, f32))) return rc;
    if ((rc = upload(ctx, P.src, src)) || (rc = upload(ctx, P.lprim, lprim))) return rc;
    if (P.lift && (rc = upload(ctx, P.dlift, dlift))) return rc;
    if (P.ngroups > 0 &&
        ((rc = upload(ctx, P.gptr, gptr)) || (rc = upload(ctx, P.gidx, gidx)) || (rc = upload(ctx, P.gdir, gdir)) ||
         (rc = upload_dss(ctx, gptr, gidx, gdir, P.ngroups, P.dss_pairs, P.dss_gptr, P.dss_gidx, P.dss_gdir,
                          P.dss_npairs, P.dss_nrest))))
      return rc;
    if (P.SL.n == 0 && P.SL.alloc(1) != cudaSuccess) return set_error(ctx, SELF_ERR_ALLOC, "allocation failed");
    P.built = true;
  }
  if (fp32) {
    if ((rc = ensuref(ctx, P.rl32, nl)) || (rc = ensuref(ctx, P.ul32, nl)) || (rc = ensuref(ctx, P.vl32, nl)) ||
        (rc = ensuref(ctx, P.vl2_32, nl)) || (rc = ensuref(ctx, P.zl32, nl)) ||
        (P.lift && (rc = ensuref(ctx, P.rd32, nl))))
      return rc;
  } else if ((rc = ensure(ctx, P.rl, nl)) || (rc = ensure(ctx, P.ul, nl)) || (rc = ensure(ctx, P.vl, nl)) ||
             (rc = ensure(ctx, P.vl2, nl)) || (rc = ensure(ctx, P.zl, nl)) || (P.lift && (rc = ensure(ctx, P.rd, nl)))) {
    return rc;
  }
  return SELF_OK;
}

template <typename R>
PcRun<R> pcl_run(self_cg2d* h, int iters);
template <>
PcRun<double> pcl_run<double>(self_cg2d* h, int iters) {
  auto& P = h->pcl;
  return PcRun<double>{P.fac64.p, P.src.p, P.gptr.p, P.gidx.p, P.gdir.p, P.lprim.p, P.dlift.p, P.ngroups, iters,
                       P.dss_pairs.p, P.dss_gptr.p, P.dss_gidx.p, P.dss_gdir.p, P.dss_npairs, P.dss_nrest,
                       P.rl.p, P.ul.p, P.vl.p, P.vl2.p, P.zl.p, P.lift ? P.rd.p : nullptr, P.SL.p};
}
template <>
PcRun<float> pcl_run<float>(self_cg2d* h, int iters) {
  auto& P = h->pcl;
  return PcRun<float>{P.fac32.p, P.src.p, P.gptr.p, P.gidx.p, P.gdir.p, P.lprim.p, P.dlift.p, P.ngroups, iters,
                      P.dss_pairs.p, P.dss_gptr.p, P.dss_gidx.p, P.dss_gdir.p, P.dss_npairs, P.dss_nrest,
                      P.rl32.p, P.ul32.p, P.vl32.p, P.vl2_32.p, P.zl32.p, P.lift ? P.rd32.p : nullptr, P.SL.p};
}

// inner CG limits of the preconditioner (pcl_start resets the other scalars and keeps these)
int pcl_limits(self_cg2d* h, int iters, double tol) {
  CGScalars sl{};
  sl.maxIters = iters;
  sl.tol = tol;
  SELF_CUDA_TRY(h->ctx, cudaMemcpyAsync(h->pcl.SL.p, &sl, sizeof(sl), cudaMemcpyHostToDevice, h->ctx->stream));
  return SELF_OK;
}

// Dirichlet values into the solution's Dirichlet nodes (SetDirichletBoundaryCondition :234-301)
void set_dirichlet_host(const self_cg2d* h, double* sol, const double* dir) {
  for (int g = 0; g < h->ngroups; ++g) {
    if (!h->h_gdir[g]) continue;
    for (int k = h->h_gptr[g]; k < h->h_gptr[g + 1]; ++k) {
      const int l = h->h_gidx[k];
      sol[l] = dir ? dir[l] : 0.0;
    }
  }
}

double read1(self_cg2d* h, const double* dptr, int* rc) {
  double v = 0;
  *rc = read_scalar(h, dptr, &v);
  return v;
}

// One GMRES cycle (IterativeSolvers_Class.f90:520-640) on the device, enqueued whole: up to msteps Arnoldi steps
// with modified Gram-Schmidt (dots accumulated in FP64) and Givens rotations in FP64, then the back substitution
// and x += V y (or dinv (V y) for the Jacobi-preconditioned flexible form).  The stop test runs on the device (the
// Givens kernel sets done; later steps of the enqueued cycle leave the solve unchanged), so the host synchronises
// once per cycle.  r holds the cycle's starting residual; the basis, matrix action and update are in the
// precision R (FP64, or FP32 for the inner solves of the refinement form).  G->r0 / G->tol set the relative stop.
struct CycleOut {
  int steps, nr, done, breakdown;
  double rc;
};

// Launch shape of mgs_onchip: one block per SM, chunk = the L-vector share of a block (a multiple of 4 nodes);
// false (streaming MGS) when the L-vector length is not a multiple of 4 (16-byte vector access), the share does not
// fit the opt-in shared memory of a block, the device has no cooperative launch, or a buffer cannot be allocated.
template <typename R>
bool mgs_onchip_plan(self_cg2d* h, int* nb, int* chunk, size_t* smem) {
  self_ctx* ctx = h->ctx;
  int coop = 0, optin = 0;
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device) != cudaSuccess || !coop) return false;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device) != cudaSuccess)
    return false;
  if (h->nl % 4 != 0) return false;  // every basis vector and block chunk must start on a 16-byte boundary
  const int sms = std::max(1, ctx->num_sms);
  const size_t c = ((h->nl + sms - 1) / sms + 3) / 4 * 4;
  const size_t bytes = c * sizeof(R);
  if (bytes + 2048 > (size_t)optin) return false;
  // for the current device, once per cycle (a process may drive several devices; the call is cheap)
  if (cudaFuncSetAttribute(mgs_onchip<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess)
    return false;
  int q = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&q, mgs_onchip<R>, kMgsThreads, bytes) != cudaSuccess || q < 1)
    return false;
  if (h->mgs_part.n < 2 * (size_t)sms && h->mgs_part.alloc(2 * (size_t)sms) != cudaSuccess) return false;
  if (!h->mgs_bar.p && h->mgs_bar.alloc(2) != cudaSuccess) return false;
  if (!h->mgs_err.p && h->mgs_err.alloc(1) != cudaSuccess) return false;
  *nb = sms;
  *chunk = (int)c;
  *smem = bytes;
  return true;
}

template <typename R>
int gmres_cycle(self_cg2d* h, R* x, const R* r, int m, int msteps, double r0, double tol, double rcur, R* V, R* w,
                R* t, const R* dinv, const OpData<R>& od, double* resi_dev, int l0, int maxIters, CycleOut* out) {
  self_ctx* ctx = h->ctx;
  cudaStream_t st = ctx->stream;
  const size_t nl = h->nl;
  int rc;
  // b = ||r|| ; v1 = r / b ; bhat(1) = b
  if ((rc = dots<R>(h, r, r, nullptr, nullptr, h->red.p))) return rc;
  sqrt_scalar<<<1, 1, 0, st>>>(h->red.p, h->red.p + 4);
  SELF_LAUNCHED(ctx);
  scale_copy<R><<<h->nblk, kRedThreads, 0, st>>>(V, r, h->red.p + 4, 1, nl);
  SELF_LAUNCHED(ctx);
  SELF_CUDA_TRY(ctx, cudaMemsetAsync(h->gm_bhat.p, 0, (m + 1) * sizeof(double), st));
  SELF_CUDA_TRY(ctx, cudaMemcpyAsync(h->gm_bhat.p, h->red.p + 4, sizeof(double), cudaMemcpyDeviceToDevice, st));
  SELF_CUDA_TRY(ctx, cudaMemsetAsync(h->gm_rho.p, 0, (size_t)m * m * sizeof(double), st));
  GMScalars G{};
  G.r0 = r0;
  G.tol = tol;
  G.rc = rcur;
  SELF_CUDA_TRY(ctx, cudaMemcpyAsync(h->GS.p, &G, sizeof(G), cudaMemcpyHostToDevice, st));
  // on-chip MGS when every SM's share of w fits its shared memory and all blocks can be resident together
  int nbm = 0, chunk = 0;
  size_t smem = 0;
  const bool onchip = mgs_onchip_plan<R>(h, &nbm, &chunk, &smem);
  if (onchip) SELF_CUDA_TRY(ctx, cudaMemsetAsync(h->mgs_err.p, 0, sizeof(int), st));
  for (int i = 0; i < msteps; ++i) {
    const R* vi = V + (size_t)i * nl;
    if (dinv) {  // z_i = PreconditionInvert(v_i)
      scale_by<R><<<h->nblk, kRedThreads, 0, st>>>(t, vi, dinv, nl);
      SELF_LAUNCHED(ctx);
      if ((rc = matrix_action<R>(h, t, w, od))) return rc;
    } else if ((rc = matrix_action<R>(h, vi, w, od))) {
      return rc;
    }
    const int l = l0 + i + 1;
    if (onchip) {  // MGS with w in shared memory, v_{i+1} written by the same launch; then Givens
      SELF_CUDA_TRY(ctx, cudaMemsetAsync(h->mgs_bar.p, 0, 2 * sizeof(unsigned int), st));
      const R* wc = w;
      size_t nlc = nl;
      int ic = i, ch = chunk;
      double *Hc = h->gm_H.p, *pc = h->mgs_part.p;
      unsigned int* bc = h->mgs_bar.p;
      int* ec = h->mgs_err.p;
      void* args[] = {(void*)&wc, (void*)&V, (void*)&nlc, (void*)&ic, (void*)&ch, (void*)&Hc, (void*)&pc, (void*)&bc,
                      (void*)&ec};
      SELF_CUDA_TRY(ctx, cudaLaunchCooperativeKernel((const void*)mgs_onchip<R>, dim3(nbm), dim3(kMgsThreads), args,
                                                     smem, st));
      SELF_LAUNCHED(ctx);
      gmres_givens<<<1, 1, 0, st>>>(h->gm_H.p, i, m, h->gm_rho.p, h->gm_c.p, h->gm_s.p, h->gm_bhat.p, h->GS.p,
                                    resi_dev, l <= maxIters ? l : 0);
      SELF_LAUNCHED(ctx);
      continue;
    }
    // MGS: h(k,i) = <v_k, w>; w -= h(k,i) v_k, the axpy of step k fused with the dot of step k+1
    if ((rc = dots<R>(h, V, w, nullptr, nullptr, h->gm_H.p))) return rc;
    for (int k = 0; k <= i; ++k) {
      const R* vk = V + (size_t)k * nl;
      const R* vn = (k < i) ? V + (size_t)(k + 1) * nl : nullptr;
      mgs_axpy_dot_fused<R><<<h->nblk, kRedThreads, 0, st>>>(w, vk, h->gm_H.p + k, vn, nl, h->partial.p, h->ticket.p,
                                                             h->gm_H.p + k + 1);
      SELF_LAUNCHED(ctx);
    }
    // gm_H[i+1] = <w,w>; Givens on the device
    gmres_givens<<<1, 1, 0, st>>>(h->gm_H.p, i, m, h->gm_rho.p, h->gm_c.p, h->gm_s.p, h->gm_bhat.p, h->GS.p,
                                  resi_dev, l <= maxIters ? l : 0);
    SELF_LAUNCHED(ctx);
    // v_{i+1} = w / h(i+1, i)
    gmres_next_basis<R><<<h->nblk, kRedThreads, 0, st>>>(V + (size_t)(i + 1) * nl, w, h->gm_H.p + i + 1, h->GS.p,
                                                         nl);
    SELF_LAUNCHED(ctx);
  }
  SELF_CUDA_TRY(ctx, cudaMemcpyAsync(&G, h->GS.p, sizeof(G), cudaMemcpyDeviceToHost, st));
  SELF_CUDA_TRY(ctx, cudaStreamSynchronize(st));
  if (onchip) {
    int err = 0;
    SELF_CUDA_TRY(ctx, cudaMemcpy(&err, h->mgs_err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) return set_error(ctx, SELF_ERR_TIMEOUT, "GMRES: a grid barrier wait of the on-chip MGS ran out");
  }
  out->steps = G.done ? G.i : msteps;
  out->nr = G.nr;
  out->done = G.done;
  out->breakdown = G.breakdown;
  out->rc = G.rc;
  if (G.nr >= 1) {
    gmres_backsolve<<<1, 1, 0, st>>>(h->gm_rho.p, h->gm_bhat.p, m, h->GS.p, h->gm_y.p);
    SELF_LAUNCHED(ctx);
    gmres_update<R><<<h->nblk, kRedThreads, 0, st>>>(x, V, h->gm_y.p, G.nr, nl, dinv);
    SELF_LAUNCHED(ctx);
  }
  return SELF_OK;
}

int gmres_buffers(self_cg2d* h, int m, bool fp32) {
  self_ctx* ctx = h->ctx;
  const size_t nl = h->nl;
  int rc;
  if (fp32) {
    if ((rc = ensuref(ctx, h->gm_V32, nl * (size_t)(m + 1)))) return rc;
  } else if ((rc = ensure(ctx, h->gm_V, nl * (size_t)(m + 1)))) {
    return rc;
  }
  if ((rc = ensure(ctx, h->gm_H, (size_t)(m + 2)))) return rc;
  if ((rc = ensure(ctx, h->gm_rho, (size_t)m * m))) return rc;
  if ((rc = ensure(ctx, h->gm_c, m)) || (rc = ensure(ctx, h->gm_s, m)) || (rc = ensure(ctx, h->gm_bhat, m + 1)) ||
      (rc = ensure(ctx, h->gm_y, m + 1)) || (rc = ensure(ctx, h->w, nl)) || (rc = ensure(ctx, h->t, nl)))
    return rc;
  if (h->GS.n == 0 && h->GS.alloc(1) != cudaSuccess) return set_error(ctx, SELF_ERR_ALLOC, "allocation failed");
  return SELF_OK;
}

int resi_to_host(self_cg2d* h, DevBuf<double>& resi_dev, double* resi_host, int maxIters, int l) {
  std::vector<double> tmp((size_t)maxIters + 1);
  SELF_CUDA_TRY(h->ctx, cudaMemcpyAsync(tmp.data(), resi_dev.p, tmp.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                        h->ctx->stream));
  SELF_CUDA_TRY(h->ctx, cudaStreamSynchronize(h->ctx->stream));
  for (int k = 1; k <= std::min(l, maxIters); ++k) resi_host[k] = tmp[k];
  return SELF_OK;
}

// GMRES(m) of IterativeSolvers_Class.f90:493-652, or with dinv the flexible right-preconditioned GMRES of
// Solve_PCGMRES (:656-822) with Jacobi: z_i = dinv v_i, w = A z_i, and x += Z y = dinv (V y) at the end of a
// cycle (the preconditioner is fixed, so the basis Z is not stored).  FP64; x, r are device vectors, r holds the
// initial residual and r0 its norm.  Returns ioerr (0, -1, or SELF_ERR_NONFINITE); iters = total Arnoldi steps
// (the reference's l).
int gmres_device(self_cg2d* h, const double* f, double* x, double* r, int m, int maxIters, double tol, double r0,
                 double* resi_host, int* iters, double* rel, const double* dinv) {
  self_ctx* ctx = h->ctx;
  int rc;
  if ((rc = gmres_buffers(h, m, false))) return rc;
  DevBuf<double> resi_dev;
  if (resi_host) {
    if ((rc = ensure(ctx, resi_dev, (size_t)maxIters + 1))) return rc;
    SELF_CUDA_TRY(ctx, cudaMemsetAsync(resi_dev.p, 0, ((size_t)maxIters + 1) * sizeof(double), ctx->stream));
    resi_host[0] = r0;
  }
  int l = 0, ioerr = -1;
  double rcur = r0;
  *iters = 0;
  if (r0 == 0.0) {
    *rel = 0.0;
    return 0;
  }
  while (l < maxIters) {
    CycleOut co{};
    if ((rc = gmres_cycle<double>(h, x, r, m, std::min(m, maxIters - l), r0, tol, rcur, h->gm_V.p, h->w.p, h->t.p,
                                  dinv, h->op64, resi_host ? resi_dev.p : nullptr, l, maxIters, &co)))
      return rc;
    l += co.steps;
    rcur = co.rc;
    if (!std::isfinite(rcur)) {
      ioerr = SELF_ERR_NONFINITE;
      break;
    }
    if (rcur / r0 <= tol) {
      ioerr = 0;
      break;
    }
    if (co.breakdown || l >= maxIters) break;
    if ((rc = residual<double>(h, f, x, r, h->op64))) return rc;
  }
  *iters = l;
  if (resi_host && (rc = resi_to_host(h, resi_dev, resi_host, maxIters, l))) return rc;
  *rel = rcur / r0;
  return ioerr;
}

// FP32-inner GMRES under FP64 iterative refinement: every refinement step is one GMRES(m) cycle in FP32 (basis,
// matrix action and update in FP32; Gram-Schmidt dots accumulated in FP64, Hessenberg, Givens and back
// substitution in FP64) on A d = r from d = 0, then x += d and r = b - A x in FP64.  The restart residual of
// GMRES(m) is thus the FP64 residual.  resi: ||r|| (FP64) per refinement step.  Returns ioerr as gmres_device.
int gmres_ir_device(self_cg2d* h, const double* f, double* x, double* r, int m, int maxIters, double tol, double r0,
                    double* resi_host, int* iters, int* outer_out, double* rel, const float* dinv32) {
  self_ctx* ctx = h->ctx;
  cudaStream_t st = ctx->stream;
  const size_t nl = h->nl;
  int rc;
  if ((rc = gmres_buffers(h, m, true)) || (rc = ensuref(ctx, h->u32, nl)) || (rc = ensuref(ctx, h->r32, nl)) ||
      (rc = ensuref(ctx, h->w32, nl)) || (rc = ensuref(ctx, h->z32, nl)) || (rc = ensure(ctx, h->z, nl)))
    return rc;
  int total = 0, outer = 0, ioerr = -1;
  double rn = r0;
  if (resi_host) resi_host[0] = r0;
  *iters = 0;
  *outer_out = 0;
  if (r0 == 0.0) {
    *rel = 0.0;
    return 0;
  }
  while (total < maxIters && rn / r0 >= tol) {
    convert<float, double><<<h->nblk, kRedThreads, 0, st>>>(h->r32.p, r, nl);
    SELF_LAUNCHED(ctx);
    SELF_CUDA_TRY(ctx, cudaMemsetAsync(h->u32.p, 0, nl * sizeof(float), st));
    CycleOut co{};
    if ((rc = gmres_cycle<float>(h, h->u32.p, h->r32.p, m, std::min(m, maxIters - total), r0, tol, rn, h->gm_V32.p,
                                 h->w32.p, h->z32.p, dinv32, h->op32, nullptr, 0, maxIters, &co)))
      return rc;
    total += co.steps;
    outer++;
    // x += d (FP64), r = b - A x in FP64
    convert<double, float><<<h->nblk, kRedThreads, 0, st>>>(h->z.p, h->u32.p, nl);
    SELF_LAUNCHED(ctx);
    axpby<double><<<h->nblk, kRedThreads, 0, st>>>(x, h->z.p, 1.0, 1.0, nl);
    SELF_LAUNCHED(ctx);
    if ((rc = residual<double>(h, f, x, r, h->op64))) return rc;
    if ((rc = dots<double>(h, r, r, nullptr, nullptr, h->red.p))) return rc;
    rn = std::sqrt(read1(h, h->red.p, &rc));
    if (rc) return rc;
    if (resi_host && outer <= maxIters) resi_host[outer] = rn;
    if (!std::isfinite(rn) || !std::isfinite(co.rc)) {
      ioerr = SELF_ERR_NONFINITE;
      break;
    }
    if (co.nr < 1) break;  // breakdown on the first column: no progress possible
  }
  if (ioerr != SELF_ERR_NONFINITE) ioerr = (rn / r0 < tol) ? 0 : -1;
  *iters = total;
  *outer_out = outer;
  *rel = rn / r0;
  return ioerr;
}

}  // namespace

extern "C" {

int self_cg2d_residual(self_cg2d* h, const double* source, const double* solution, double* r) {
  if (!h || !source || !solution || !r) return SELF_ERR_INVALID;
  self_ctx* ctx = h->ctx;
  SELF_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  std::vector<double> load = make_load(h, source);
  int rc;
  if ((rc = upload_vec(h, h->f, load.data())) || (rc = upload_vec(h, h->u, solution)) ||
      (rc = ensure(ctx, h->r, h->nl)))
    return rc;
  if ((rc = residual<double>(h, h->f.p, h->u.p, h->r.p, h->op64))) return rc;
  return download_vec(h, r, h->r.p);
}

int self_cg2d_dot(self_cg2d* h, const double* u, const double* v, double* out) {
  if (!h || !u || !v || !out) return SELF_ERR_INVALID;
  self_ctx* ctx = h->ctx;
  SELF_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  int rc;
  if ((rc = upload_vec(h, h->v, u)) || (rc = upload_vec(h, h->w, v))) return rc;
  if ((rc = mask_dev<double>(h, h->v.p)) || (rc = mask_dev<double>(h, h->w.p))) return rc;
  if ((rc = dots<double>(h, h->v.p, h->w.p, nullptr, nullptr, h->red.p))) return rc;
  return read_scalar(h, h->red.p, out);
}

int self_cg2d_mask(self_cg2d* h, double* u) {
  if (!h || !u) return SELF_ERR_INVALID;
  SELF_CUDA_TRY(h->ctx, cudaSetDevice(h->ctx->device));
  int rc;
  if ((rc = upload_vec(h, h->v, u)) || (rc = mask_dev<double>(h, h->v.p))) return rc;
  return download_vec(h, u, h->v.p);
}

int self_cg2d_unmask(self_cg2d* h, double* u) {
  if (!h || !u) return SELF_ERR_INVALID;
  SELF_CUDA_TRY(h->ctx, cudaSetDevice(h->ctx->device));
  int rc;
  if ((rc = upload_vec(h, h->v, u)) || (rc = ensure(h->ctx, h->w, h->nl)) || (rc = unmask_dev<double>(h, h->w.p, h->v.p)))
    return rc;
  return download_vec(h, u, h->w.p);
}

int self_cg2d_solve(self_cg2d* h, const self_solve_opts* o, const double* source, const double* dirichlet,
                    double* solution, double* resi, self_solve_report* rep) {
  if (!h || !o || !source || !solution) return SELF_ERR_INVALID;
  self_ctx* ctx = h->ctx;
  SELF_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  if (o->maxIters < 0 || !(o->tolerance > 0)) return set_error(ctx, SELF_ERR_INVALID, "bad solver options");
  if (o->method < SELF_SOLVE_CG || o->method > SELF_SOLVE_PCG_LINEAR)
    return set_error(ctx, SELF_ERR_INVALID, "solver method %d", o->method);
  const bool lin = o->method == SELF_SOLVE_PCG_LINEAR;
  if (lin && (o->pc_iterations < 0 || !(o->pc_tolerance >= 0)))
    return set_error(ctx, SELF_ERR_INVALID, "preconditioner iterations %d / tolerance %g", o->pc_iterations,
                     o->pc_tolerance);
  const bool gm = o->method == SELF_SOLVE_GMRES || o->method == SELF_SOLVE_PGMRES_JACOBI;
  if (gm && (o->m < 1 || o->m > 512))
    return set_error(ctx, SELF_ERR_INVALID, "GMRES restart length %d", o->m);
  if (gm && o->precision != SELF_PREC_FP64 && o->precision != SELF_PREC_FP32)
    return set_error(ctx, SELF_ERR_UNSUPPORTED, "GMRES precision %d", o->precision);
  const size_t nl = h->nl;
  int rc;
  std::vector<double> x0(solution, solution + nl);
  set_dirichlet_host(h, x0.data(), dirichlet);
  std::vector<double> load = make_load(h, source);
  if ((rc = upload_vec(h, h->f, load.data())) || (rc = upload_vec(h, h->u, x0.data())) ||
      (rc = ensure(ctx, h->r, nl)) || (rc = ensure(ctx, h->v, nl)) || (rc = ensure(ctx, h->w, nl)) ||
      (rc = ensure(ctx, h->z, nl)) || (!gm && (rc = ensure(ctx, h->v2, nl))))
    return rc;
  // the linear-FEM preconditioner with pc_iterations = 0 is the identity (w = r): plain CG
  const bool use_pcl = lin && o->pc_iterations > 0;
  if (use_pcl) {
    if ((rc = pcl_ensure(h, o->precision != SELF_PREC_FP64, o->pc_nodes))) return rc;
    if ((rc = pcl_limits(h, o->pc_iterations, o->pc_tolerance))) return rc;
  }
  if ((rc = residual<double>(h, h->f.p, h->u.p, h->r.p, h->op64))) return rc;
  self_solve_report R{};
  R.ioerr = -2;
  int iters = 0;
  double rel = 0, r0 = 0;
  // a NaN or Inf in the source, the initial guess or the Dirichlet data shows in ||r0||: stop before iterating
  if ((rc = dots<double>(h, h->r.p, h->r.p, nullptr, nullptr, h->red.p))) return rc;
  r0 = std::sqrt(read1(h, h->red.p, &rc));
  if (rc) return rc;
  if (!std::isfinite(r0)) {
    R.ioerr = SELF_ERR_NONFINITE;
    R.r0 = r0;
    R.rel_residual = r0;
    if (rep) *rep = R;
    return set_error(ctx, SELF_ERR_NONFINITE, "non-finite initial residual (NaN or Inf in the source, initial guess "
                     "or Dirichlet data)");
  }
  if (gm && o->precision == SELF_PREC_FP64) {
    R.ioerr = gmres_device(h, h->f.p, h->u.p, h->r.p, o->m, o->maxIters, o->tolerance, r0, resi, &iters, &rel,
                           o->method == SELF_SOLVE_PGMRES_JACOBI ? h->op64.dinv.p : nullptr);
    R.outer_iterations = 1;
  } else if (gm) {
    R.ioerr = gmres_ir_device(h, h->f.p, h->u.p, h->r.p, o->m, o->maxIters, o->tolerance, r0, resi, &iters,
                              &R.outer_iterations, &rel,
                              o->method == SELF_SOLVE_PGMRES_JACOBI ? h->op32.dinv.p : nullptr);
  } else {
    const bool jac = o->method == SELF_SOLVE_PCG_JACOBI;
    if (o->precision == SELF_PREC_FP64) {
      DevBuf<double> resi_dev;
      if (resi) {
        if ((rc = ensure(ctx, resi_dev, (size_t)o->maxIters + 1))) return rc;
        SELF_CUDA_TRY(ctx, cudaMemsetAsync(resi_dev.p, 0, ((size_t)o->maxIters + 1) * sizeof(double), ctx->stream));
      }
      // the compact layout (default) when the FP64 compact operator applies: CG on the correction d (d0 = 0,
      // the residual of the initial guess as right-hand side), x += d at the primary copies
      bool cpt64 = false;
      if (!use_pcl && o->inner_layout != SELF_LAYOUT_LOCAL) {
        if (!h->cpt.tried && (rc = compact_build(h))) return rc;
        if ((rc = compact_fp64_ready(h, &cpt64))) return rc;
      }
      if (cpt64) {
        auto& Cp = h->cpt;
        compact_gather<double><<<h->nblk, kRedThreads, 0, ctx->stream>>>(Cp.f64.r.p, h->r.p, Cp.cl.p, Cp.ng, Cp.ngp);
        SELF_LAUNCHED(ctx);
        SELF_CUDA_TRY(ctx, cudaMemsetAsync(Cp.f64.u.p, 0, (size_t)Cp.ngp * sizeof(double), ctx->stream));
        R.ioerr = pcg_device_compact<double>(h, jac, o->maxIters, o->tolerance, r0, resi ? resi_dev.p : nullptr, true,
                                             &iters, &rel);
        compact_scatter_add<double><<<h->nblk, kRedThreads, 0, ctx->stream>>>(h->u.p, Cp.f64.u.p, Cp.cl.p, Cp.ng);
        SELF_LAUNCHED(ctx);
      } else {
        const PcRun<double> pc = use_pcl ? pcl_run<double>(h, o->pc_iterations) : PcRun<double>{};
        R.ioerr = pcg_device<double>(h, h->u.p, h->r.p, h->v.p, h->w.p, h->z.p, jac ? h->op64.dinv.p : nullptr,
                                     o->maxIters, o->tolerance, r0, resi ? resi_dev.p : nullptr, &iters, &rel,
                                     h->op64, true, use_pcl ? &pc : nullptr);
      }
      if (resi) {
        SELF_CUDA_TRY(ctx, cudaMemcpyAsync(resi, resi_dev.p, ((size_t)o->maxIters + 1) * sizeof(double),
                                           cudaMemcpyDeviceToHost, ctx->stream));
        SELF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
        resi[0] = r0;
      }
      R.outer_iterations = 1;
    } else {
      // FP32 inner (P)CG under FP64 iterative refinement: x += A32^-1 r64, r64 = b - A64 x
      h->tc = (o->tensor_cores && h->N == 7) ? 1 : 0;
      const bool want_cpt = !use_pcl && !h->tc && o->inner_layout != SELF_LAYOUT_LOCAL;
      if (want_cpt && !h->cpt.tried && (rc = compact_build(h))) return rc;
      const bool use_cpt = want_cpt && h->cpt.ok;
      if (!use_cpt &&
          ((rc = ensuref(ctx, h->u32, nl)) || (rc = ensuref(ctx, h->r32, nl)) || (rc = ensuref(ctx, h->v32, nl)) ||
           (rc = ensuref(ctx, h->w32, nl)) || (rc = ensuref(ctx, h->z32, nl)) || (rc = ensuref(ctx, h->v2_32, nl))))
        return rc;
      const double inner_tol = o->inner_tolerance > 0 ? o->inner_tolerance : 1e-4;
      const int max_outer = o->max_outer > 0 ? o->max_outer : 30;
      double rn = r0;
      int outer = 0, total = 0;
      R.ioerr = (r0 < o->tolerance) ? 0 : -1;
      if (resi) resi[0] = r0;
      while (outer < max_outer && rn / r0 >= o->tolerance && total < o->maxIters) {
        outer++;
        int it_in = 0;
        double rel_in = 0;
        if (use_cpt) {  // compact layout: r32 = the unknowns of r64, x += d at the primary copies
          auto& Cp = h->cpt;
          compact_gather<float><<<h->nblk, kRedThreads, 0, ctx->stream>>>(Cp.f32.r.p, h->r.p, Cp.cl.p, Cp.ng, Cp.ngp);
          SELF_LAUNCHED(ctx);
          SELF_CUDA_TRY(ctx, cudaMemsetAsync(Cp.f32.u.p, 0, (size_t)Cp.ngp * sizeof(float), ctx->stream));
          const int inner_err = pcg_device_compact<float>(h, jac, o->maxIters - total, inner_tol, rn, nullptr, false,
                                                          &it_in, &rel_in);
          total += it_in;
          if (inner_err == SELF_ERR_TIMEOUT)
            return set_error(ctx, SELF_ERR_TIMEOUT, "FP32 inner solve: a staged-copy barrier wait ran out");
          compact_scatter_add<float><<<h->nblk, kRedThreads, 0, ctx->stream>>>(h->u.p, Cp.f32.u.p, Cp.cl.p, Cp.ng);
          SELF_LAUNCHED(ctx);
        } else {
          convert<float, double><<<h->nblk, kRedThreads, 0, ctx->stream>>>(h->r32.p, h->r.p, nl);
          SELF_LAUNCHED(ctx);
          SELF_CUDA_TRY(ctx, cudaMemsetAsync(h->u32.p, 0, nl * sizeof(float), ctx->stream));
          const PcRun<float> pc = use_pcl ? pcl_run<float>(h, o->pc_iterations) : PcRun<float>{};
          const int inner_err = pcg_device<float>(h, h->u32.p, h->r32.p, h->v32.p, h->w32.p, h->z32.p,
                                                  jac ? h->op32.dinv.p : nullptr, o->maxIters - total, inner_tol, rn,
                                                  nullptr, &it_in, &rel_in, h->op32, false, use_pcl ? &pc : nullptr);
          total += it_in;
          if (inner_err == SELF_ERR_TIMEOUT) {  // a bounded tensor-core wait ran out in the inner solve
            h->tc = 0;
            return set_error(ctx, SELF_ERR_TIMEOUT, "FP32 inner solve: a tensor-core barrier wait ran out");
          }
          // x += d (FP64)
          convert<double, float><<<h->nblk, kRedThreads, 0, ctx->stream>>>(h->z.p, h->u32.p, nl);
          SELF_LAUNCHED(ctx);
          axpby<double><<<h->nblk, kRedThreads, 0, ctx->stream>>>(h->u.p, h->z.p, 1.0, 1.0, nl);
          SELF_LAUNCHED(ctx);
        }
        // r = b - A x in FP64
        if ((rc = residual<double>(h, h->f.p, h->u.p, h->r.p, h->op64))) return rc;
        if ((rc = dots<double>(h, h->r.p, h->r.p, nullptr, nullptr, h->red.p))) return rc;
        rn = std::sqrt(read1(h, h->red.p, &rc));
        if (rc) return rc;
        if (resi && outer <= o->maxIters) resi[outer] = rn;
        if (!(rn == rn)) {
          R.ioerr = SELF_ERR_NONFINITE;
          break;
        }
        if (it_in == 0) break;
      }
      h->tc = 0;
      iters = total;
      rel = rn / r0;
      R.outer_iterations = outer;
      if (R.ioerr != SELF_ERR_NONFINITE) R.ioerr = (rel < o->tolerance) ? 0 : -1;
    }
  }
  // UnMask the solution and restore the Dirichlet values
  if ((rc = unmask_dev<double>(h, h->w.p, h->u.p))) return rc;
  if ((rc = download_vec(h, solution, h->w.p))) return rc;
  set_dirichlet_host(h, solution, dirichlet);
  R.iterations = iters;
  R.r0 = r0;
  R.rel_residual = rel;
  if (rep) *rep = R;
  if (R.ioerr == SELF_ERR_NONFINITE) return set_error(ctx, SELF_ERR_NONFINITE, "non-finite residual");
  return SELF_OK;
}

int self_cg2d_precondition(self_cg2d* h, const self_solve_opts* o, const double* r, double* w, int* iterations) {
  if (!h || !o || !r || !w) return SELF_ERR_INVALID;
  self_ctx* ctx = h->ctx;
  SELF_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  if (o->pc_iterations < 0 || !(o->pc_tolerance >= 0))
    return set_error(ctx, SELF_ERR_INVALID, "preconditioner iterations %d / tolerance %g", o->pc_iterations,
                     o->pc_tolerance);
  int rc;
  if ((rc = upload_vec(h, h->r, r)) || (rc = ensure(ctx, h->w, h->nl))) return rc;
  if ((rc = mask_dev<double>(h, h->r.p))) return rc;
  int its = 0;
  if (o->pc_iterations == 0) {  // u = r
    if ((rc = unmask_dev<double>(h, h->w.p, h->r.p))) return rc;
  } else {
    if ((rc = pcl_ensure(h, false, o->pc_nodes)) || (rc = pcl_limits(h, o->pc_iterations, o->pc_tolerance)))
      return rc;
    CGScalars hs{};  // outer scalars: not done, so the preconditioner kernels run
    SELF_CUDA_TRY(ctx, cudaMemcpyAsync(h->S.p, &hs, sizeof(hs), cudaMemcpyHostToDevice, ctx->stream));
    const PcRun<double> pc = pcl_run<double>(h, o->pc_iterations);
    if ((rc = pc_linear_apply<double>(h, h->r.p, pc))) return rc;
    cg_unmask<double><<<h->nblk, kRedThreads, 0, ctx->stream>>>(h->w.p, pc.ul, pc.src, h->nl);  // linear UnMask
    SELF_LAUNCHED(ctx);
    CGScalars sl{};
    SELF_CUDA_TRY(ctx, cudaMemcpyAsync(&sl, h->pcl.SL.p, sizeof(sl), cudaMemcpyDeviceToHost, ctx->stream));
    SELF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    its = sl.iter;
  }
  if ((rc = download_vec(h, w, h->w.p))) return rc;
  if (iterations) *iterations = its;
  return SELF_OK;
}

}  // extern "C"

namespace selfgpu {
namespace cg {

int compile_host(self_ctx* ctx, const self_cg2d_desc* d, HostCompiled& out) {
  if (!d || d->N < 2 || d->N > 9 || d->nEl < 1 || d->op != 0)
    return set_error(ctx, SELF_ERR_INVALID, "batched problems: Helmholtz operator, N in 2..9");
  self_cg2d h;
  h.ctx = ctx;
  h.upload_dev = false;
  h.N = d->N;
  h.n = d->N + 1;
  h.nEl = d->nEl;
  h.nEdges = d->nEdges;
  h.nNodes = d->nNodes;
  h.op = 0;
  h.nf = 4;
  h.lambda = d->lambda;
  h.nl = (size_t)h.n * h.n * h.nEl;
  int rc = compile_topology(&h, d);
  if (rc) return rc;
  std::vector<double> Jww;
  if ((rc = build_factors(&h, d, Jww))) return rc;
  out.N = h.N;
  out.n = h.n;
  out.nEl = h.nEl;
  out.ngroups = h.ngroups;
  out.nl = h.nl;
  out.src = std::move(h.h_src);
  out.gptr = std::move(h.h_gptr);
  out.gidx = std::move(h.h_gidx);
  out.gdir = std::move(h.h_gdir);
  out.fac = std::move(h.h_fac);
  out.dinv = std::move(h.h_dinv);
  out.Jww = std::move(Jww);
  out.D.assign(d->dmat, d->dmat + (size_t)h.n * h.n);
  return SELF_OK;
}

}  // namespace cg
}  // namespace selfgpu
