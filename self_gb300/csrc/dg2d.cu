// DGSEM 2-D tendency and low-storage RK3 on sm_103a (plain FP64 form).
//
// Replaces, on the GPU, the per-stage work of ConservativeShallowWaterClass.f90 and
// AdvectionClass.f90: CalculateSolutionAtBoundaries (DGSEMSolutionStorageClass_2D.f90:749-802),
// EdgeFlux with the LLF / upwind Riemann solvers (:1266-1360, :1555-1604; Advection :1382-1478,
// :1756-1787), MappedTimeDerivative with XFlux/YFlux, DGSystemDerivative and Source (:1364-1551,
// :1608-1694) and the RK3 register update of ForwardStepRK3 (:1173-1218).
//
// One RK stage is two kernels:
//   dg_edge_flux   one thread per (edge, edge node): both traces, Riemann flux x |n|, written to
//                  the primary side and (negated, through start/inc) to the secondary side;
//   dg_volume      one thread per element node, several elements per CTA: contravariant fluxes
//                  into shared memory, the two 1-D weak-derivative contractions, lift, 1/J, source,
//                  G <- a G + dq/dt, q <- q + g dt G, then the boundary traces of the new q for
//                  the next stage's edge kernel (the trace pass is fused into this epilogue).
// Layout in HBM: E-vectors q, G (element-contiguous, i fastest); per element a 5 n^2 metric block
// (dxds, dxdp, dyds, dydp, 1/J); per element an aux block (dhdx, dhdy, f [, h] [, relaxation]);
// traces and boundary fluxes (i, v, side, e); per edge a 4 n block (nx, ny, |n|, u.n).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <memory>
#include <vector>

#include "dg2d_fp32.cuh"
#include "internal.hpp"
#include "line_ops.cuh"

using namespace selfgpu;

namespace selfgpu {
namespace dg {

__constant__ double c_rk3_a[3] = {0.0, -5.0 / 9.0, -153.0 / 128.0};

template <int N1>
struct NodalConst {
  double dS[N1 * N1];  // weak-derivative matrix, s direction, column major
  double dP[N1 * N1];  // p direction
  double lW[N1], lE[N1], lS[N1], lN[N1];
  double qwinv[N1];  // 1 / quadrature weight
  double qw[N1];     // quadrature weight (bit-faithful mode divides)
  double lWq[N1], lEq[N1], lSq[N1], lNq[N1];  // lifts over the weight, lX(k) / w(k) (plain mode)
  EOTable<N1> eS, eP;  // even-odd tables of dS, dP (plain mode, when eo)
  int eo;              // both matrices centro-antisymmetric
};

struct VolArgs {
  const double* q;
  double* qout;
  double* G;
  double* tend;  // tendency output (mode 0)
  const double* bf;
  double* bs;  // traces of the new state (write_traces)
  const double* metrics;
  const double* aux;
  int nEl, naux, has_drag, has_relax;
  double g, drag, a, gdt;
  int mode;  // 0 tendency only, 1 RK stage with a = 0 (G not read), 2 RK stage reading G
  int write_traces;
  const double *gx, *gy;  // advection with kappa > 0: concentration gradient (i, j, v, e), else null
  double kappa;
};

struct EdgeArgs {
  const double* bs;
  double* bf;
  const int* edges;     // 6 per edge
  const double* egeo;   // 4 n per edge: nx, ny, |n|, u.n (advection) or the edge depth (linear / skew SW)
  const double* eplan;  // skew SW: 2 n per edge, planetary vorticity traces of the primary and secondary side
  const double *gtx, *gty;  // advection with kappa > 0: traces of the concentration gradient, else null
  double kappa;
  int nEdges;
  double g, t;
  double sg;  // sqrt(g) (correctly rounded on the host, as on the device)
};

// ------------------------------------------------------------------------------------ arithmetic
// EX = true is the bit-faithful FP64 mode: no FMA contraction (__dmul_rn/__dadd_rn), true divisions by J, H
// and the quadrature weights, and the reference's statement order, so the result equals the Fortran-order
// CPU restatement bit for bit.  EX = false lets the compiler contract and uses precomputed reciprocals.
template <bool EX>
struct Ar {
  static __device__ __forceinline__ double mul(double a, double b) { return EX ? __dmul_rn(a, b) : a * b; }
  static __device__ __forceinline__ double add(double a, double b) { return EX ? __dadd_rn(a, b) : a + b; }
  static __device__ __forceinline__ double sub(double a, double b) { return EX ? __dsub_rn(a, b) : a - b; }
};

// ------------------------------------------------------------------------------------ physics
struct SWFlux {
  template <int NEQ, bool EX>
  static __device__ __forceinline__ void riemann(const double* in, const double* ex, double nx, double ny,
                                                 double un_adv, double fin, double fout, double g, double sg, double* f) {
    (void)fin;
    (void)fout;
    (void)un_adv;
    // RiemannSolver (ConservativeShallowWaterClass.f90:1555-1604), g taken from the parameters
    using A = Ar<EX>;
    const double uL = in[0], vL = in[1], pL = in[2];
    const double uR = ex[0], vR = ex[1], pR = ex[2];
    const double uOut = A::add(A::mul(uR, nx), A::mul(vR, ny));
    const double uIn = A::add(A::mul(uL, nx), A::mul(vL, ny));
    if (EX) {
      const double oR = uOut / pR, oL = uIn / pL;
      const double cR = sqrt(A::mul(g, pR)), cL = sqrt(A::mul(g, pL));
      const double fac =
          fmax(fmax(fmax(fabs(A::add(oR, cR)), fabs(A::sub(oR, cR))), fabs(A::add(oL, cL))), fabs(A::sub(oL, cL)));
      const double hgR = A::mul(A::mul(A::mul(0.5, g), pR), pR), hgL = A::mul(A::mul(A::mul(0.5, g), pL), pL);
      const double a0 = A::add(A::add(A::add(A::mul(oR, uR), A::mul(hgR, nx)), A::mul(oL, uL)), A::mul(hgL, nx));
      const double a1 = A::add(A::add(A::add(A::mul(oR, vR), A::mul(hgR, ny)), A::mul(oL, vL)), A::mul(hgL, ny));
      const double a2 = A::add(uOut, uIn);
      f[0] = A::mul(0.5, A::sub(a0, A::mul(fac, A::sub(uR, uL))));
      f[1] = A::mul(0.5, A::sub(a1, A::mul(fac, A::sub(vR, vL))));
      f[2] = A::mul(0.5, A::sub(a2, A::mul(fac, A::sub(pR, pL))));
    } else {
      // depths are positive: one reciprocal square root per side gives 1/H and sqrt(g H) = sqrt(g) H / sqrt(H)
      const double rR = rsqrt(pR), rL = rsqrt(pL);  // sg = sqrt(g), formed once on the host
      const double ipR = rR * rR, ipL = rL * rL;
      const double cR = sg * (pR * rR), cL = sg * (pL * rL);
      const double wR = uOut * ipR, wL = uIn * ipL;
      const double fac = fmax(fmax(fabs(wR + cR), fabs(wR - cR)), fmax(fabs(wL + cL), fabs(wL - cL)));
      const double a0 = wR * uR + 0.5 * g * pR * pR * nx + wL * uL + 0.5 * g * pL * pL * nx;
      const double a1 = wR * vR + 0.5 * g * pR * pR * ny + wL * vL + 0.5 * g * pL * pL * ny;
      const double a2 = uOut + uIn;
      f[0] = 0.5 * (a0 - fac * (uR - uL));
      f[1] = 0.5 * (a1 - fac * (vR - vL));
      f[2] = 0.5 * (a2 - fac * (pR - pL));
    }
  }
  template <int NEQ, bool EX>
  static __device__ __forceinline__ void external(int bc, double nx, double ny, double t, const double* in,
                                                  double* ex) {
    (void)t;
    using A = Ar<EX>;
    if (bc == SELF_NO_NORMAL_FLOW) {  // GetExternalState (:1698-1729)
      const double c = A::mul(A::mul(2.0, nx), ny);
      ex[0] = A::sub(A::mul(A::sub(A::mul(ny, ny), A::mul(nx, nx)), in[0]), A::mul(c, in[1]));
      ex[1] = A::sub(A::mul(A::sub(A::mul(nx, nx), A::mul(ny, ny)), in[1]), A::mul(c, in[0]));
      ex[2] = in[2];
    } else {
      ex[0] = ex[1] = ex[2] = 0.0;
    }
  }
};

// LINEAR formulation of ShallowWaterClass (state u, v, eta); `depth` is the edge depth HALF*(inBathy + exBathy)
// (interior) or inBathy (boundary), precomputed per edge node from the bathymetry traces.
struct SWLinFlux {
  template <int NEQ, bool EX>
  static __device__ __forceinline__ void riemann(const double* in, const double* ex, double nx, double ny,
                                                 double depth, double fin, double fout, double g, double sg, double* f) {
    (void)fin;
    (void)fout;
    // RiemannSolver, LINEAR branch (ShallowWaterClass.f90:2106-2113)
    using A = Ar<EX>;
    const double uOut = A::add(A::mul(ex[0], nx), A::mul(ex[1], ny));
    const double uIn = A::add(A::mul(in[0], nx), A::mul(in[1], ny));
    const double fac = sqrt(A::mul(g, depth));
    const double m = A::mul(0.5, A::add(A::mul(g, A::add(ex[2], in[2])), A::mul(fac, A::sub(uIn, uOut))));
    f[0] = A::mul(m, nx);
    f[1] = A::mul(m, ny);
    f[2] = A::mul(0.5, A::add(A::mul(depth, A::add(uIn, uOut)), A::mul(fac, A::sub(in[2], ex[2]))));
  }
  template <int NEQ, bool EX>
  static __device__ __forceinline__ void external(int bc, double nx, double ny, double t, const double* in,
                                                  double* ex) {
    SWFlux::external<NEQ, EX>(bc, nx, ny, t, in, ex);  // GetExternalState (:2298-2325): the same mirror
  }
};

// SKEW_SYMMETRIC formulation of ShallowWaterClass with the relative vorticity as the 4th variable (u, v, eta,
// zeta): the skew-symmetric flux for the first three and VorticityFluxSolver for zeta, with zIn = zeta_in + f_in,
// zOut = zeta_out + f_out (f_out = f_in on the boundary, RelativeVorticityEdgeFlux :1628-1724).
struct SWSkewFlux {
  template <int NEQ, bool EX>
  static __device__ __forceinline__ void riemann(const double* in, const double* ex, double nx, double ny,
                                                 double depth, double fin, double fout, double g, double sg, double* f) {
    // RiemannSolver, SKEW_SYMMETRIC branch (ShallowWaterClass.f90:2114-2133)
    using A = Ar<EX>;
    const double uL = in[0], vL = in[1], pL = in[2], uR = ex[0], vR = ex[1], pR = ex[2];
    const double uOut = A::add(A::mul(uR, nx), A::mul(vR, ny));
    const double uIn = A::add(A::mul(uL, nx), A::mul(vL, ny));
    const double g16 = A::mul(16.0, g);
    const double sR = sqrt(A::add(A::mul(uOut, uOut), A::mul(g16, A::add(pR, depth))));
    const double sL = sqrt(A::add(A::mul(uIn, uIn), A::mul(g16, A::add(pL, depth))));
    const double fac = fmax(fmax(fmax(fabs(A::mul(0.25, A::add(uOut, sR))), fabs(A::mul(0.25, A::sub(uOut, sR)))),
                                 fabs(A::mul(0.25, A::add(uIn, sL)))),
                            fabs(A::mul(0.25, A::sub(uIn, sL))));
    const double e = A::add(A::add(A::add(A::mul(0.5, A::add(A::mul(uR, uR), A::mul(vR, vR))), A::mul(g, pR)),
                                   A::mul(0.5, A::add(A::mul(uL, uL), A::mul(vL, vL)))),
                            A::mul(g, pL));
    const double a2 = A::add(A::mul(uIn, A::add(pL, depth)), A::mul(uOut, A::add(pR, depth)));
    f[0] = A::mul(0.5, A::sub(A::mul(e, nx), A::mul(fac, A::sub(uR, uL))));
    f[1] = A::mul(0.5, A::sub(A::mul(e, ny), A::mul(fac, A::sub(vR, vL))));
    f[2] = A::mul(0.5, A::sub(a2, A::mul(fac, A::sub(pR, pL))));
    // VorticityFluxSolver (:2041-2068)
    const double zIn = A::add(in[3], fin), zOut = A::add(ex[3], fout);
    f[3] = A::mul(0.5, A::sub(A::add(A::mul(uOut, zOut), A::mul(uIn, zIn)),
                              A::mul(fmax(fabs(uOut), fabs(uIn)), A::sub(zOut, zIn))));
  }
  template <int NEQ, bool EX>
  static __device__ __forceinline__ void external(int bc, double nx, double ny, double t, const double* in,
                                                  double* ex) {
    SWFlux::external<NEQ, EX>(bc, nx, ny, t, in, ex);
    ex[3] = bc == SELF_NO_NORMAL_FLOW ? in[3] : 0.0;  // GetExternalVorticity (:2329-2356)
  }
};

struct AdvFlux {
  template <int NEQ, bool EX>
  static __device__ __forceinline__ void riemann(const double* in, const double* ex, double nx, double ny,
                                                 double un, double fin, double fout, double g, double sg, double* f) {
    (void)fin;
    (void)fout;
    (void)nx;
    (void)ny;
    (void)g;
    using A = Ar<EX>;
    // RiemannSolver (AdvectionClass.f90:1756-1787) with kappa = 0
#pragma unroll
    for (int v = 0; v < NEQ; ++v)
      f[v] = A::mul(0.5, A::sub(A::mul(un, A::add(ex[v], in[v])), A::mul(fabs(un), A::sub(ex[v], in[v]))));
  }
  template <int NEQ, bool EX>
  static __device__ __forceinline__ void external(int bc, double nx, double ny, double t, const double* in,
                                                  double* ex) {
    (void)nx;
    (void)ny;
    (void)in;
#pragma unroll
    for (int v = 0; v < NEQ; ++v) ex[v] = 0.0;  // GetExternalState (:1851-1886)
    if (bc == SELF_INFLOW_ONE) ex[0] = tanh(t);
    if (NEQ > 1 && bc == SELF_INFLOW_TWO) ex[NEQ > 1 ? 1 : 0] = tanh(t);
  }
};

// ------------------------------------------------------------------------------------ edge kernel
template <int N1, int NEQ, class Phys, bool EX>
__global__ void __launch_bounds__(256) dg_edge_flux(EdgeArgs A) {
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = gid / N1;
  const int i = gid - k * N1;
  if (k >= A.nEdges) return;
  const int* E = A.edges + 6 * k;
  const int e1 = E[0] - 1, s1 = E[1] - 1, e2f = E[2];
  const double* eg = A.egeo + (size_t)k * 4 * N1;
  const double nx = eg[i], ny = eg[N1 + i], len = eg[2 * N1 + i], un = eg[3 * N1 + i];
  const double fin = A.eplan ? A.eplan[(size_t)k * 2 * N1 + i] : 0.0;
  const double fout = A.eplan ? A.eplan[(size_t)k * 2 * N1 + N1 + i] : 0.0;
  double in[NEQ], ex[NEQ], f[NEQ];
  const double* b1 = A.bs + (size_t)N1 * NEQ * (s1 + 4 * (size_t)e1);
#pragma unroll
  for (int v = 0; v < NEQ; ++v) in[v] = b1[i + N1 * v];
  // the exterior state (neighbour's trace or boundary condition), then one Riemann solve for both kinds of edge:
  // a warp holding interior and boundary edges does not run the solver twice
  const bool interior = e2f > 0;
  int e2 = 0, s2 = 0, kk = 0;
  if (interior) {
    const int start = E[4], inc = E[5];
    e2 = e2f - 1;
    s2 = abs(E[3]) - 1;
    kk = start - inc + i * inc;
    const double* b2 = A.bs + (size_t)N1 * NEQ * (s2 + 4 * (size_t)e2);
#pragma unroll
    for (int v = 0; v < NEQ; ++v) ex[v] = b2[kk + N1 * v];
  } else {
    Phys::template external<NEQ, EX>(e2f, nx, ny, A.t, in, ex);
  }
  Phys::template riemann<NEQ, EX>(in, ex, nx, ny, un, fin, fout, A.g, A.sg, f);
  using X = Ar<EX>;
  const size_t o1i = (size_t)N1 * NEQ * (s1 + 4 * (size_t)e1) + i;
  if (interior) {
    if (A.gtx) {  // BR1: - kappa dc/dn with the averaged gradient (AdvectionClass.f90 EdgeFlux :1413-1420)
      const size_t o2i = (size_t)N1 * NEQ * (s2 + 4 * (size_t)e2) + kk;
#pragma unroll
      for (int v = 0; v < NEQ; ++v) {
        const double gx = X::mul(X::add(A.gtx[o1i + N1 * v], A.gtx[o2i + N1 * v]), 0.5);
        const double gy = X::mul(X::add(A.gty[o1i + N1 * v], A.gty[o2i + N1 * v]), 0.5);
        f[v] = X::sub(f[v], X::mul(A.kappa, X::add(X::mul(gx, nx), X::mul(gy, ny))));
      }
    }
    double* o1 = A.bf + (size_t)N1 * NEQ * (s1 + 4 * (size_t)e1);
    double* o2 = A.bf + (size_t)N1 * NEQ * (s2 + 4 * (size_t)e2);
#pragma unroll
    for (int v = 0; v < NEQ; ++v) {
      const double fl = X::mul(f[v], len);
      o1[i + N1 * v] = fl;
      o2[kk + N1 * v] = -fl;
    }
  } else {
    if (A.gtx) {  // BR1: the inner gradient on the boundary
#pragma unroll
      for (int v = 0; v < NEQ; ++v)
        f[v] = X::sub(f[v], X::mul(A.kappa, X::add(X::mul(A.gtx[o1i + N1 * v], nx), X::mul(A.gty[o1i + N1 * v], ny))));
    }
    double* o1 = A.bf + (size_t)N1 * NEQ * (s1 + 4 * (size_t)e1);
#pragma unroll
    for (int v = 0; v < NEQ; ++v) o1[i + N1 * v] = X::mul(f[v], len);
  }
}

// ------------------------------------------------------------------------------------ volume kernel
template <int N1>
constexpr int elems_per_block() {
  return (N1 * N1 >= 256) ? 1 : (256 / (N1 * N1));
}

template <int N1, int NEQ, bool EX>
__device__ __forceinline__ void write_traces(const NodalConst<N1>& C, const double* sq /*[EPB][NEQ][N1*N1]*/,
                                             double* bs, int e, int tid) {
  // 4 sides x NEQ x N1 values per element; side 0..3 = S,E,N,W (CalculateSolutionAtBoundaries).  A thread takes a
  // pair: one column trace (S or N: along j at column k) and one row trace (E or W: along i at row k) of the same
  // variable, so a warp never splits between the two access patterns and N1 = 8 needs one round of 48 threads
  using A = Ar<EX>;
  constexpr int NP = 2 * NEQ * N1;
  for (int t = tid; t < NP; t += N1 * N1) {
    const int k = t % N1;
    const int v = (t / N1) % NEQ;
    const int hsel = t / (N1 * NEQ);  // 0: S and E, 1: N and W
    const double* Q = sq + v * N1 * N1;
    const double* Lc = hsel ? C.lN : C.lS;
    const double* Lr = hsel ? C.lW : C.lE;
    double ac = 0.0, ar = 0.0;
#pragma unroll
    for (int m = 0; m < N1; ++m) {
      ac = A::add(ac, A::mul(Lc[m], Q[k + N1 * m]));
      ar = A::add(ar, A::mul(Lr[m], Q[m + N1 * k]));
    }
    const int sc = hsel ? 2 : 0, sr = hsel ? 3 : 1;
    bs[(size_t)N1 * NEQ * (sc + 4 * (size_t)e) + k + N1 * v] = ac;
    bs[(size_t)N1 * NEQ * (sr + 4 * (size_t)e) + k + N1 * v] = ar;
  }
}

// Resident blocks asked of the compiler for dg_volume: the plain form is bound by the FP64 pipe and ran 11 % faster
// at N1 = 8 with 3 blocks of 256 threads per SM (80 registers, a few bytes spilled) than with 2 (86 registers); at
// other degrees that cap spills hundreds of bytes, so the compiler chooses
template <int N1, bool EX>
constexpr int vol_min_blocks() {
  return (!EX && N1 == 8) ? 3 : 1;
}

// PH: 0 advection, 1 conservative shallow water, 2 linear shallow water, 3 skew-symmetric shallow water (NEQ 4)
template <int N1, int NEQ, int PH, bool EX>
__global__ void __launch_bounds__(256, vol_min_blocks<N1, EX>()) dg_volume(VolArgs A, NodalConst<N1> Cg) {
  constexpr bool SW = PH == 1;
  using X = Ar<EX>;
  constexpr int NN = N1 * N1;
  constexpr int EPB = elems_per_block<N1>();
  __shared__ NodalConst<N1> C;
  __shared__ double sF[EPB][NEQ][NN];
  __shared__ double sG[EPB][NEQ][NN];
  __shared__ double sB[EPB][4][NEQ][N1];

  const int tid = threadIdx.x;           // node within element
  const int le = threadIdx.y;            // element within block
  const int e = blockIdx.x * EPB + le;
  const bool active = e < A.nEl;
  {
    const int flat = tid + NN * le;
    constexpr int NC = sizeof(NodalConst<N1>) / sizeof(double);
    const double* src = reinterpret_cast<const double*>(&Cg);
    double* dst = reinterpret_cast<double*>(&C);
    for (int t = flat; t < NC; t += NN * EPB) dst[t] = src[t];
  }
  const int i = tid % N1, j = tid / N1;
  double qv[NEQ];
  double dxds = 0, dxdp = 0, dyds = 0, dydp = 0, jac = 0;  // jac: 1/J (fast) or J (exact)
  if (active) {
    const double* qe = A.q + (size_t)e * NEQ * NN;
#pragma unroll
    for (int v = 0; v < NEQ; ++v) qv[v] = qe[v * NN + tid];
    const double* me = A.metrics + (size_t)e * 5 * NN;
    dxds = me[tid];
    dxdp = me[NN + tid];
    dyds = me[2 * NN + tid];
    dydp = me[3 * NN + tid];
    jac = me[4 * NN + tid];
    // boundary fluxes of this element into shared memory
    const double* be = A.bf + (size_t)e * 4 * NEQ * N1;
    double* sb = &sB[le][0][0][0];
    for (int t = tid; t < 4 * NEQ * N1; t += NN) sb[t] = be[t];
    double xF[NEQ], yF[NEQ];
    if (PH == 3) {
      // XFlux / YFlux, SKEW_SYMMETRIC (ShallowWaterClass.f90:2179-2187, 2226-2234) and the vorticity fluxes
      // u (zeta + f), v (zeta + f) of VorticityTimeDerivative (:1934-1936); aux = (h, f, ...)
      const double* ae = A.aux + (size_t)e * A.naux * NN;
      const double hh = ae[tid], fc = ae[NN + tid];
      const double KE = X::mul(X::add(X::mul(qv[0], qv[0]), X::mul(qv[1], qv[1])), 0.5);
      const double gp = X::add(X::mul(A.g, qv[2]), KE);
      const double H = X::add(hh, qv[2]);
      xF[0] = gp;
      xF[1] = 0.0;
      xF[2] = X::mul(H, qv[0]);
      yF[0] = 0.0;
      yF[1] = gp;
      yF[2] = X::mul(H, qv[1]);
      const double za = X::add(qv[NEQ > 3 ? 3 : 0], fc);
      xF[NEQ > 3 ? 3 : 0] = X::mul(qv[0], za);
      yF[NEQ > 3 ? 3 : 0] = X::mul(qv[1], za);
    } else if (PH == 2) {
      // XFlux / YFlux, LINEAR (ShallowWaterClass.f90:2171-2177, 2218-2224): aux = (h, f, ...)
      const double hh = A.aux[(size_t)e * A.naux * NN + tid];
      const double gp = X::mul(A.g, qv[2]);
      xF[0] = gp;
      xF[1] = 0.0;
      xF[2] = X::mul(hh, qv[0]);
      yF[0] = 0.0;
      yF[1] = gp;
      yF[2] = X::mul(hh, qv[1]);
    } else if (SW) {
      // XFlux / YFlux (:1608-1658)
      if (EX) {
        const double p = X::mul(X::mul(X::mul(A.g, 0.5), qv[2]), qv[2]);
        xF[0] = X::add(X::mul(qv[0], qv[0]) / qv[2], p);
        xF[1] = X::mul(qv[0], qv[1]) / qv[2];
        xF[2] = qv[0];
        yF[0] = X::mul(qv[1], qv[0]) / qv[2];
        yF[1] = X::add(X::mul(qv[1], qv[1]) / qv[2], p);
        yF[2] = qv[1];
      } else {
        const double iH = 1.0 / qv[2];
        const double p = A.g * 0.5 * qv[2] * qv[2];
        xF[0] = qv[0] * qv[0] * iH + p;
        xF[1] = qv[0] * qv[1] * iH;
        xF[2] = qv[0];
        yF[0] = qv[1] * qv[0] * iH;
        yF[1] = qv[1] * qv[1] * iH + p;
        yF[2] = qv[1];
      }
    } else {
      const double* ae = A.aux + (size_t)e * A.naux * NN;
      const double u = ae[tid], vv = ae[NN + tid];
#pragma unroll
      for (int v = 0; v < NEQ; ++v) {
        xF[v] = X::mul(qv[v], u);
        yF[v] = X::mul(qv[v], vv);
        if (A.gx) {  // XFlux / YFlux (AdvectionClass.f90:1790-1825): c u - kappa dc/dx, c v - kappa dc/dy
          xF[v] = X::sub(xF[v], X::mul(A.kappa, A.gx[(size_t)e * NEQ * NN + v * NN + tid]));
          yF[v] = X::sub(yF[v], X::mul(A.kappa, A.gy[(size_t)e * NEQ * NN + v * NN + tid]));
        }
      }
    }
#pragma unroll
    for (int v = 0; v < NEQ; ++v) {
      sF[le][v][tid] = X::sub(X::mul(dydp, xF[v]), X::mul(dxdp, yF[v]));
      sG[le][v][tid] = X::add(X::mul(-dyds, xF[v]), X::mul(dxds, yF[v]));
    }
  }
  __syncthreads();
  if constexpr (!EX) {
    // plain mode: the weak-derivative contractions as line tasks, one grid line of one variable per thread, in place
    // (row j of F becomes (dS F)(., j), column i of G becomes (dP G)(i, .)); with the even-odd form 3/4 of the FP64
    // operations of the node-by-node sums, the bound of this kernel.  Tasks are ordered direction-major, so a warp
    // runs one direction.
    constexpr int NT1 = EPB * NEQ * N1;  // tasks per direction
    const int flat = tid + NN * le;
    for (int task = flat; task < 2 * NT1; task += NN * EPB) {
      const int dir = task / NT1, rest = task - dir * NT1;
      const int el = rest / (NEQ * N1), v = (rest / N1) % NEQ, k = rest % N1;
      if (blockIdx.x * EPB + el >= A.nEl) continue;
      double* base = dir == 0 ? &sF[el][v][N1 * k] : &sG[el][v][k];
      const int st = dir == 0 ? 1 : N1;
      double x[N1], y[N1];
#pragma unroll
      for (int m = 0; m < N1; ++m) x[m] = base[m * st];
      if (C.eo) {
        eo_matvec<N1>(dir == 0 ? C.eS : C.eP, x, y);
      } else {
        const double* Dm = dir == 0 ? C.dS : C.dP;
#pragma unroll
        for (int r = 0; r < N1; ++r) {
          double acc = 0.0;
#pragma unroll
          for (int m = 0; m < N1; ++m) acc = fma(Dm[r + N1 * m], x[m], acc);
          y[r] = acc;
        }
      }
#pragma unroll
      for (int m = 0; m < N1; ++m) base[m * st] = y[m];
    }
    __syncthreads();
  }
  double tend[NEQ];
  if (active) {
#pragma unroll
    for (int v = 0; v < NEQ; ++v) {
      // s direction: MATMUL(dMatS, F(:,j)) + lift, along the row j; then the p direction and 1/J
      double ds = 0.0, dp = 0.0;
      if (EX) {
#pragma unroll
        for (int m = 0; m < N1; ++m) ds = X::add(ds, X::mul(C.dS[i + N1 * m], sF[le][v][m + N1 * j]));
#pragma unroll
        for (int m = 0; m < N1; ++m) dp = X::add(dp, X::mul(C.dP[j + N1 * m], sG[le][v][i + N1 * m]));
      } else {
        ds = sF[le][v][tid];
        dp = sG[le][v][tid];
      }
      if (EX) {
        ds = X::add(ds, X::add(X::mul(sB[le][1][v][j], C.lE[i]), X::mul(sB[le][3][v][j], C.lW[i])) / C.qw[i]);
        dp = X::add(dp, X::add(X::mul(sB[le][2][v][i], C.lN[j]), X::mul(sB[le][0][v][i], C.lS[j])) / C.qw[j]);
        tend[v] = X::sub(-ds, dp) / jac;
      } else {
        ds = fma(sB[le][1][v][j], C.lEq[i], fma(sB[le][3][v][j], C.lWq[i], ds));
        dp = fma(sB[le][2][v][i], C.lNq[j], fma(sB[le][0][v][i], C.lSq[j], dp));
        tend[v] = (-ds - dp) * jac;
      }
    }
    const double* ae = A.aux + (size_t)e * A.naux * NN;
    if (SW) {
      // Source (:1662-1694): ((f V + g H dh/dx) - drag U/h) - (U - relax) ts, left to right
      const double dhdx = ae[tid], dhdy = ae[NN + tid], f = ae[2 * NN + tid];
      double s0 = X::add(X::mul(f, qv[1]), X::mul(X::mul(A.g, qv[2]), dhdx));
      double s1 = X::add(X::mul(-f, qv[0]), X::mul(X::mul(A.g, qv[2]), dhdy));
      double s2 = 0.0;
      int o = 3;
      if (A.has_drag) {
        const double hh = ae[3 * NN + tid];
        if (EX) {
          s0 = X::sub(s0, X::mul(A.drag, qv[0]) / hh);
          s1 = X::sub(s1, X::mul(A.drag, qv[1]) / hh);
        } else {
          const double ih = 1.0 / hh;
          s0 -= A.drag * qv[0] * ih;
          s1 -= A.drag * qv[1] * ih;
        }
        o = 4;
      }
      if (A.has_relax) {
        const double ts = ae[(o + 3) * NN + tid];
        s0 = X::sub(s0, X::mul(X::sub(qv[0], ae[o * NN + tid]), ts));
        s1 = X::sub(s1, X::mul(X::sub(qv[1], ae[(o + 1) * NN + tid]), ts));
        s2 = -X::mul(X::sub(qv[2], ae[(o + 2) * NN + tid]), ts);
      }
      tend[0] = X::add(tend[0], s0);
      tend[1] = X::add(tend[1], s1);
      if (NEQ > 2 && A.has_relax) tend[NEQ > 2 ? 2 : 0] = X::add(tend[NEQ > 2 ? 2 : 0], s2);
    } else if (PH == 2 || PH == 3) {
      // Source, LINEAR / SKEW_SYMMETRIC (ShallowWaterClass.f90:2272-2281): (w v - drag u) - (u - relax) ts with
      // w = f + relativeFactor zeta (0 / 1); aux = (h, f, relax u, v, eta, timescale); no vorticity source
      const double f = PH == 3 ? X::add(ae[NN + tid], X::mul(1.0, qv[NEQ > 3 ? 3 : 0])) : ae[NN + tid];
      double s0 = X::mul(f, qv[1]), s1 = X::mul(-f, qv[0]), s2 = 0.0;
      if (A.has_drag) {
        s0 = X::sub(s0, X::mul(A.drag, qv[0]));
        s1 = X::sub(s1, X::mul(A.drag, qv[1]));
      }
      if (A.has_relax) {
        const double ts = ae[5 * NN + tid];
        s0 = X::sub(s0, X::mul(X::sub(qv[0], ae[2 * NN + tid]), ts));
        s1 = X::sub(s1, X::mul(X::sub(qv[1], ae[3 * NN + tid]), ts));
        s2 = -X::mul(X::sub(qv[2], ae[4 * NN + tid]), ts);
      }
      tend[0] = X::add(tend[0], s0);
      tend[1] = X::add(tend[1], s1);
      if (NEQ > 2 && A.has_relax) tend[NEQ > 2 ? 2 : 0] = X::add(tend[NEQ > 2 ? 2 : 0], s2);
    } else if (A.has_relax) {
#pragma unroll
      for (int v = 0; v < NEQ; ++v)
        tend[v] = X::add(tend[v], X::mul(X::sub(ae[(2 + v) * NN + tid], qv[v]), ae[(2 + NEQ + v) * NN + tid]));
    }
    if (A.mode == 0) {
      double* te = A.tend + (size_t)e * NEQ * NN;
#pragma unroll
      for (int v = 0; v < NEQ; ++v) te[v * NN + tid] = tend[v];
    } else {
      double* Ge = A.G + (size_t)e * NEQ * NN;
      double* qo = A.qout + (size_t)e * NEQ * NN;
#pragma unroll
      for (int v = 0; v < NEQ; ++v) {
        double g = (A.mode == 2) ? X::add(X::mul(A.a, Ge[v * NN + tid]), tend[v]) : tend[v];
        Ge[v * NN + tid] = g;
        qv[v] = X::add(qv[v], X::mul(A.gdt, g));
        qo[v * NN + tid] = qv[v];
      }
    }
  }
  if (A.write_traces) {
    __syncthreads();  // sF is reused for the new state
    if (active) {
#pragma unroll
      for (int v = 0; v < NEQ; ++v) sF[le][v][tid] = qv[v];
    }
    __syncthreads();
    if (active) write_traces<N1, NEQ, EX>(C, &sF[le][0][0], A.bs, e, tid);
  }
}

// Boundary traces of q alone (start of a run, and the tendency entry point).
template <int N1, int NEQ, bool EX>
__global__ void __launch_bounds__(256) dg_traces(const double* q, double* bs, int nEl, NodalConst<N1> Cg) {
  constexpr int NN = N1 * N1;
  constexpr int EPB = elems_per_block<N1>();
  __shared__ NodalConst<N1> C;
  __shared__ double sQ[EPB][NEQ][NN];
  const int tid = threadIdx.x, le = threadIdx.y;
  const int e = blockIdx.x * EPB + le;
  {
    const int flat = tid + NN * le;
    constexpr int NC = sizeof(NodalConst<N1>) / sizeof(double);
    const double* src = reinterpret_cast<const double*>(&Cg);
    double* dst = reinterpret_cast<double*>(&C);
    for (int t = flat; t < NC; t += NN * EPB) dst[t] = src[t];
  }
  if (e < nEl) {
#pragma unroll
    for (int v = 0; v < NEQ; ++v) sQ[le][v][tid] = q[(size_t)e * NEQ * NN + v * NN + tid];
  }
  __syncthreads();
  if (e < nEl) write_traces<N1, NEQ, EX>(C, &sQ[le][0][0], bs, e, tid);
}


// ------------------------------------------------------------------------------------ BR1 gradient passes
// Advection-diffusion with kappa > 0 (AdvectionClass.f90 GlobalTimeDerivative :1316-1378): before the edge flux
// and the volume pass of a stage, the concentration gradient is formed by the DG weak derivative of c with
// central boundary fluxes (EdgeGradientFlux :1482-1563, CalculateConcentrationGradient :1123-1264) and traced to
// the element sides (CalculateGradientAtBoundaries :1092-1104).
struct GradArgs {
  const double* q;
  const double* bs;     // traces of c
  double *bgx, *bgy;    // boundary fluxes of the gradient passes
  double *gx, *gy;      // gradient (i, j, v, e)
  double *gtx, *gty;    // its traces
  const int* edges;
  const double* egeo;
  const double* metrics;
  int nEdges, nEl;
  double t;
};

// central flux HALF*(c_in + c_ex)*n*|n| of every edge node, +/- to the two sides; outer state GetExternalState
template <int N1, int NEQ, bool EX>
__global__ void __launch_bounds__(256) dg_grad_edge(GradArgs A) {
  using X = Ar<EX>;
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = gid / N1;
  const int i = gid - k * N1;
  if (k >= A.nEdges) return;
  const int* E = A.edges + 6 * k;
  const int e1 = E[0] - 1, s1 = E[1] - 1, e2f = E[2];
  const double* eg = A.egeo + (size_t)k * 4 * N1;
  const double nx = eg[i], ny = eg[N1 + i], len = eg[2 * N1 + i];
  const size_t b1 = (size_t)N1 * NEQ * (s1 + 4 * (size_t)e1) + i;
  size_t b2 = 0;
  if (e2f > 0) {
    const int kk = E[4] - E[5] + i * E[5];
    b2 = (size_t)N1 * NEQ * (abs(E[3]) - 1 + 4 * (size_t)(e2f - 1)) + kk;
  }
#pragma unroll
  for (int v = 0; v < NEQ; ++v) {
    const double in = A.bs[b1 + N1 * v];
    double ex = 0.0;
    if (e2f > 0) {
      ex = A.bs[b2 + N1 * v];
    } else {
      if (e2f == SELF_INFLOW_ONE && v == 0) ex = tanh(A.t);
      if (e2f == SELF_INFLOW_TWO && v == 1) ex = tanh(A.t);
    }
    const double avg = X::mul(0.5, X::add(in, ex));
    const double fx = X::mul(X::mul(avg, nx), len), fy = X::mul(X::mul(avg, ny), len);
    A.bgx[b1 + N1 * v] = fx;
    A.bgy[b1 + N1 * v] = fy;
    if (e2f > 0) {
      A.bgx[b2 + N1 * v] = -fx;
      A.bgy[b2 + N1 * v] = -fy;
    }
  }
}

// gradient of c per element and variable (s direction with the west/east lifts, p direction with the
// south/north lifts, divided by J), then its traces
template <int N1, int NEQ, bool EX>
__global__ void __launch_bounds__(256) dg_grad_volume(GradArgs A, NodalConst<N1> Cg) {
  using X = Ar<EX>;
  constexpr int NN = N1 * N1;
  constexpr int EPB = elems_per_block<N1>();
  __shared__ NodalConst<N1> C;
  __shared__ double s1x[EPB][NN], s1y[EPB][NN], s2x[EPB][NN], s2y[EPB][NN];
  __shared__ double sBx[EPB][4][N1], sBy[EPB][4][N1];
  const int tid = threadIdx.x, le = threadIdx.y;
  const int e = blockIdx.x * EPB + le;
  const bool active = e < A.nEl;
  {
    const int flat = tid + NN * le;
    constexpr int NC = sizeof(NodalConst<N1>) / sizeof(double);
    const double* src = reinterpret_cast<const double*>(&Cg);
    double* dst = reinterpret_cast<double*>(&C);
    for (int t = flat; t < NC; t += NN * EPB) dst[t] = src[t];
  }
  const int i = tid % N1, j = tid / N1;
  double dxds = 0, dxdp = 0, dyds = 0, dydp = 0, jac = 0;
  if (active) {
    const double* me = A.metrics + (size_t)e * 5 * NN;
    dxds = me[tid];
    dxdp = me[NN + tid];
    dyds = me[2 * NN + tid];
    dydp = me[3 * NN + tid];
    jac = me[4 * NN + tid];
  }
  for (int v = 0; v < NEQ; ++v) {
    __syncthreads();  // the previous variable is done with the scratch arrays
    if (active) {
      const double c = A.q[(size_t)e * NEQ * NN + v * NN + tid];
      s1x[le][tid] = X::sub(X::mul(dydp, c), X::mul(dxdp, 0.0));
      s1y[le][tid] = X::sub(X::mul(dydp, 0.0), X::mul(dxdp, c));
      s2x[le][tid] = X::add(X::mul(-dyds, c), X::mul(dxds, 0.0));
      s2y[le][tid] = X::add(X::mul(-dyds, 0.0), X::mul(dxds, c));
      for (int t = tid; t < 4 * N1; t += NN) {
        const int side = t / N1, kq = t - side * N1;
        const size_t b = (size_t)N1 * NEQ * (side + 4 * (size_t)e) + kq + N1 * v;
        sBx[le][side][kq] = A.bgx[b];
        sBy[le][side][kq] = A.bgy[b];
      }
    }
    __syncthreads();
    double gx = 0.0, gy = 0.0;
    if (active) {
      double ax = 0.0, ay = 0.0, bx = 0.0, by = 0.0;
#pragma unroll
      for (int m = 0; m < N1; ++m) {
        ax = X::add(ax, X::mul(C.dS[i + N1 * m], s1x[le][m + N1 * j]));
        ay = X::add(ay, X::mul(C.dS[i + N1 * m], s1y[le][m + N1 * j]));
      }
#pragma unroll
      for (int m = 0; m < N1; ++m) {
        bx = X::add(bx, X::mul(C.dP[j + N1 * m], s2x[le][i + N1 * m]));
        by = X::add(by, X::mul(C.dP[j + N1 * m], s2y[le][i + N1 * m]));
      }
      if (EX) {
        ax = X::add(ax, X::add(X::mul(sBx[le][1][j], C.lE[i]), X::mul(sBx[le][3][j], C.lW[i])) / C.qw[i]);
        ay = X::add(ay, X::add(X::mul(sBy[le][1][j], C.lE[i]), X::mul(sBy[le][3][j], C.lW[i])) / C.qw[i]);
        bx = X::add(bx, X::add(X::mul(sBx[le][2][i], C.lN[j]), X::mul(sBx[le][0][i], C.lS[j])) / C.qw[j]);
        by = X::add(by, X::add(X::mul(sBy[le][2][i], C.lN[j]), X::mul(sBy[le][0][i], C.lS[j])) / C.qw[j]);
        gx = X::add(ax, bx) / jac;
        gy = X::add(ay, by) / jac;
      } else {
        ax += (sBx[le][1][j] * C.lE[i] + sBx[le][3][j] * C.lW[i]) * C.qwinv[i];
        ay += (sBy[le][1][j] * C.lE[i] + sBy[le][3][j] * C.lW[i]) * C.qwinv[i];
        bx += (sBx[le][2][i] * C.lN[j] + sBx[le][0][i] * C.lS[j]) * C.qwinv[j];
        by += (sBy[le][2][i] * C.lN[j] + sBy[le][0][i] * C.lS[j]) * C.qwinv[j];
        gx = (ax + bx) * jac;
        gy = (ay + by) * jac;
      }
      A.gx[(size_t)e * NEQ * NN + v * NN + tid] = gx;
      A.gy[(size_t)e * NEQ * NN + v * NN + tid] = gy;
    }
    __syncthreads();  // the contravariant arrays are read; they now hold the gradient for the traces
    if (active) {
      s1x[le][tid] = gx;
      s1y[le][tid] = gy;
    }
    __syncthreads();
    if (active) {
      for (int t = tid; t < 4 * N1; t += NN) {
        const int side = t / N1, kq = t - side * N1;
        double accx = 0.0, accy = 0.0;
        if (side == 0 || side == 2) {
          const double* L = (side == 0) ? C.lS : C.lN;
#pragma unroll
          for (int m = 0; m < N1; ++m) {
            accx = X::add(accx, X::mul(L[m], s1x[le][kq + N1 * m]));
            accy = X::add(accy, X::mul(L[m], s1y[le][kq + N1 * m]));
          }
        } else {
          const double* L = (side == 1) ? C.lE : C.lW;
#pragma unroll
          for (int m = 0; m < N1; ++m) {
            accx = X::add(accx, X::mul(L[m], s1x[le][m + N1 * kq]));
            accy = X::add(accy, X::mul(L[m], s1y[le][m + N1 * kq]));
          }
        }
        const size_t b = (size_t)N1 * NEQ * (side + 4 * (size_t)e) + kq + N1 * v;
        A.gtx[b] = accx;
        A.gty[b] = accy;
      }
    }
  }
}
}  // namespace dg
}  // namespace selfgpu

// ====================================================================================== handle
struct self_dg2d {
  self_ctx* ctx = nullptr;
  int N = 0, n = 0, nEl = 0, nEdges = 0, nEq = 0, model = 0, precision = 0;
  int naux = 0, has_drag = 0, has_relax = 0, has_inflow = 0;
  double g = 9.81, drag = 0.0, dt = 0.0, kappa = 0.0;
  std::vector<double> dS, dP, lW, lE, lS, lN, qw;
  DevBuf<double> q, G, bs, bf, metrics, aux, egeo, eplan, tend;
  DevBuf<double> gx, gy, gtx, gty, bgx, bgy;  // advection with kappa > 0: BR1 gradient, traces, boundary fluxes
  DevBuf<int> edges;
  bool traces_valid = false;
  cudaGraphExec_t step_graph = nullptr;
  long long step_graph_launches = 0;  // kernels in the captured step graph
  selfgpu::dg32::State* f32 = nullptr;  // FP32 form
  ~self_dg2d() {
    if (step_graph) cudaGraphExecDestroy(step_graph);
    if (f32) selfgpu::dg32::destroy(f32);
  }
};

namespace {

using namespace selfgpu::dg;

template <int N1>
NodalConst<N1> make_const(const self_dg2d* h) {
  NodalConst<N1> C;
  for (int k = 0; k < N1 * N1; ++k) {
    C.dS[k] = h->dS[k];
    C.dP[k] = h->dP[k];
  }
  for (int k = 0; k < N1; ++k) {
    C.lW[k] = h->lW[k];
    C.lE[k] = h->lE[k];
    C.lS[k] = h->lS[k];
    C.lN[k] = h->lN[k];
    C.qwinv[k] = 1.0 / h->qw[k];
    C.qw[k] = h->qw[k];
    C.lWq[k] = h->lW[k] / h->qw[k];
    C.lEq[k] = h->lE[k] / h->qw[k];
    C.lSq[k] = h->lS[k] / h->qw[k];
    C.lNq[k] = h->lN[k] / h->qw[k];
  }
  C.eo = eo_table<N1>(h->dS.data(), false, C.eS) && eo_table<N1>(h->dP.data(), false, C.eP);
  return C;
}

template <int N1, int NEQ, int PH, bool EX>
int launch_edge_t(self_dg2d* h, double t) {
  self_ctx* ctx = h->ctx;
  cudaStream_t st = ctx->stream;
  EdgeArgs EA;
  EA.bs = h->bs.p;
  EA.bf = h->bf.p;
  EA.edges = h->edges.p;
  EA.egeo = h->egeo.p;
  EA.eplan = h->eplan.p;
  const bool br1 = PH == 0 && h->kappa != 0.0;
  EA.gtx = br1 ? h->gtx.p : nullptr;
  EA.gty = br1 ? h->gty.p : nullptr;
  EA.kappa = h->kappa;
  EA.nEdges = h->nEdges;
  EA.g = h->g;
  EA.sg = std::sqrt(h->g);
  EA.t = t;
  const int nthr = h->nEdges * N1;
  if (PH == 1)
    dg_edge_flux<N1, NEQ, SWFlux, EX><<<(nthr + 255) / 256, 256, 0, st>>>(EA);
  else if (PH == 2)
    dg_edge_flux<N1, NEQ, SWLinFlux, EX><<<(nthr + 255) / 256, 256, 0, st>>>(EA);
  else if (PH == 3)
    dg_edge_flux<N1, NEQ, SWSkewFlux, EX><<<(nthr + 255) / 256, 256, 0, st>>>(EA);
  else
    dg_edge_flux<N1, NEQ, AdvFlux, EX><<<(nthr + 255) / 256, 256, 0, st>>>(EA);
  SELF_LAUNCHED(ctx);
  return SELF_OK;
}

template <int N1, int NEQ, int PH, bool EX>
int launch_volume_t(self_dg2d* h, int mode, double a, double gdt, const double* qin, double* qout, double* tend,
                    int write_traces) {
  self_ctx* ctx = h->ctx;
  cudaStream_t st = ctx->stream;
  VolArgs VA;
  VA.q = qin;
  VA.qout = qout;
  VA.G = h->G.p;
  VA.tend = tend;
  VA.bf = h->bf.p;
  VA.bs = h->bs.p;
  VA.metrics = h->metrics.p;
  VA.aux = h->aux.p;
  VA.nEl = h->nEl;
  VA.naux = h->naux;
  VA.has_drag = h->has_drag;
  VA.has_relax = h->has_relax;
  VA.g = h->g;
  VA.drag = h->drag;
  VA.a = a;
  VA.gdt = gdt;
  VA.mode = mode;
  VA.write_traces = write_traces;
  const bool br1 = PH == 0 && h->kappa != 0.0;
  VA.gx = br1 ? h->gx.p : nullptr;
  VA.gy = br1 ? h->gy.p : nullptr;
  VA.kappa = h->kappa;
  constexpr int EPB = elems_per_block<N1>();
  dim3 blk(N1 * N1, EPB);
  dg_volume<N1, NEQ, PH, EX><<<(h->nEl + EPB - 1) / EPB, blk, 0, st>>>(VA, make_const<N1>(h));
  SELF_LAUNCHED(ctx);
  return SELF_OK;
}

// BR1 gradient passes of one stage (advection with kappa > 0): central edge fluxes, then gradient + traces
template <int N1, int NEQ, bool EX>
int launch_gradient_t(self_dg2d* h, double t, const double* qin) {
  self_ctx* ctx = h->ctx;
  cudaStream_t st = ctx->stream;
  GradArgs GA;
  GA.q = qin;
  GA.bs = h->bs.p;
  GA.bgx = h->bgx.p;
  GA.bgy = h->bgy.p;
  GA.gx = h->gx.p;
  GA.gy = h->gy.p;
  GA.gtx = h->gtx.p;
  GA.gty = h->gty.p;
  GA.edges = h->edges.p;
  GA.egeo = h->egeo.p;
  GA.metrics = h->metrics.p;
  GA.nEdges = h->nEdges;
  GA.nEl = h->nEl;
  GA.t = t;
  const int nthr = h->nEdges * N1;
  dg_grad_edge<N1, NEQ, EX><<<(nthr + 255) / 256, 256, 0, st>>>(GA);
  SELF_LAUNCHED(ctx);
  constexpr int EPB = elems_per_block<N1>();
  dim3 blk(N1 * N1, EPB);
  dg_grad_volume<N1, NEQ, EX><<<(h->nEl + EPB - 1) / EPB, blk, 0, st>>>(GA, make_const<N1>(h));
  SELF_LAUNCHED(ctx);
  return SELF_OK;
}

template <int N1, int NEQ, int PH, bool EX>
int launch_stage_t(self_dg2d* h, int mode, double a, double gdt, double t, const double* qin, double* qout,
                   double* tend, int write_traces) {
  if (PH == 0 && h->kappa != 0.0) {
    const int rg = launch_gradient_t<N1, NEQ, EX>(h, t, qin);
    if (rg) return rg;
  }
  int rc = launch_edge_t<N1, NEQ, PH, EX>(h, t);
  if (rc) return rc;
  return launch_volume_t<N1, NEQ, PH, EX>(h, mode, a, gdt, qin, qout, tend, write_traces);
}

template <int N1, int NEQ, bool EX>
int launch_traces_t(self_dg2d* h, const double* q) {
  constexpr int EPB = elems_per_block<N1>();
  dim3 blk(N1 * N1, EPB);
  dg_traces<N1, NEQ, EX><<<(h->nEl + EPB - 1) / EPB, blk, 0, h->ctx->stream>>>(q, h->bs.p, h->nEl, make_const<N1>(h));
  SELF_LAUNCHED(h->ctx);
  return SELF_OK;
}

// dispatch over (N+1, nEq, model, exactness)
template <int N1, bool EX>
int stage_nx(self_dg2d* h, int mode, double a, double gdt, double t, const double* qin, double* qout, double* tend,
             int wt) {
  if (h->model == SELF_MODEL_SW_CONSERVATIVE)
    return launch_stage_t<N1, 3, 1, EX>(h, mode, a, gdt, t, qin, qout, tend, wt);
  if (h->model == SELF_MODEL_SW_LINEAR) return launch_stage_t<N1, 3, 2, EX>(h, mode, a, gdt, t, qin, qout, tend, wt);
  if (h->model == SELF_MODEL_SW_SKEW) return launch_stage_t<N1, 4, 3, EX>(h, mode, a, gdt, t, qin, qout, tend, wt);
  switch (h->nEq) {
    case 1: return launch_stage_t<N1, 1, 0, EX>(h, mode, a, gdt, t, qin, qout, tend, wt);
    case 2: return launch_stage_t<N1, 2, 0, EX>(h, mode, a, gdt, t, qin, qout, tend, wt);
    case 3: return launch_stage_t<N1, 3, 0, EX>(h, mode, a, gdt, t, qin, qout, tend, wt);
    case 4: return launch_stage_t<N1, 4, 0, EX>(h, mode, a, gdt, t, qin, qout, tend, wt);
  }
  return SELF_ERR_UNSUPPORTED;
}
template <int N1>
int stage_n(self_dg2d* h, int mode, double a, double gdt, double t, const double* qin, double* qout, double* tend,
            int wt) {
  if (h->precision == SELF_PREC_FP64_EXACT) return stage_nx<N1, true>(h, mode, a, gdt, t, qin, qout, tend, wt);
  return stage_nx<N1, false>(h, mode, a, gdt, t, qin, qout, tend, wt);
}
template <int N1, bool EX>
int edge_nx(self_dg2d* h, double t) {
  if (h->model == SELF_MODEL_SW_CONSERVATIVE) return launch_edge_t<N1, 3, 1, EX>(h, t);
  if (h->model == SELF_MODEL_SW_LINEAR) return launch_edge_t<N1, 3, 2, EX>(h, t);
  if (h->model == SELF_MODEL_SW_SKEW) return launch_edge_t<N1, 4, 3, EX>(h, t);
  switch (h->nEq) {
    case 1: return launch_edge_t<N1, 1, 0, EX>(h, t);
    case 2: return launch_edge_t<N1, 2, 0, EX>(h, t);
    case 3: return launch_edge_t<N1, 3, 0, EX>(h, t);
    case 4: return launch_edge_t<N1, 4, 0, EX>(h, t);
  }
  return SELF_ERR_UNSUPPORTED;
}
template <int N1>
int edge_n(self_dg2d* h, double t) {
  return h->precision == SELF_PREC_FP64_EXACT ? edge_nx<N1, true>(h, t) : edge_nx<N1, false>(h, t);
}
template <int N1, bool EX>
int volume_nx(self_dg2d* h, int mode, double a, double gdt, const double* qin, double* qout, double* tend, int wt) {
  if (h->model == SELF_MODEL_SW_CONSERVATIVE)
    return launch_volume_t<N1, 3, 1, EX>(h, mode, a, gdt, qin, qout, tend, wt);
  if (h->model == SELF_MODEL_SW_LINEAR) return launch_volume_t<N1, 3, 2, EX>(h, mode, a, gdt, qin, qout, tend, wt);
  if (h->model == SELF_MODEL_SW_SKEW) return launch_volume_t<N1, 4, 3, EX>(h, mode, a, gdt, qin, qout, tend, wt);
  switch (h->nEq) {
    case 1: return launch_volume_t<N1, 1, 0, EX>(h, mode, a, gdt, qin, qout, tend, wt);
    case 2: return launch_volume_t<N1, 2, 0, EX>(h, mode, a, gdt, qin, qout, tend, wt);
    case 3: return launch_volume_t<N1, 3, 0, EX>(h, mode, a, gdt, qin, qout, tend, wt);
    case 4: return launch_volume_t<N1, 4, 0, EX>(h, mode, a, gdt, qin, qout, tend, wt);
  }
  return SELF_ERR_UNSUPPORTED;
}
template <int N1>
int volume_n(self_dg2d* h, int mode, double a, double gdt, const double* qin, double* qout, double* tend, int wt) {
  if (h->precision == SELF_PREC_FP64_EXACT) return volume_nx<N1, true>(h, mode, a, gdt, qin, qout, tend, wt);
  return volume_nx<N1, false>(h, mode, a, gdt, qin, qout, tend, wt);
}
template <int N1, bool EX>
int traces_nx(self_dg2d* h, const double* q) {
  switch (h->nEq) {
    case 1: return launch_traces_t<N1, 1, EX>(h, q);
    case 2: return launch_traces_t<N1, 2, EX>(h, q);
    case 3: return launch_traces_t<N1, 3, EX>(h, q);
    case 4: return launch_traces_t<N1, 4, EX>(h, q);
  }
  return SELF_ERR_UNSUPPORTED;
}
template <int N1>
int traces_n(self_dg2d* h, const double* q) {
  return h->precision == SELF_PREC_FP64_EXACT ? traces_nx<N1, true>(h, q) : traces_nx<N1, false>(h, q);
}

#define SELF_DISPATCH_N(FN, ...)                       \
  switch (h->n) {                                      \
    case 3: return FN<3>(__VA_ARGS__);                 \
    case 4: return FN<4>(__VA_ARGS__);                 \
    case 5: return FN<5>(__VA_ARGS__);                 \
    case 6: return FN<6>(__VA_ARGS__);                 \
    case 7: return FN<7>(__VA_ARGS__);                 \
    case 8: return FN<8>(__VA_ARGS__);                 \
    case 9: return FN<9>(__VA_ARGS__);                 \
    case 10: return FN<10>(__VA_ARGS__);               \
  }                                                    \
  return SELF_ERR_UNSUPPORTED;

int launch_stage(self_dg2d* h, int mode, double a, double gdt, double t, const double* qin, double* qout,
                 double* tend, int wt) {
  SELF_DISPATCH_N(stage_n, h, mode, a, gdt, t, qin, qout, tend, wt)
}
int launch_traces(self_dg2d* h, const double* q) { SELF_DISPATCH_N(traces_n, h, q) }
int launch_edge_only(self_dg2d* h, double t) { SELF_DISPATCH_N(edge_n, h, t) }
int launch_volume_only(self_dg2d* h, int mode, double a, double gdt, const double* qin, double* qout, double* tend,
                       int wt) {
  SELF_DISPATCH_N(volume_n, h, mode, a, gdt, qin, qout, tend, wt)
}

const double kRK3a[3] = {0.0, -5.0 / 9.0, -153.0 / 128.0};
const double kRK3b[3] = {0.0, 1.0 / 3.0, 3.0 / 4.0};
const double kRK3g[3] = {1.0 / 3.0, 15.0 / 16.0, 8.0 / 15.0};

int enqueue_step(self_dg2d* h, double t0) {
  for (int m = 0; m < 3; ++m) {
    int rc = launch_stage(h, m == 0 ? 1 : 2, kRK3a[m], kRK3g[m] * h->dt, t0 + kRK3b[m] * h->dt, h->q.p, h->q.p,
                          nullptr, 1);
    if (rc) return rc;
  }
  return SELF_OK;
}

template <typename T>
int upload(self_ctx* ctx, DevBuf<T>& b, const std::vector<T>& host) {
  if (b.alloc(host.size()) != cudaSuccess) return set_error(ctx, SELF_ERR_ALLOC, "device allocation failed");
  SELF_CUDA_TRY(ctx, cudaMemcpy(b.p, host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice));
  return SELF_OK;
}

}  // namespace

namespace selfgpu {
namespace dg32 {
self_ctx* handle_ctx(self_dg2d* h) { return h->ctx; }
const int* handle_edges(self_dg2d* h) { return h->edges.p; }
// FP64 tendency of the lake at rest (U = V = 0, H = h): the reference part of the FP32 perturbation form.
int fp64_lake_tendency(const self_dg2d_desc* d, self_ctx* ctx, std::vector<double>& R0) {
  self_dg2d_desc d64 = *d;
  d64.precision = SELF_PREC_FP64;
  self_dg2d* h64 = nullptr;
  int rc = self_dg2d_create(ctx, &d64, &h64);
  if (rc) return rc;
  const size_t NN = (size_t)(d->N + 1) * (d->N + 1);
  std::vector<double> q0(NN * 3 * d->nEl, 0.0);
  for (size_t e = 0; e < (size_t)d->nEl; ++e)
    for (size_t k = 0; k < NN; ++k) q0[(e * 3 + 2) * NN + k] = d->h[e * NN + k];
  R0.assign(q0.size(), 0.0);
  rc = self_dg2d_set_state(h64, q0.data());
  if (!rc) rc = self_dg2d_tendency(h64, 0.0, R0.data());
  self_dg2d_destroy(h64);
  return rc;
}
}  // namespace dg32
}  // namespace selfgpu

extern "C" {

int self_dg2d_create(self_ctx* ctx, const self_dg2d_desc* d, self_dg2d** out) {
  if (!ctx || !d || !out) return SELF_ERR_INVALID;
  SELF_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  const int n = d->N + 1;
  if (n < 3 || n > 10) return set_error(ctx, SELF_ERR_UNSUPPORTED, "polynomial degree %d outside 2..9", d->N);
  if (d->nEl < 1 || d->nEdges < 1) return set_error(ctx, SELF_ERR_INVALID, "empty mesh");
  if (d->model == SELF_MODEL_SW_CONSERVATIVE) {
    if (d->nEq != 3) return set_error(ctx, SELF_ERR_INVALID, "shallow water needs nEq = 3");
    if (!d->h || !d->dhdx || !d->dhdy || !d->fcor) return set_error(ctx, SELF_ERR_INVALID, "missing bathymetry");
  } else if (d->model == SELF_MODEL_SW_LINEAR || d->model == SELF_MODEL_SW_SKEW) {
    if (d->nEq != (d->model == SELF_MODEL_SW_SKEW ? 4 : 3))
      return set_error(ctx, SELF_ERR_INVALID, "linear shallow water needs nEq = 3, skew-symmetric nEq = 4");
    if (!d->h || !d->fcor) return set_error(ctx, SELF_ERR_INVALID, "missing bathymetry or planetary vorticity");
  } else if (d->model == SELF_MODEL_ADVECTION) {
    if (d->nEq < 1 || d->nEq > 4) return set_error(ctx, SELF_ERR_UNSUPPORTED, "advection nEq must be 1..4");
    if (!d->u || !d->v) return set_error(ctx, SELF_ERR_INVALID, "missing velocity");
  } else {
    return set_error(ctx, SELF_ERR_INVALID, "unknown model %d", d->model);
  }
  if (d->precision != SELF_PREC_FP64 && d->precision != SELF_PREC_FP32 && d->precision != SELF_PREC_FP64_EXACT)
    return set_error(ctx, SELF_ERR_INVALID, "unknown precision");
  if (d->precision == SELF_PREC_FP32 && d->model != SELF_MODEL_SW_CONSERVATIVE && d->model != SELF_MODEL_ADVECTION)
    return set_error(ctx, SELF_ERR_UNSUPPORTED, "FP32 form");
  std::unique_ptr<self_dg2d> h(new self_dg2d());
  h->ctx = ctx;
  h->N = d->N;
  h->n = n;
  h->nEl = d->nEl;
  h->nEdges = d->nEdges;
  h->nEq = d->nEq;
  h->model = d->model;
  h->precision = d->precision;
  h->g = d->g;
  h->drag = d->linear_drag;
  h->dt = d->dt;
  h->kappa = d->kappa;
  if (d->kappa != 0.0 && (d->model != SELF_MODEL_ADVECTION || d->precision == SELF_PREC_FP32))
    return set_error(ctx, SELF_ERR_UNSUPPORTED, "kappa > 0 (BR1 diffusion): FP64 advection only");
  if (!(d->kappa >= 0.0)) return set_error(ctx, SELF_ERR_INVALID, "kappa %g", d->kappa);
  const size_t NN = (size_t)n * n, nEl = d->nEl;
  h->dS.assign(d->dmatS, d->dmatS + NN);
  h->dP.assign(d->dmatP, d->dmatP + NN);
  h->lW.assign(d->lagW, d->lagW + n);
  h->lE.assign(d->lagE, d->lagE + n);
  h->lS.assign(d->lagS, d->lagS + n);
  h->lN.assign(d->lagN, d->lagN + n);
  h->qw.assign(d->qweight, d->qweight + n);
  // edge table validation (all indices are checked here so that the kernels need no bounds tests)
  std::vector<int> ed(d->edges, d->edges + 6 * (size_t)d->nEdges);
  for (int k = 0; k < d->nEdges; ++k) {
    const int* E = &ed[6 * k];
    if (E[0] < 1 || E[0] > d->nEl || E[1] < 1 || E[1] > 4)
      return set_error(ctx, SELF_ERR_INVALID, "edge %d: bad primary element/side", k + 1);
    if (E[2] > 0) {
      if (E[2] > d->nEl || std::abs(E[3]) < 1 || std::abs(E[3]) > 4)
        return set_error(ctx, SELF_ERR_INVALID, "edge %d: bad secondary element/side", k + 1);
      int first = E[4] - E[5], last = first + d->N * E[5];
      if ((E[5] != 1 && E[5] != -1) || first < 0 || first > d->N || last < 0 || last > d->N)
        return set_error(ctx, SELF_ERR_INVALID, "edge %d: bad start/increment", k + 1);
    } else if (E[2] == SELF_INFLOW_ONE || E[2] == SELF_INFLOW_TWO) {
      h->has_inflow = 1;
    }
  }
  // metric block (dxds, dxdp, dyds, dydp, 1/J) per element
  std::vector<double> met(5 * NN * nEl);
  for (size_t e = 0; e < nEl; ++e)
    for (size_t k = 0; k < NN; ++k) {
      size_t id = e * NN + k;
      if (!(d->J[id] != 0.0)) return set_error(ctx, SELF_ERR_INVALID, "zero Jacobian in element %zu", e + 1);
      met[(e * 5 + 0) * NN + k] = d->dxds[id];
      met[(e * 5 + 1) * NN + k] = d->dxdp[id];
      met[(e * 5 + 2) * NN + k] = d->dyds[id];
      met[(e * 5 + 3) * NN + k] = d->dydp[id];
      met[(e * 5 + 4) * NN + k] = d->precision == SELF_PREC_FP64_EXACT ? d->J[id] : 1.0 / d->J[id];
    }
  // aux block
  std::vector<const double*> fields;
  h->has_relax = (d->relax && d->rfac) ? 1 : 0;
  const bool swl = d->model == SELF_MODEL_SW_LINEAR || d->model == SELF_MODEL_SW_SKEW;
  const bool sws = d->model == SELF_MODEL_SW_SKEW;
  if (d->model == SELF_MODEL_SW_CONSERVATIVE) {
    h->has_drag = d->linear_drag != 0.0 ? 1 : 0;
    fields = {d->dhdx, d->dhdy, d->fcor};
    if (h->has_drag) fields.push_back(d->h);
  } else if (swl) {
    h->has_drag = d->linear_drag != 0.0 ? 1 : 0;
    fields = {d->h, d->fcor};
  } else {
    fields = {d->u, d->v};
  }
  h->naux = (int)fields.size();
  int nrelax = 0;
  if (h->has_relax) nrelax = (d->model == SELF_MODEL_SW_CONSERVATIVE || swl) ? 4 : 2 * d->nEq;
  h->naux += nrelax;
  std::vector<double> aux((size_t)h->naux * NN * nEl);
  for (size_t e = 0; e < nEl; ++e) {
    int f = 0;
    for (const double* src : fields) {
      for (size_t k = 0; k < NN; ++k) aux[(e * h->naux + f) * NN + k] = src[e * NN + k];
      ++f;
    }
    if (h->has_relax) {
      for (int v = 0; v < (sws ? 3 : d->nEq); ++v, ++f)
        for (size_t k = 0; k < NN; ++k) aux[(e * h->naux + f) * NN + k] = d->relax[(e * d->nEq + v) * NN + k];
      if (d->model == SELF_MODEL_SW_CONSERVATIVE || swl) {
        for (size_t k = 0; k < NN; ++k) aux[(e * h->naux + f) * NN + k] = d->rfac[e * NN + k];
      } else {
        for (int v = 0; v < d->nEq; ++v, ++f)
          for (size_t k = 0; k < NN; ++k) aux[(e * h->naux + f) * NN + k] = d->rfac[(e * d->nEq + v) * NN + k];
      }
    }
  }
  // per-edge geometry: primary side normals, lengths and (advection) normal velocity or (linear shallow water)
  // the edge depth HALF*(inBathy + exBathy), inBathy on the boundary (ShallowWaterClass.f90 EdgeFlux :1530-1624)
  // from the bathymetry traces (CalculateBathymetryAtBoundaries :1357-1368, CalculateSolutionAtBoundaries order)
  auto h_trace = [&](int e, int s, int i) {
    double acc = 0.0;
    if (s == 0 || s == 2) {
      const double* L = s == 0 ? d->lagS : d->lagN;
      for (int m = 0; m < n; ++m) acc = acc + L[m] * d->h[(size_t)e * NN + i + (size_t)n * m];
    } else {
      const double* L = s == 1 ? d->lagE : d->lagW;
      for (int m = 0; m < n; ++m) acc = acc + L[m] * d->h[(size_t)e * NN + m + (size_t)n * i];
    }
    return acc;
  };
  std::vector<double> eg((size_t)4 * n * d->nEdges, 0.0), ep;
  if (sws) ep.assign((size_t)2 * n * d->nEdges, 0.0);
  auto f_trace = [&](int e, int s, int i) {  // planetary vorticity traces (CalculateVorticityAtBoundaries order)
    double acc = 0.0;
    if (s == 0 || s == 2) {
      const double* L = s == 0 ? d->lagS : d->lagN;
      for (int m = 0; m < n; ++m) acc = acc + L[m] * d->fcor[(size_t)e * NN + i + (size_t)n * m];
    } else {
      const double* L = s == 1 ? d->lagE : d->lagW;
      for (int m = 0; m < n; ++m) acc = acc + L[m] * d->fcor[(size_t)e * NN + m + (size_t)n * i];
    }
    return acc;
  };
  for (int k = 0; k < d->nEdges; ++k) {
    const int e1 = ed[6 * k] - 1, s1 = ed[6 * k + 1] - 1;
    for (int i = 0; i < n; ++i) {
      size_t ib = (size_t)i + n * (s1 + 4 * (size_t)e1);
      double nx = d->nhx[ib], ny = d->nhy[ib];
      eg[(size_t)k * 4 * n + i] = nx;
      eg[(size_t)k * 4 * n + n + i] = ny;
      eg[(size_t)k * 4 * n + 2 * n + i] = d->nlen[ib];
      if (d->model == SELF_MODEL_ADVECTION) {
        // CalculateVelocityAtBoundaries: Lagrange traces of the element velocity on side s1
        const double* L = (s1 == 0) ? d->lagS : (s1 == 1) ? d->lagE : (s1 == 2) ? d->lagN : d->lagW;
        double ub = 0.0, vb = 0.0;
        for (int m = 0; m < n; ++m) {
          size_t id = (s1 == 0 || s1 == 2) ? (size_t)e1 * NN + i + n * m : (size_t)e1 * NN + m + n * i;
          ub += L[m] * d->u[id];
          vb += L[m] * d->v[id];
        }
        eg[(size_t)k * 4 * n + 3 * n + i] = ub * nx + vb * ny;
      } else if (swl) {
        double dep = h_trace(e1, s1, i);
        if (ed[6 * k + 2] > 0) {
          const int e2 = ed[6 * k + 2] - 1, s2 = std::abs(ed[6 * k + 3]) - 1;
          const int kk = ed[6 * k + 4] - ed[6 * k + 5] + i * ed[6 * k + 5];
          dep = 0.5 * (dep + h_trace(e2, s2, kk));
        }
        eg[(size_t)k * 4 * n + 3 * n + i] = dep;
        if (sws) {
          const double fi = f_trace(e1, s1, i);
          double fo = fi;
          if (ed[6 * k + 2] > 0) {
            const int e2 = ed[6 * k + 2] - 1, s2 = std::abs(ed[6 * k + 3]) - 1;
            fo = f_trace(e2, s2, ed[6 * k + 4] - ed[6 * k + 5] + i * ed[6 * k + 5]);
          }
          ep[(size_t)k * 2 * n + i] = fi;
          ep[(size_t)k * 2 * n + n + i] = fo;
        }
      }
    }
  }
  int rc;
  if ((rc = upload(ctx, h->edges, ed))) return rc;
  if ((rc = upload(ctx, h->egeo, eg))) return rc;
  if (sws && (rc = upload(ctx, h->eplan, ep))) return rc;
  if (d->precision != SELF_PREC_FP32) {
    if ((rc = upload(ctx, h->metrics, met))) return rc;
    if ((rc = upload(ctx, h->aux, aux))) return rc;
    const size_t nq = NN * d->nEq * nEl, nb = (size_t)n * d->nEq * 4 * nEl;
    if (h->q.alloc(nq) || h->G.alloc(nq) || h->bs.alloc(nb) || h->bf.alloc(nb))
      return set_error(ctx, SELF_ERR_ALLOC, "device allocation of the state failed");
    if (h->kappa != 0.0 && (h->gx.alloc(nq) || h->gy.alloc(nq) || h->gtx.alloc(nb) || h->gty.alloc(nb) ||
                            h->bgx.alloc(nb) || h->bgy.alloc(nb)))
      return set_error(ctx, SELF_ERR_ALLOC, "device allocation of the gradient fields failed");
    SELF_CUDA_TRY(ctx, cudaMemset(h->q.p, 0, h->q.bytes()));
    SELF_CUDA_TRY(ctx, cudaMemset(h->G.p, 0, h->G.bytes()));
    SELF_CUDA_TRY(ctx, cudaMemset(h->bf.p, 0, h->bf.bytes()));
  } else {
    h->f32 = selfgpu::dg32::make_state();
    rc = selfgpu::dg32::create(h.get(), h->f32, d, met, aux, eg);
    if (rc) return rc;
  }
  *out = h.release();
  return SELF_OK;
}

int self_dg2d_destroy(self_dg2d* h) {
  if (!h) return SELF_OK;
  cudaSetDevice(h->ctx->device);
  cudaStreamSynchronize(h->ctx->stream);
  delete h;
  return SELF_OK;
}

int self_dg2d_set_state(self_dg2d* h, const double* q) {
  if (!h || !q) return SELF_ERR_INVALID;
  self_ctx* ctx = h->ctx;
  SELF_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  if (h->precision == SELF_PREC_FP32) return selfgpu::dg32::set_state(h, h->f32, q);
  SELF_CUDA_TRY(ctx, cudaMemcpyAsync(h->q.p, q, h->q.bytes(), cudaMemcpyHostToDevice, ctx->stream));
  SELF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  h->traces_valid = false;
  return SELF_OK;
}

int self_dg2d_get_state(self_dg2d* h, double* q) {
  if (!h || !q) return SELF_ERR_INVALID;
  self_ctx* ctx = h->ctx;
  SELF_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  if (h->precision == SELF_PREC_FP32) return selfgpu::dg32::get_state(h, h->f32, q);
  SELF_CUDA_TRY(ctx, cudaMemcpyAsync(q, h->q.p, h->q.bytes(), cudaMemcpyDeviceToHost, ctx->stream));
  SELF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return SELF_OK;
}

long long self_dg2d_bytes(const self_dg2d* h) {
  if (!h) return 0;
  long long b = (long long)(h->q.bytes() + h->G.bytes() + h->bs.bytes() + h->bf.bytes() + h->metrics.bytes() +
                            h->aux.bytes() + h->egeo.bytes() + h->tend.bytes() + h->edges.bytes());
  if (h->f32) b += selfgpu::dg32::bytes(h->f32);
  return b;
}

int self_dg2d_state_device(self_dg2d* h, void** dptr, size_t* bytes) {
  if (!h || !dptr) return SELF_ERR_INVALID;
  if (h->precision == SELF_PREC_FP32) return selfgpu::dg32::state_device(h, h->f32, dptr, bytes);
  *dptr = h->q.p;
  if (bytes) *bytes = h->q.bytes();
  return SELF_OK;
}

int self_dg2d_tendency(self_dg2d* h, double t, double* dqdt) {
  if (!h) return SELF_ERR_INVALID;
  self_ctx* ctx = h->ctx;
  SELF_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  if (h->precision == SELF_PREC_FP32) return selfgpu::dg32::tendency(h, h->f32, t, dqdt);
  if (h->tend.n == 0 && h->tend.alloc(h->q.n) != cudaSuccess)
    return set_error(ctx, SELF_ERR_ALLOC, "device allocation failed");
  int rc = launch_traces(h, h->q.p);
  if (rc) return rc;
  rc = launch_stage(h, 0, 0.0, 0.0, t, h->q.p, nullptr, h->tend.p, 0);
  if (rc) return rc;
  if (dqdt) {
    SELF_CUDA_TRY(ctx, cudaMemcpyAsync(dqdt, h->tend.p, h->tend.bytes(), cudaMemcpyDeviceToHost, ctx->stream));
  }
  SELF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return SELF_OK;
}

int self_dg2d_rk3_async(self_dg2d* h, double tn, int nsteps) {
  if (!h || nsteps < 0) return SELF_ERR_INVALID;
  self_ctx* ctx = h->ctx;
  SELF_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  if (h->precision == SELF_PREC_FP32) return selfgpu::dg32::rk3(h, h->f32, tn, nsteps);
  int rc;
  if (!h->traces_valid) {
    if ((rc = launch_traces(h, h->q.p))) return rc;
    h->traces_valid = true;
  }
  if (h->has_inflow) {  // time-dependent boundary data: plain launches
    for (int s = 0; s < nsteps; ++s)
      if ((rc = enqueue_step(h, tn + s * h->dt))) return rc;
    return SELF_OK;
  }
  if (!h->step_graph) {  // capture one RK3 step (6 kernels) once, replay it nsteps times
    cudaGraph_t g;
    const long long l0 = ctx->launches.load();
    SELF_CUDA_TRY(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    rc = enqueue_step(h, tn);
    cudaError_t ce = cudaStreamEndCapture(ctx->stream, &g);
    if (rc) return rc;
    if (ce != cudaSuccess) return set_error(ctx, SELF_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
    ce = cudaGraphInstantiate(&h->step_graph, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return set_error(ctx, SELF_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ce));
    h->step_graph_launches = ctx->launches.load() - l0;
    ctx->launches.fetch_sub(h->step_graph_launches);  // captured, not launched
  }
  for (int s = 0; s < nsteps; ++s) {
    SELF_CUDA_TRY(ctx, cudaGraphLaunch(h->step_graph, ctx->stream));
    ctx->launches.fetch_add(h->step_graph_launches);
  }
  return SELF_OK;
}

int self_dg2d_time_kernels(self_dg2d* h, int reps, size_t flush_bytes, double* ms) {
  if (!h || !ms || reps < 1) return SELF_ERR_INVALID;
  self_ctx* ctx = h->ctx;
  SELF_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  if (h->precision == SELF_PREC_FP32) return selfgpu::dg32::time_kernels(h, h->f32, reps, flush_bytes, ms);
  DevBuf<double> q0, G0;
  if (q0.alloc(h->q.n) || G0.alloc(h->G.n)) return set_error(ctx, SELF_ERR_ALLOC, "device allocation failed");
  SELF_CUDA_TRY(ctx, cudaMemcpyAsync(q0.p, h->q.p, h->q.bytes(), cudaMemcpyDeviceToDevice, ctx->stream));
  SELF_CUDA_TRY(ctx, cudaMemcpyAsync(G0.p, h->G.p, h->G.bytes(), cudaMemcpyDeviceToDevice, ctx->stream));
  int rc;
  if (!h->traces_valid) {
    if ((rc = launch_traces(h, h->q.p))) return rc;
  }
  double te = 0, tv = 0, t;
  for (int r = 0; r < reps; ++r) {
    // one full stage, each of its two kernels timed alone after an L2 flush
    if ((rc = self_ctx_flush_l2(ctx, flush_bytes))) return rc;
    if ((rc = self_ctx_timer_start(ctx))) return rc;
    if ((rc = launch_edge_only(h, 0.0))) return rc;
    if ((rc = self_ctx_timer_stop(ctx, &t))) return rc;
    te += t;
    if ((rc = self_ctx_flush_l2(ctx, flush_bytes))) return rc;
    if ((rc = self_ctx_timer_start(ctx))) return rc;
    if ((rc = launch_volume_only(h, 2, kRK3a[1], kRK3g[1] * h->dt, h->q.p, h->q.p, nullptr, 1))) return rc;
    if ((rc = self_ctx_timer_stop(ctx, &t))) return rc;
    tv += t;
  }
  ms[0] = te / reps;
  ms[1] = tv / reps;
  SELF_CUDA_TRY(ctx, cudaMemcpyAsync(h->q.p, q0.p, h->q.bytes(), cudaMemcpyDeviceToDevice, ctx->stream));
  SELF_CUDA_TRY(ctx, cudaMemcpyAsync(h->G.p, G0.p, h->G.bytes(), cudaMemcpyDeviceToDevice, ctx->stream));
  SELF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  h->traces_valid = false;
  return SELF_OK;
}

int self_dg2d_test_wait_timeout(self_dg2d* h, int polls) {
  if (!h) return SELF_ERR_INVALID;
  SELF_CUDA_TRY(h->ctx, cudaSetDevice(h->ctx->device));
  if (h->precision != SELF_PREC_FP32)
    return set_error(h->ctx, SELF_ERR_UNSUPPORTED, "time-out test hook: fused FP32 stage only");
  return selfgpu::dg32::arm_wait_timeout(h, h->f32, polls);
}

int self_dg2d_rk3(self_dg2d* h, double tn, int nsteps) {
  int rc = self_dg2d_rk3_async(h, tn, nsteps);
  if (rc) return rc;
  if (h->precision == SELF_PREC_FP32) return selfgpu::dg32::sync_and_check(h, h->f32);
  SELF_CUDA_TRY(h->ctx, cudaStreamSynchronize(h->ctx->stream));
  return SELF_OK;
}

}  // extern "C"
