// CPU oracle (test infrastructure): DGSEM 2-D tendency and low-storage RK3.
// Restates src/highend/shallowwater/ConservativeShallowWaterClass.f90 (ForwardStepRK3 :1173-1218,
// GlobalTimeDerivative :1222-1262, EdgeFlux :1266-1360, MappedTimeDerivative :1364-1522,
// DGSystemDerivative :1526-1551, RiemannSolver :1555-1604, XFlux/YFlux :1608-1658, Source :1662-1694,
// GetExternalState :1698-1729, CalculateBathymetryGradient :1733-1868), the matching routines of
// src/highend/advection-diffusion2d/AdvectionClass.f90 (:1268-1886) and
// src/dgsem/DGSEMSolutionStorageClass_2D.f90 CalculateSolutionAtBoundaries (:749-802).
// Model 3 restates the LINEAR formulation of src/highend/shallowwater/ShallowWaterClass.f90 (state u, v, eta):
// EdgeFlux :1530-1624 (depth HALF*(inBathy + exBathy) at interior edges, inBathy on the boundary, the bathymetry
// traces of CalculateBathymetryAtBoundaries :1357-1368), RiemannSolver :2072-2161 (LINEAR branch), XFlux/YFlux
// :2165-2256, Source :2260-2294 (vorticity = f, relativeFactor = 0), GetExternalState :2298-2325 (NO_NORMAL_FLOW
// mirror, other flags zero) and MappedTimeDerivative :1728-1887 (same DG structure).
// Model 4 restates its SKEW_SYMMETRIC formulation with the relative vorticity as a 4th state variable (the
// reference keeps it in vorticity(:)%solution(:,:,2) and advances it with the same RK3 coefficients,
// ForwardStepRK3 :1372-1432): RiemannSolver SKEW_SYMMETRIC branch, XFlux/YFlux with the kinetic energy, Source with
// vorticity = f + zeta (relativeFactor = 1), RelativeVorticityEdgeFlux :1628-1724 (VorticityFluxSolver
// :2041-2068, GetExternalVorticity :2329-2356: NO_NORMAL_FLOW copies the interior value, other flags zero; the
// boundary's outer planetary vorticity is the inner one) and VorticityTimeDerivative :1891-2008.
// Advection with kappa > 0 restates the BR1 passes of AdvectionClass.f90: GlobalTimeDerivative :1316-1378
// (traces, EdgeGradientFlux :1482-1563 = central flux HALF*(in + ex)*n*|n|, CalculateConcentrationGradient
// :1123-1264 = DG weak derivative with lift, divided by J, CalculateGradientAtBoundaries :1092-1104, EdgeFlux
// :1382-1478 with the averaged gradient on interior edges and the inner one on the boundary, RiemannSolver
// :1756-1787 minus kappa dc/dn, XFlux/YFlux :1790-1825 = c u - kappa dc/dx, c v - kappa dc/dy).
// Decision: V2D, never initialised in ForwardStepRK3, is taken as zero (its first use multiplies it by
// rk3_a(1) = 0).
// Decision: the Riemann solver's undeclared "g" (:1589-1592) is the parameter g (locG).
// OpenMP over elements and edges follows the reference's !$OMP DO placement.
#include <cmath>
#include <cstring>
#include <vector>

#include "oracle.h"

namespace {

// ConstantsDictionary.f90:66-68
const double rk3_a[3] = {0.0, -5.0 / 9.0, -153.0 / 128.0};
const double rk3_b[3] = {0.0, 1.0 / 3.0, 3.0 / 4.0};
const double rk3_g[3] = {1.0 / 3.0, 15.0 / 16.0, 8.0 / 15.0};

struct Idx {
  int n, nEq;
  size_t q(int i, int j, int v, int e) const { return (size_t)i + n * (j + (size_t)n * (v + (size_t)nEq * e)); }
  size_t f(int i, int j, int e) const { return (size_t)i + n * (j + (size_t)n * e); }
  size_t b(int i, int v, int s, int e) const { return (size_t)i + n * (v + (size_t)nEq * (s + 4 * (size_t)e)); }
  size_t nh(int i, int s, int e) const { return (size_t)i + n * (s + 4 * (size_t)e); }
};

// DGSystemDerivative: MATMUL(dMat, intFlux) + (rFlux*lagRight + lFlux*lagLeft)/qWei
void dg_system_derivative(int n, const double* dMat, const double* qw, double lF, double rF, const double* f,
                          const double* lL, const double* lR, double* out) {
  for (int k = 0; k < n; ++k) {
    double s = 0.0;
    for (int m = 0; m < n; ++m) s = s + dMat[k + m * n] * f[m];
    out[k] = s;
  }
  for (int k = 0; k < n; ++k) out[k] = out[k] + (rF * lR[k] + lF * lL[k]) / qw[k];
}

void sw_riemann(const double* in, const double* out, const double* nH, double g, double* flux) {
  double jump[3] = {out[0] - in[0], out[1] - in[1], out[2] - in[2]};
  double uL = in[0], vL = in[1], pL = in[2];
  double uR = out[0], vR = out[1], pR = out[2];
  double uOut = uR * nH[0] + vR * nH[1];
  double uIn = uL * nH[0] + vL * nH[1];
  double c1 = std::fabs(uOut / pR + std::sqrt(g * pR));
  double c2 = std::fabs(uOut / pR - std::sqrt(g * pR));
  double c3 = std::fabs(uIn / pL + std::sqrt(g * pL));
  double c4 = std::fabs(uIn / pL - std::sqrt(g * pL));
  double fac = std::fmax(std::fmax(std::fmax(c1, c2), c3), c4);
  double aS[3];
  aS[0] = (uOut / pR) * uR + 0.5 * g * pR * pR * nH[0] + (uIn / pL) * uL + 0.5 * g * pL * pL * nH[0];
  aS[1] = (uOut / pR) * vR + 0.5 * g * pR * pR * nH[1] + (uIn / pL) * vL + 0.5 * g * pL * pL * nH[1];
  aS[2] = uOut + uIn;
  for (int k = 0; k < 3; ++k) flux[k] = 0.5 * (aS[k] - fac * jump[k]);
}

// RiemannSolver, LINEAR branch (ShallowWaterClass.f90:2106-2113), depth h at the edge node
void swl_riemann(const double* in, const double* out, const double* nH, double h, double g, double* flux) {
  double uL = in[0], vL = in[1], pL = in[2];
  double uR = out[0], vR = out[1], pR = out[2];
  double uOut = uR * nH[0] + vR * nH[1];
  double uIn = uL * nH[0] + vL * nH[1];
  double fac = std::sqrt(g * h);
  flux[0] = 0.5 * (g * (pR + pL) + fac * (uIn - uOut)) * nH[0];
  flux[1] = 0.5 * (g * (pR + pL) + fac * (uIn - uOut)) * nH[1];
  flux[2] = 0.5 * (h * (uIn + uOut) + fac * (pL - pR));
}

// RiemannSolver, SKEW_SYMMETRIC branch (ShallowWaterClass.f90:2114-2133), depth h at the edge node
void sws_riemann(const double* in, const double* out, const double* nH, double h, double g, double* flux) {
  double jump[3] = {out[0] - in[0], out[1] - in[1], out[2] - in[2]};
  double uL = in[0], vL = in[1], pL = in[2];
  double uR = out[0], vR = out[1], pR = out[2];
  double uOut = uR * nH[0] + vR * nH[1];
  double uIn = uL * nH[0] + vL * nH[1];
  double c1 = std::fabs(0.25 * (uOut + std::sqrt(uOut * uOut + 16.0 * g * (pR + h))));
  double c2 = std::fabs(0.25 * (uOut - std::sqrt(uOut * uOut + 16.0 * g * (pR + h))));
  double c3 = std::fabs(0.25 * (uIn + std::sqrt(uIn * uIn + 16.0 * g * (pL + h))));
  double c4 = std::fabs(0.25 * (uIn - std::sqrt(uIn * uIn + 16.0 * g * (pL + h))));
  double fac = std::fmax(std::fmax(std::fmax(c1, c2), c3), c4);
  double e = 0.5 * (uR * uR + vR * vR) + g * pR + 0.5 * (uL * uL + vL * vL) + g * pL;
  double aS[3] = {e * nH[0], e * nH[1], uIn * (pL + h) + uOut * (pR + h)};
  for (int k = 0; k < 3; ++k) flux[k] = 0.5 * (aS[k] - fac * jump[k]);
}

// VorticityFluxSolver (ShallowWaterClass.f90:2041-2068)
double vort_flux(const double* in, const double* out, double zIn, double zOut, const double* nH) {
  double uOut = out[0] * nH[0] + out[1] * nH[1];
  double uIn = in[0] * nH[0] + in[1] * nH[1];
  return 0.5 * (uOut * zOut + uIn * zIn - std::fmax(std::fabs(uOut), std::fabs(uIn)) * (zOut - zIn));
}

// trace of a nodal field on side s of element e at side node i (CalculateSolutionAtBoundaries order)
double field_trace(const orc_dg_problem* p, const double* fld, int s, int i, int e) {
  const int n = p->N + 1;
  Idx I{n, 1};
  double acc = 0.0;
  if (s == 0 || s == 2) {
    const double* L = s == 0 ? p->lS : p->lN;
    for (int j = 0; j < n; ++j) acc = acc + L[j] * fld[I.f(i, j, e)];
  } else {
    const double* L = s == 1 ? p->lE : p->lW;
    for (int m = 0; m < n; ++m) acc = acc + L[m] * fld[I.f(m, i, e)];
  }
  return acc;
}

void sw_external(const double* nH, const double* in, double* ex) {  // NO_NORMAL_FLOW mirror
  ex[0] = (nH[1] * nH[1] - nH[0] * nH[0]) * in[0] - 2.0 * nH[0] * nH[1] * in[1];
  ex[1] = (nH[0] * nH[0] - nH[1] * nH[1]) * in[1] - 2.0 * nH[0] * nH[1] * in[0];
  ex[2] = in[2];
}

}  // namespace

extern "C" {

int orc_set_threads(int n) {
#ifdef _OPENMP
  extern void omp_set_num_threads(int);
  omp_set_num_threads(n);
#endif
  return 0;
}

int orc_dg_traces(const orc_dg_problem* p, const double* q, double* bs) {
  const int n = p->N + 1, nEq = p->nEq;
  Idx I{n, nEq};
#pragma omp parallel for schedule(static)
  for (int e = 0; e < p->nEl; ++e) {
    for (int j = 0; j < n; ++j)
      for (int v = 0; v < nEq; ++v) {
        double w = 0.0, ea = 0.0;
        for (int i = 0; i < n; ++i) w = w + p->lW[i] * q[I.q(i, j, v, e)];
        for (int i = 0; i < n; ++i) ea = ea + p->lE[i] * q[I.q(i, j, v, e)];
        bs[I.b(j, v, 3, e)] = w;
        bs[I.b(j, v, 1, e)] = ea;
      }
    for (int i = 0; i < n; ++i)
      for (int v = 0; v < nEq; ++v) {
        double s = 0.0, no = 0.0;
        for (int j = 0; j < n; ++j) s = s + p->lS[j] * q[I.q(i, j, v, e)];
        for (int j = 0; j < n; ++j) no = no + p->lN[j] * q[I.q(i, j, v, e)];
        bs[I.b(i, v, 0, e)] = s;
        bs[I.b(i, v, 2, e)] = no;
      }
  }
  return 0;
}

static int edge_flux(const orc_dg_problem* p, double t, const double* bs, const double* gtx, const double* gty,
                     double* bf);

int orc_dg_edge_flux(const orc_dg_problem* p, double t, const double* bs, double* bf) {
  return edge_flux(p, t, bs, nullptr, nullptr, bf);
}

static int edge_flux(const orc_dg_problem* p, double t, const double* bs, const double* gtx, const double* gty,
                     double* bf) {
  const int n = p->N + 1, nEq = p->nEq, N = p->N;
  Idx I{n, nEq};
  int err = 0;
#pragma omp parallel for schedule(static) reduction(| : err)
  for (int k = 0; k < p->nEdges; ++k) {
    const int* E = p->edges + 6 * k;
    int e1 = E[0] - 1, s1 = E[1] - 1, e2 = E[2], s2 = std::abs(E[3]) - 1, start = E[4], inc = E[5];
    double in[16], ex[16], fl[16], nH[2];
    if (nEq > 16) {
      err |= 1;
      continue;
    }
    if (e2 > 0) {
      e2 -= 1;
      int kk = start - inc;
      for (int i = 0; i <= N; ++i) {
        nH[0] = p->nhx[I.nh(i, s1, e1)];
        nH[1] = p->nhy[I.nh(i, s1, e1)];
        double len = p->nlen[I.nh(i, s1, e1)];
        for (int v = 0; v < nEq; ++v) {
          in[v] = bs[I.b(i, v, s1, e1)];
          ex[v] = bs[I.b(kk, v, s2, e2)];
        }
        if (p->model == 1) {
          sw_riemann(in, ex, nH, p->g, fl);
        } else if (p->model == 3) {
          const double hd = 0.5 * (field_trace(p, p->h, s1, i, e1) + field_trace(p, p->h, s2, kk, e2));
          swl_riemann(in, ex, nH, hd, p->g, fl);
        } else if (p->model == 4) {
          const double hd = 0.5 * (field_trace(p, p->h, s1, i, e1) + field_trace(p, p->h, s2, kk, e2));
          sws_riemann(in, ex, nH, hd, p->g, fl);
          const double zIn = in[3] + field_trace(p, p->fcor, s1, i, e1);
          const double zOut = ex[3] + field_trace(p, p->fcor, s2, kk, e2);
          fl[3] = vort_flux(in, ex, zIn, zOut, nH);
        } else {
          // advection (AdvectionClass.f90:1756-1787) with the primary element's boundary velocity
          // (CalculateVelocityAtBoundaries: Lagrange traces of u and v)
          double ub = 0.0, vb = 0.0;
          const double* L = (s1 == 0) ? p->lS : (s1 == 1) ? p->lE : (s1 == 2) ? p->lN : p->lW;
          for (int m = 0; m < n; ++m) {
            size_t id = (s1 == 0 || s1 == 2) ? I.f(i, m, e1) : I.f(m, i, e1);
            ub = ub + L[m] * p->u[id];
            vb = vb + L[m] * p->v[id];
          }
          double un = ub * nH[0] + vb * nH[1];
          for (int v = 0; v < nEq; ++v) {
            double jump = ex[v] - in[v];
            fl[v] = 0.5 * (un * (ex[v] + in[v]) - std::fabs(un) * jump);
            if (gtx) {  // - kappa dc/dn with the averaged gradient
              double gx = (gtx[I.b(i, v, s1, e1)] + gtx[I.b(kk, v, s2, e2)]) * 0.5;
              double gy = (gty[I.b(i, v, s1, e1)] + gty[I.b(kk, v, s2, e2)]) * 0.5;
              fl[v] = fl[v] - p->kappa * (gx * nH[0] + gy * nH[1]);
            }
          }
        }
        for (int v = 0; v < nEq; ++v) {
          double f = fl[v] * len;
          bf[I.b(i, v, s1, e1)] = f;
          bf[I.b(kk, v, s2, e2)] = -f;
        }
        kk = kk + inc;
      }
    } else {
      for (int i = 0; i <= N; ++i) {
        nH[0] = p->nhx[I.nh(i, s1, e1)];
        nH[1] = p->nhy[I.nh(i, s1, e1)];
        double len = p->nlen[I.nh(i, s1, e1)];
        for (int v = 0; v < nEq; ++v) in[v] = bs[I.b(i, v, s1, e1)];
        if (p->model == 1 || p->model == 3 || p->model == 4) {
          if (e2 == ORC_NO_NORMAL_FLOW) {
            sw_external(nH, in, ex);
          } else {
            ex[0] = ex[1] = ex[2] = 0.0;
          }
          if (p->model == 1) {
            sw_riemann(in, ex, nH, p->g, fl);
          } else if (p->model == 3) {
            swl_riemann(in, ex, nH, field_trace(p, p->h, s1, i, e1), p->g, fl);
          } else {
            sws_riemann(in, ex, nH, field_trace(p, p->h, s1, i, e1), p->g, fl);
            const double relOut = e2 == ORC_NO_NORMAL_FLOW ? in[3] : 0.0;
            const double fIn = field_trace(p, p->fcor, s1, i, e1);
            fl[3] = vort_flux(in, ex, in[3] + fIn, relOut + fIn, nH);
          }
        } else {
          for (int v = 0; v < nEq; ++v) ex[v] = 0.0;
          if (e2 == ORC_INFLOW_ONE) ex[0] = std::tanh(t);
          if (e2 == ORC_INFLOW_TWO && nEq > 1) ex[1] = std::tanh(t);
          double ub = 0.0, vb = 0.0;
          const double* L = (s1 == 0) ? p->lS : (s1 == 1) ? p->lE : (s1 == 2) ? p->lN : p->lW;
          for (int m = 0; m < n; ++m) {
            size_t id = (s1 == 0 || s1 == 2) ? I.f(i, m, e1) : I.f(m, i, e1);
            ub = ub + L[m] * p->u[id];
            vb = vb + L[m] * p->v[id];
          }
          double un = ub * nH[0] + vb * nH[1];
          for (int v = 0; v < nEq; ++v) {
            double jump = ex[v] - in[v];
            fl[v] = 0.5 * (un * (ex[v] + in[v]) - std::fabs(un) * jump);
            if (gtx)  // - kappa dc/dn with the inner gradient
              fl[v] = fl[v] - p->kappa * (gtx[I.b(i, v, s1, e1)] * nH[0] + gty[I.b(i, v, s1, e1)] * nH[1]);
          }
        }
        for (int v = 0; v < nEq; ++v) bf[I.b(i, v, s1, e1)] = fl[v] * len;
      }
    }
  }
  return err ? -1 : 0;
}

// MappedTimeDerivative for one element
static void mapped_time_derivative(const orc_dg_problem* p, double t, const double* q, const double* bf,
                                   const double* gx, const double* gy, double* tend, int e) {
  const int n = p->N + 1, nEq = p->nEq;
  Idx I{n, nEq};
  std::vector<double> cf(n * nEq), der(n), xF(nEq), yF(nEq), sol(nEq);
  auto fluxes = [&](int i, int j) {
    for (int v = 0; v < nEq; ++v) sol[v] = q[I.q(i, j, v, e)];
    if (p->model == 1) {
      // XFlux / YFlux (:1608-1658)
      double g = p->g;
      xF[0] = sol[0] * sol[0] / (sol[2]) + g * 0.5 * sol[2] * sol[2];
      xF[1] = sol[0] * sol[1] / (sol[2]);
      xF[2] = sol[0];
      yF[0] = sol[1] * sol[0] / (sol[2]);
      yF[1] = sol[1] * sol[1] / (sol[2]) + g * 0.5 * sol[2] * sol[2];
      yF[2] = sol[1];
    } else if (p->model == 4) {
      // XFlux / YFlux, SKEW_SYMMETRIC (ShallowWaterClass.f90:2179-2187, 2226-2234), and the vorticity fluxes
      // u (zeta + f), v (zeta + f) of VorticityTimeDerivative (:1934-1936)
      double g = p->g, h = p->h[I.f(i, j, e)], f = p->fcor[I.f(i, j, e)];
      double KE = (sol[0] * sol[0] + sol[1] * sol[1]) * 0.5;
      xF[0] = g * sol[2] + KE;
      xF[1] = 0.0;
      xF[2] = (h + sol[2]) * sol[0];
      yF[0] = 0.0;
      yF[1] = g * sol[2] + KE;
      yF[2] = (h + sol[2]) * sol[1];
      xF[3] = sol[0] * (sol[3] + f);
      yF[3] = sol[1] * (sol[3] + f);
    } else if (p->model == 3) {
      // XFlux / YFlux, LINEAR (ShallowWaterClass.f90:2171-2177, 2218-2224)
      double g = p->g, h = p->h[I.f(i, j, e)];
      xF[0] = g * sol[2];
      xF[1] = 0.0;
      xF[2] = h * sol[0];
      yF[0] = 0.0;
      yF[1] = g * sol[2];
      yF[2] = h * sol[1];
    } else {
      double u = p->u[I.f(i, j, e)], v = p->v[I.f(i, j, e)];
      for (int k = 0; k < nEq; ++k) {
        xF[k] = sol[k] * u;
        yF[k] = sol[k] * v;
        if (gx) {
          xF[k] = xF[k] - p->kappa * gx[I.q(i, j, k, e)];
          yF[k] = yF[k] - p->kappa * gy[I.q(i, j, k, e)];
        }
      }
    }
  };
  // s-direction (:1398-1445)
  for (int j = 0; j < n; ++j) {
    for (int i = 0; i < n; ++i) {
      size_t id = I.f(i, j, e);
      double dxdp = p->dxdp[id], dydp = p->dydp[id];
      fluxes(i, j);
      for (int v = 0; v < nEq; ++v) cf[i + n * v] = dydp * xF[v] - dxdp * yF[v];
    }
    for (int v = 0; v < nEq; ++v) {
      double fL = bf[I.b(j, v, 3, e)], fR = bf[I.b(j, v, 1, e)];
      dg_system_derivative(n, p->dmatS, p->qw, fL, fR, &cf[n * v], p->lW, p->lE, der.data());
      for (int i = 0; i < n; ++i) tend[I.q(i, j, v, e)] = -der[i];
    }
  }
  // p-direction (:1448-1494)
  for (int i = 0; i < n; ++i) {
    for (int j = 0; j < n; ++j) {
      size_t id = I.f(i, j, e);
      double dxds = p->dxds[id], dyds = p->dyds[id];
      fluxes(i, j);
      for (int v = 0; v < nEq; ++v) cf[j + n * v] = -dyds * xF[v] + dxds * yF[v];
    }
    for (int v = 0; v < nEq; ++v) {
      double fL = bf[I.b(i, v, 0, e)], fR = bf[I.b(i, v, 2, e)];
      dg_system_derivative(n, p->dmatP, p->qw, fL, fR, &cf[n * v], p->lS, p->lN, der.data());
      for (int j = 0; j < n; ++j) {
        double Jn = p->J[I.f(i, j, e)];
        tend[I.q(i, j, v, e)] = (tend[I.q(i, j, v, e)] - der[j]) / Jn;
      }
    }
  }
  // sources (:1497-1519)
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      size_t id = I.f(i, j, e);
      for (int v = 0; v < nEq; ++v) sol[v] = q[I.q(i, j, v, e)];
      if (p->model == 1) {
        double relax[3] = {0, 0, 0}, ts = 0.0;
        if (p->relax) {
          for (int v = 0; v < 3; ++v) relax[v] = p->relax[I.q(i, j, v, e)];
        }
        if (p->rfac) ts = p->rfac[id];
        double plv = p->fcor[id], h = p->h[id], dhdx = p->dhdx[id], dhdy = p->dhdy[id];
        double g = p->g, lD = p->drag;
        double s0 = plv * sol[1] + g * sol[2] * dhdx - lD * sol[0] / h - (sol[0] - relax[0]) * ts;
        double s1 = -plv * sol[0] + g * sol[2] * dhdy - lD * sol[1] / h - (sol[1] - relax[1]) * ts;
        double s2 = -(sol[2] - relax[2]) * ts;
        tend[I.q(i, j, 0, e)] = tend[I.q(i, j, 0, e)] + s0;
        tend[I.q(i, j, 1, e)] = tend[I.q(i, j, 1, e)] + s1;
        tend[I.q(i, j, 2, e)] = tend[I.q(i, j, 2, e)] + s2;
      } else if (p->model == 3 || p->model == 4) {
        // Source, LINEAR / SKEW_SYMMETRIC (ShallowWaterClass.f90:2272-2281): vorticity = f + relativeFactor zeta
        // (relativeFactor 0 / 1, :1876); the vorticity equation has no source
        double relax[3] = {0, 0, 0}, ts = 0.0;
        if (p->relax) {
          for (int v = 0; v < 3; ++v) relax[v] = p->relax[I.q(i, j, v, e)];
        }
        if (p->rfac) ts = p->rfac[id];
        double vort = p->model == 4 ? p->fcor[id] + 1.0 * sol[3] : p->fcor[id], lD = p->drag;
        double s0 = vort * sol[1] - lD * sol[0] - (sol[0] - relax[0]) * ts;
        double s1 = -vort * sol[0] - lD * sol[1] - (sol[1] - relax[1]) * ts;
        double s2 = -(sol[2] - relax[2]) * ts;
        tend[I.q(i, j, 0, e)] = tend[I.q(i, j, 0, e)] + s0;
        tend[I.q(i, j, 1, e)] = tend[I.q(i, j, 1, e)] + s1;
        tend[I.q(i, j, 2, e)] = tend[I.q(i, j, 2, e)] + s2;
      } else {
        for (int v = 0; v < nEq; ++v) {
          double r = p->relax ? p->relax[I.q(i, j, v, e)] : 0.0;
          double rf = p->rfac ? p->rfac[I.q(i, j, v, e)] : 0.0;
          tend[I.q(i, j, v, e)] = tend[I.q(i, j, v, e)] + (r - sol[v]) * rf;
        }
      }
    }
}

// EdgeGradientFlux: central flux of the traces into the boundary fluxes of dC/dx and dC/dy
static void edge_gradient_flux(const orc_dg_problem* p, double t, const double* bs, double* bgx, double* bgy) {
  const int n = p->N + 1, nEq = p->nEq, N = p->N;
  Idx I{n, nEq};
#pragma omp parallel for schedule(static)
  for (int k = 0; k < p->nEdges; ++k) {
    const int* E = p->edges + 6 * k;
    int e1 = E[0] - 1, s1 = E[1] - 1, e2 = E[2], s2 = std::abs(E[3]) - 1, start = E[4], inc = E[5];
    int kk = start - inc;
    for (int i = 0; i <= N; ++i) {
      double nx = p->nhx[I.nh(i, s1, e1)], ny = p->nhy[I.nh(i, s1, e1)], len = p->nlen[I.nh(i, s1, e1)];
      for (int v = 0; v < nEq; ++v) {
        double in = bs[I.b(i, v, s1, e1)], ex;
        if (e2 > 0) {
          ex = bs[I.b(kk, v, s2, e2 - 1)];
        } else {
          ex = 0.0;  // GetExternalState (:1851-1886)
          if (e2 == ORC_INFLOW_ONE && v == 0) ex = std::tanh(t);
          if (e2 == ORC_INFLOW_TWO && v == 1) ex = std::tanh(t);
        }
        double fx = 0.5 * (in + ex) * nx * len, fy = 0.5 * (in + ex) * ny * len;
        bgx[I.b(i, v, s1, e1)] = fx;
        bgy[I.b(i, v, s1, e1)] = fy;
        if (e2 > 0) {
          bgx[I.b(kk, v, s2, e2 - 1)] = -fx;
          bgy[I.b(kk, v, s2, e2 - 1)] = -fy;
        }
      }
      kk = kk + inc;
    }
  }
}

// CalculateConcentrationGradient for one element
static void concentration_gradient(const orc_dg_problem* p, const double* q, const double* bgx, const double* bgy,
                                   double* gx, double* gy, int e) {
  const int n = p->N + 1, nEq = p->nEq;
  Idx I{n, nEq};
  std::vector<double> c1(n), c2(n), d1(n), d2(n);
  for (int v = 0; v < nEq; ++v) {
    for (int j = 0; j < n; ++j) {
      for (int i = 0; i < n; ++i) {
        size_t id = I.f(i, j, e);
        double sol = q[I.q(i, j, v, e)];
        c1[i] = p->dydp[id] * sol - p->dxdp[id] * 0.0;
        c2[i] = p->dydp[id] * 0.0 - p->dxdp[id] * sol;
      }
      dg_system_derivative(n, p->dmatS, p->qw, bgx[I.b(j, v, 3, e)], bgx[I.b(j, v, 1, e)], c1.data(), p->lW, p->lE,
                           d1.data());
      dg_system_derivative(n, p->dmatS, p->qw, bgy[I.b(j, v, 3, e)], bgy[I.b(j, v, 1, e)], c2.data(), p->lW, p->lE,
                           d2.data());
      for (int i = 0; i < n; ++i) {
        gx[I.q(i, j, v, e)] = d1[i];
        gy[I.q(i, j, v, e)] = d2[i];
      }
    }
    for (int i = 0; i < n; ++i) {
      for (int j = 0; j < n; ++j) {
        size_t id = I.f(i, j, e);
        double sol = q[I.q(i, j, v, e)];
        c1[j] = -p->dyds[id] * sol + p->dxds[id] * 0.0;
        c2[j] = -p->dyds[id] * 0.0 + p->dxds[id] * sol;
      }
      dg_system_derivative(n, p->dmatP, p->qw, bgx[I.b(i, v, 0, e)], bgx[I.b(i, v, 2, e)], c1.data(), p->lS, p->lN,
                           d1.data());
      dg_system_derivative(n, p->dmatP, p->qw, bgy[I.b(i, v, 0, e)], bgy[I.b(i, v, 2, e)], c2.data(), p->lS, p->lN,
                           d2.data());
      for (int j = 0; j < n; ++j) {
        double Jn = p->J[I.f(i, j, e)];
        gx[I.q(i, j, v, e)] = (gx[I.q(i, j, v, e)] + d1[j]) / Jn;
        gy[I.q(i, j, v, e)] = (gy[I.q(i, j, v, e)] + d2[j]) / Jn;
      }
    }
  }
}

int orc_dg_tendency(const orc_dg_problem* p, double t, const double* q, double* tend) {
  const bool br1 = p->model == 2 && p->kappa != 0.0;
  if (p->kappa != 0.0 && !br1) return -5;
  const int n = p->N + 1;
  size_t nb = (size_t)n * p->nEq * 4 * p->nEl, nq = (size_t)n * n * p->nEq * p->nEl;
  std::vector<double> bs(nb, 0.0), bf(nb, 0.0);
  orc_dg_traces(p, q, bs.data());
  std::vector<double> bgx, bgy, gx, gy, gtx, gty;
  if (br1) {
    bgx.assign(nb, 0.0);
    bgy.assign(nb, 0.0);
    gx.assign(nq, 0.0);
    gy.assign(nq, 0.0);
    gtx.assign(nb, 0.0);
    gty.assign(nb, 0.0);
    edge_gradient_flux(p, t, bs.data(), bgx.data(), bgy.data());
#pragma omp parallel for schedule(static)
    for (int e = 0; e < p->nEl; ++e) concentration_gradient(p, q, bgx.data(), bgy.data(), gx.data(), gy.data(), e);
    orc_dg_traces(p, gx.data(), gtx.data());  // CalculateGradientAtBoundaries
    orc_dg_traces(p, gy.data(), gty.data());
  }
  if (edge_flux(p, t, bs.data(), br1 ? gtx.data() : nullptr, br1 ? gty.data() : nullptr, bf.data()) != 0) return -1;
#pragma omp parallel for schedule(static)
  for (int e = 0; e < p->nEl; ++e)
    mapped_time_derivative(p, t, q, bf.data(), br1 ? gx.data() : nullptr, br1 ? gy.data() : nullptr, tend, e);
  return 0;
}

int orc_dg_rk3(const orc_dg_problem* p, double tn, int nsteps, double* q) {
  const int n = p->N + 1;
  size_t nq = (size_t)n * n * p->nEq * p->nEl;
  std::vector<double> G(nq), dS(nq);
  double dt = p->dt;
  for (int step = 0; step < nsteps; ++step) {
    double t0 = tn + step * dt;
    std::fill(G.begin(), G.end(), 0.0);
    for (int m = 0; m < 3; ++m) {
      double t = t0 + rk3_b[m] * dt;
      int rc = orc_dg_tendency(p, t, q, dS.data());
      if (rc) return rc;
      double a = rk3_a[m], gdt = rk3_g[m] * dt;
#pragma omp parallel for schedule(static)
      for (long long k = 0; k < (long long)nq; ++k) {
        G[k] = a * G[k] + dS[k];
        q[k] = q[k] + gdt * G[k];
      }
    }
  }
  return 0;
}

// CalculateBathymetryGradient (:1733-1868): weak DG derivative of h with the boundary values of h.
int orc_sw_bathymetry_gradient(const orc_dg_problem* p, double* dhdx, double* dhdy) {
  const int n = p->N + 1;
  Idx I{n, 1};
#pragma omp parallel for schedule(static)
  for (int e = 0; e < p->nEl; ++e) {
    std::vector<double> hb(4 * n), cf(2 * n), der(n), tend(2 * n * n);
    for (int j = 0; j < n; ++j) {
      double w = 0, ea = 0;
      for (int i = 0; i < n; ++i) w = w + p->lW[i] * p->h[I.f(i, j, e)];
      for (int i = 0; i < n; ++i) ea = ea + p->lE[i] * p->h[I.f(i, j, e)];
      hb[j + n * 3] = w;
      hb[j + n * 1] = ea;
    }
    for (int i = 0; i < n; ++i) {
      double s = 0, no = 0;
      for (int j = 0; j < n; ++j) s = s + p->lS[j] * p->h[I.f(i, j, e)];
      for (int j = 0; j < n; ++j) no = no + p->lN[j] * p->h[I.f(i, j, e)];
      hb[i + n * 0] = s;
      hb[i + n * 2] = no;
    }
    for (int j = 0; j < n; ++j) {
      for (int i = 0; i < n; ++i) {
        size_t id = I.f(i, j, e);
        double h = p->h[id];
        double xF[2] = {h, 0.0}, yF[2] = {0.0, h};
        for (int v = 0; v < 2; ++v) cf[i + n * v] = p->dydp[id] * xF[v] - p->dxdp[id] * yF[v];
      }
      double nv[2], len, fR[2], fL[2];
      nv[0] = p->nhx[I.nh(j, 1, e)];
      nv[1] = p->nhy[I.nh(j, 1, e)];
      len = p->nlen[I.nh(j, 1, e)];
      fR[0] = (hb[j + n * 1] * nv[0]) * len;
      fR[1] = (hb[j + n * 1] * nv[1]) * len;
      nv[0] = p->nhx[I.nh(j, 3, e)];
      nv[1] = p->nhy[I.nh(j, 3, e)];
      len = p->nlen[I.nh(j, 3, e)];
      fL[0] = (hb[j + n * 3] * nv[0]) * len;
      fL[1] = (hb[j + n * 3] * nv[1]) * len;
      for (int v = 0; v < 2; ++v) {
        dg_system_derivative(n, p->dmatS, p->qw, fL[v], fR[v], &cf[n * v], p->lW, p->lE, der.data());
        for (int i = 0; i < n; ++i) tend[i + n * (j + n * v)] = der[i];
      }
    }
    for (int i = 0; i < n; ++i) {
      for (int j = 0; j < n; ++j) {
        size_t id = I.f(i, j, e);
        double h = p->h[id];
        double xF[2] = {h, 0.0}, yF[2] = {0.0, h};
        for (int v = 0; v < 2; ++v) cf[j + n * v] = -p->dyds[id] * xF[v] + p->dxds[id] * yF[v];
      }
      double nv[2], len, fR[2], fL[2];
      nv[0] = p->nhx[I.nh(i, 2, e)];
      nv[1] = p->nhy[I.nh(i, 2, e)];
      len = p->nlen[I.nh(i, 2, e)];
      fR[0] = (hb[i + n * 2] * nv[0]) * len;
      fR[1] = (hb[i + n * 2] * nv[1]) * len;
      nv[0] = p->nhx[I.nh(i, 0, e)];
      nv[1] = p->nhy[I.nh(i, 0, e)];
      len = p->nlen[I.nh(i, 0, e)];
      fL[0] = (hb[i + n * 0] * nv[0]) * len;
      fL[1] = (hb[i + n * 0] * nv[1]) * len;
      for (int v = 0; v < 2; ++v) {
        dg_system_derivative(n, p->dmatP, p->qw, fL[v], fR[v], &cf[n * v], p->lS, p->lN, der.data());
        for (int j = 0; j < n; ++j) {
          double Jn = p->J[I.f(i, j, e)];
          tend[i + n * (j + n * v)] = (tend[i + n * (j + n * v)] + der[j]) / Jn;
        }
      }
    }
    for (int k = 0; k < n * n; ++k) {
      dhdx[(size_t)n * n * e + k] = tend[k];
      dhdy[(size_t)n * n * e + k] = tend[n * n + k];
    }
  }
  return 0;
}

}  // extern "C"
