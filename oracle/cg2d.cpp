// CPU oracle (test infrastructure): CGSEM 2-D operator, direct-stiffness summation, masks, PCG and GMRES.
// Restates src/cgsem/CGsemElliptic_2D_Class.f90 (SetDirichletBoundaryCondition :234-301, Mask :350-430,
// MaskSide :434-466, UnMask :470-542, UnMaskSide :546-613, GlobalSum :617-702, SumSide :706-787,
// CalculateGradient :791-850, FluxDivergence :854-926, MatrixAction :930-976, Residual :980-1068,
// DotProduct :1072-1110, Solve_PCConjugateGradient :1114-1207), the GMRES(m) of
// src/highend/Stommel/Stommel_Class.f90 :1161-1322 (= IterativeSolvers_Class.f90 :493-652 on
// element-local vectors) and Solve_PCGMRES (IterativeSolvers_Class.f90 :656-822) with Jacobi.
// Documented decisions (not restatements):
//  * Mask_CGsemElliptic_2D tests an uninitialised eID (:385-391); the secondary side of every
//    interior edge is masked, the evident intent;
//  * the operator gains a mass term: Lu -= lambda*J*w_i*w_j*u (sign of the reference's -K);
//  * op 1 adds the advection term: Lu -= J*w_i*w_j*(vx*ux + vy*uy) (Galerkin GLL form);
//  * Jacobi preconditioner: w = r / assembled diagonal (new; the reference uses a linear-FEM inner CG);
//  * ioerr = 0 on convergence (the reference leaves ioerr = -2 because "ioerr = 0" follows EXIT).
#include <cmath>
#include <cstring>
#include <vector>

#include "oracle.h"
#include "oracle_internal.hpp"

namespace {

struct CGIdx {
  int n;
  size_t f(int i, int j, int e) const { return (size_t)i + n * (j + (size_t)n * e); }
};

// sideMap (QuadMeshClass.f90:191): S -> iP=0, E -> iS=N, N -> iP=N, W -> iS=0
inline void side_node(int side /*1..4*/, int k, int N, int& i, int& j) {
  switch (side) {
    case 1: i = k; j = 0; break;
    case 2: i = N; j = k; break;
    case 3: i = k; j = N; break;
    default: i = 0; j = k; break;
  }
}
// cornerMap (QuadMeshClass.f90:192-193)
inline void corner_node(int c /*1..4*/, int N, int& i, int& j) {
  static const int ci[4] = {0, 1, 1, 0}, cj[4] = {0, 0, 1, 1};
  i = ci[c - 1] * N;
  j = cj[c - 1] * N;
}

void mask_side(const orc_cg_problem* p, int e /*1-based*/, int s, double* u) {
  CGIdx I{p->N + 1};
  int si = std::abs(s);
  for (int k = 1; k <= p->N - 1; ++k) {
    int i, j;
    side_node(si, k, p->N, i, j);
    u[I.f(i, j, e - 1)] = 0.0;
  }
}

}  // namespace

extern "C" {

int orc_cg_mask(const orc_cg_problem* p, double* u) {
  CGIdx I{p->N + 1};
  for (int k = 0; k < p->nEdges; ++k) {
    const int* E = p->edges + 6 * k;
    if (E[2] == ORC_DIRICHLET) {
      mask_side(p, E[0], E[1], u);
    } else if (E[2] > 0) {
      mask_side(p, E[2], E[3], u);
    }
  }
  for (int nd = 0; nd < p->nNodes; ++nd) {
    int a = p->n2e_ptr[nd], b = p->n2e_ptr[nd + 1];
    if (p->nodeType[nd] != ORC_DIRICHLET) a += 1;  // keep the first element's copy
    for (int c = a; c < b; ++c) {
      int i, j;
      corner_node(p->n2e_local[c], p->N, i, j);
      u[I.f(i, j, p->n2e_elem[c] - 1)] = 0.0;
    }
  }
  return 0;
}

int orc_cg_unmask(const orc_cg_problem* p, double* u) {
  CGIdx I{p->N + 1};
  const int N = p->N;
  for (int k = 0; k < p->nEdges; ++k) {
    const int* E = p->edges + 6 * k;
    if (E[2] <= 0) continue;
    double temp[64];
    for (int m = 1; m <= N - 1; ++m) {
      int i, j;
      side_node(E[1], m, N, i, j);
      temp[m] = u[I.f(i, j, E[0] - 1)];
    }
    int jj = E[4];
    for (int m = 1; m <= N - 1; ++m) {
      int i, j;
      side_node(std::abs(E[3]), jj, N, i, j);
      u[I.f(i, j, E[2] - 1)] = temp[m];
      jj = jj + E[5];
    }
  }
  for (int nd = 0; nd < p->nNodes; ++nd) {
    if (p->nodeType[nd] == ORC_DIRICHLET) continue;
    int a = p->n2e_ptr[nd], b = p->n2e_ptr[nd + 1];
    int i0, j0;
    corner_node(p->n2e_local[a], N, i0, j0);
    double v0 = u[I.f(i0, j0, p->n2e_elem[a] - 1)];
    for (int c = a + 1; c < b; ++c) {
      int i, j;
      corner_node(p->n2e_local[c], N, i, j);
      u[I.f(i, j, p->n2e_elem[c] - 1)] = v0;
    }
  }
  return 0;
}

int orc_cg_global_sum(const orc_cg_problem* p, double* u) {
  CGIdx I{p->N + 1};
  const int N = p->N;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < p->nEdges; ++k) {
    const int* E = p->edges + 6 * k;
    if (E[2] <= 0) continue;
    int e[2] = {E[0], E[2]}, s[2] = {E[1], std::abs(E[3])};
    double temp[2][64];
    for (int c = 0; c < 2; ++c)
      for (int m = 1; m <= N - 1; ++m) {
        int i, j;
        side_node(s[c], m, N, i, j);
        temp[c][m] = u[I.f(i, j, e[c] - 1)];
      }
    int nn = E[4];
    for (int m = 1; m <= N - 1; ++m) {
      double sum = temp[0][m] + temp[1][nn];
      temp[0][m] = sum;
      temp[1][nn] = sum;
      nn = nn + E[5];
    }
    for (int c = 0; c < 2; ++c)
      for (int m = 1; m <= N - 1; ++m) {
        int i, j;
        side_node(s[c], m, N, i, j);
        u[I.f(i, j, e[c] - 1)] = temp[c][m];
      }
  }
#pragma omp parallel for schedule(static)
  for (int nd = 0; nd < p->nNodes; ++nd) {
    if (p->nodeType[nd] == ORC_DIRICHLET) continue;
    int a = p->n2e_ptr[nd], b = p->n2e_ptr[nd + 1];
    double sum = 0.0;
    for (int c = a; c < b; ++c) {
      int i, j;
      corner_node(p->n2e_local[c], N, i, j);
      sum = sum + u[I.f(i, j, p->n2e_elem[c] - 1)];
    }
    for (int c = a; c < b; ++c) {
      int i, j;
      corner_node(p->n2e_local[c], N, i, j);
      u[I.f(i, j, p->n2e_elem[c] - 1)] = sum;
    }
  }
  return 0;
}

// FluxDivergence (+ CalculateGradient) of one element, with the documented mass/advection additions
static void local_op(const orc_cg_problem* p, int e, const double* u, double* Lu) {
  const int n = p->N + 1;
  CGIdx I{n};
  const double* D = p->dmat;
  const double* w = p->qw;
  double us[256], up[256], ux[256], uy[256], F1[256], F2[256], d1[256], d2[256];
  const double* ue = u + (size_t)n * n * e;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      double s = 0.0;
      for (int m = 0; m < n; ++m) s = s + D[i + m * n] * ue[m + n * j];
      us[i + n * j] = s;
    }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double s = 0.0;
      for (int m = 0; m < n; ++m) s = s + D[j + m * n] * ue[i + n * m];
      up[i + n * j] = s;
    }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      size_t id = I.f(i, j, e);
      double Jn = p->J[id];
      ux[i + n * j] = (p->dydp[id] * us[i + n * j] - p->dyds[id] * up[i + n * j]) / Jn;
      uy[i + n * j] = (p->dxds[id] * up[i + n * j] - p->dxdp[id] * us[i + n * j]) / Jn;
    }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      size_t id = I.f(i, j, e);
      double k = p->kcoef[id];
      F1[i + n * j] = k * (ux[i + n * j] * p->dydp[id] - uy[i + n * j] * p->dxdp[id]) * w[i];
      F2[i + n * j] = k * (uy[i + n * j] * p->dxds[id] - ux[i + n * j] * p->dyds[id]) * w[j];
    }
  // MATMUL( TRANSPOSE(dMat), F )
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      double s = 0.0;
      for (int m = 0; m < n; ++m) s = s + D[m + i * n] * F1[m + n * j];
      d1[i + n * j] = s;
    }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double s = 0.0;
      for (int m = 0; m < n; ++m) s = s + D[m + j * n] * F2[i + n * m];
      d2[i + n * j] = s;
    }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      size_t id = I.f(i, j, e);
      double r = -(d1[i + n * j] * w[j] + d2[i + n * j] * w[i]);
      double mw = p->J[id] * w[i] * w[j];
      if (p->lambda != 0.0) r = r - p->lambda * mw * ue[i + n * j];
      if (p->op == 1) r = r - mw * (p->vx * ux[i + n * j] + p->vy * uy[i + n * j]);
      Lu[(size_t)n * n * e + i + n * j] = r;
    }
}

int orc_cg_local_operator(const orc_cg_problem* p, const double* u, double* Lu) {
  if (p->N + 1 > 16) return -1;
#pragma omp parallel for schedule(static)
  for (int e = 0; e < p->nEl; ++e) local_op(p, e, u, Lu);
  return 0;
}

int orc_cg_matrix_action(const orc_cg_problem* p, double* u, double* Au) {
  orc_cg_unmask(p, u);
  int rc = orc_cg_local_operator(p, u, Au);
  if (rc) return rc;
  orc_cg_global_sum(p, Au);
  orc_cg_mask(p, Au);
  orc_cg_mask(p, u);
  return 0;
}

}  // extern "C"

namespace orc {
void cg_set_dirichlet(const orc_cg_problem* p, double* sol, const double* dir) {
  CGIdx I{p->N + 1};
  const int N = p->N;
  for (int k = 0; k < p->nEdges; ++k) {
    const int* E = p->edges + 6 * k;
    if (E[2] != ORC_DIRICHLET) continue;
    for (int m = 1; m <= N - 1; ++m) {
      int i, j;
      side_node(E[1], m, N, i, j);
      size_t id = I.f(i, j, E[0] - 1);
      sol[id] = dir ? dir[id] : 0.0;
    }
  }
  for (int nd = 0; nd < p->nNodes; ++nd) {
    if (p->nodeType[nd] != ORC_DIRICHLET) continue;
    for (int c = p->n2e_ptr[nd]; c < p->n2e_ptr[nd + 1]; ++c) {
      int i, j;
      corner_node(p->n2e_local[c], N, i, j);
      size_t id = I.f(i, j, p->n2e_elem[c] - 1);
      sol[id] = dir ? dir[id] : 0.0;
    }
  }
}
}  // namespace orc

extern "C" {

int orc_cg_residual(const orc_cg_problem* p, const double* source, double* solution, const double* dir,
                    double* r) {
  const int n = p->N + 1;
  size_t nl = (size_t)n * n * p->nEl;
  std::vector<double> Au(nl);
  int rc = orc_cg_matrix_action(p, solution, Au.data());
  if (rc) return rc;
  for (int e = 0; e < p->nEl; ++e)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        size_t id = (size_t)i + n * (j + (size_t)n * e);
        r[id] = source[id] * p->J[id] * p->qw[i] * p->qw[j] - Au[id];
      }
  orc_cg_global_sum(p, r);
  orc_cg_mask(p, r);
  orc_cg_mask(p, solution);
  orc::cg_set_dirichlet(p, solution, dir);
  return 0;
}

double orc_cg_dot(const orc_cg_problem* p, double* u, double* v) {
  orc_cg_mask(p, u);
  orc_cg_mask(p, v);
  const int n = p->N + 1;
  double s = 0.0;
  for (int e = 0; e < p->nEl; ++e)
    for (int j = 0; j < n; ++j) {
      double d = 0.0;
      for (int i = 0; i < n; ++i) {
        size_t id = (size_t)i + n * (j + (size_t)n * e);
        d = d + u[id] * v[id];
      }
      s = s + d;
    }
  return s;
}

// Assembled diagonal of the operator, closed form of the local operator applied to unit vectors,
// then summed over shared copies.  Masked positions hold 1.
int orc_cg_jacobi_diagonal(const orc_cg_problem* p, double* diag) {
  const int n = p->N + 1;
  const double* D = p->dmat;
  const double* w = p->qw;
#pragma omp parallel for schedule(static)
  for (int e = 0; e < p->nEl; ++e) {
    for (int b = 0; b < n; ++b)
      for (int a = 0; a < n; ++a) {
        size_t id = (size_t)a + n * (b + (size_t)n * e);
        double s1 = 0.0, s2 = 0.0;
        for (int k = 0; k < n; ++k) {  // sum over s at fixed p = b
          size_t ik = (size_t)k + n * (b + (size_t)n * e);
          double c1 = p->kcoef[ik] * w[k] * (p->dydp[ik] * p->dydp[ik] + p->dxdp[ik] * p->dxdp[ik]) / p->J[ik];
          s1 = s1 + D[k + a * n] * D[k + a * n] * c1;
        }
        for (int k = 0; k < n; ++k) {  // sum over p at fixed s = a
          size_t ik = (size_t)a + n * (k + (size_t)n * e);
          double c2 = p->kcoef[ik] * w[k] * (p->dxds[ik] * p->dxds[ik] + p->dyds[ik] * p->dyds[ik]) / p->J[ik];
          s2 = s2 + D[k + b * n] * D[k + b * n] * c2;
        }
        double cross = -p->kcoef[id] * (p->dyds[id] * p->dydp[id] + p->dxds[id] * p->dxdp[id]) / p->J[id];
        double dd = D[a + a * n] * D[b + b * n];
        double val = -(w[b] * (s1 + dd * cross * w[a]) + w[a] * (s2 + dd * cross * w[b]));
        double mw = p->J[id] * w[a] * w[b];
        val = val - p->lambda * mw;
        if (p->op == 1) {
          double uxd = (p->dydp[id] * D[a + a * n] - p->dyds[id] * D[b + b * n]) / p->J[id];
          double uyd = (p->dxds[id] * D[b + b * n] - p->dxdp[id] * D[a + a * n]) / p->J[id];
          val = val - mw * (p->vx * uxd + p->vy * uyd);
        }
        diag[id] = val;
      }
  }
  orc_cg_global_sum(p, diag);
  const size_t nl = (size_t)n * n * p->nEl;
  std::vector<double> one(nl, 1.0);
  orc_cg_mask(p, one.data());
  for (size_t k = 0; k < nl; ++k)
    if (one[k] == 0.0) diag[k] = 1.0;
  return 0;
}

int orc_cg_solve_pcg(const orc_cg_problem* p, const double* source, double* solution, const double* dir,
                     int maxIters, double tol, int precond, double* resi, int* iters) {
  const int n = p->N + 1;
  const size_t nl = (size_t)n * n * p->nEl;
  std::vector<double> u(nl), r(nl), v(nl), z(nl), w(nl), diag;
  if (precond == 1) {
    diag.resize(nl);
    orc_cg_jacobi_diagonal(p, diag.data());
  }
  if (dir) orc::cg_set_dirichlet(p, solution, dir);
  int ioerr = -2;
  std::memcpy(u.data(), solution, nl * sizeof(double));
  int rc = orc_cg_residual(p, source, solution, dir, r.data());
  if (rc) return rc;
  double r0 = std::sqrt(orc_cg_dot(p, r.data(), r.data()));
  for (int k = 0; k <= maxIters; ++k) resi[k] = 0.0;
  resi[0] = r0;
  double rNorm = r0, num = 0, den = 0, a, b;
  *iters = 0;
  if (r0 < tol) return 0;
  for (int iter = 1; iter <= maxIters; ++iter) {
    orc_cg_unmask(p, r.data());
    if (precond == 1) {
      for (size_t k = 0; k < nl; ++k) w[k] = r[k] / diag[k];
    } else {
      std::memcpy(w.data(), r.data(), nl * sizeof(double));
    }
    num = orc_cg_dot(p, r.data(), w.data());
    if (iter == 1) {
      std::memcpy(v.data(), w.data(), nl * sizeof(double));
    } else {
      b = num / den;
      for (size_t k = 0; k < nl; ++k) v[k] = w[k] + b * v[k];
    }
    orc_cg_matrix_action(p, v.data(), z.data());
    a = num / orc_cg_dot(p, v.data(), z.data());
    for (size_t k = 0; k < nl; ++k) u[k] = u[k] + a * v[k];
    for (size_t k = 0; k < nl; ++k) r[k] = r[k] - a * z[k];
    den = num;
    rNorm = std::sqrt(orc_cg_dot(p, r.data(), r.data()));
    resi[iter] = rNorm;
    *iters = iter;
    if (rNorm / r0 < tol) {
      ioerr = 0;
      break;
    }
  }
  if (rNorm / r0 > tol) ioerr = -1;
  orc_cg_unmask(p, u.data());
  std::memcpy(solution, u.data(), nl * sizeof(double));
  orc::cg_set_dirichlet(p, solution, dir);
  return ioerr;
}

int orc_cg_solve_gmres(const orc_cg_problem* p, const double* source, double* solution, const double* dir,
                       int m, int maxIters, double tol, double* resi, int* iters) {
  const int n = p->N + 1;
  const size_t nl = (size_t)n * n * p->nEl;
  std::vector<double> r(nl, 0.0), w(nl), V(nl * (m + 1), 0.0);
  std::vector<double> rho(m * m, 0.0), h((m + 1) * m, 0.0), c(m, 0.0), s(m, 0.0), bhat(m + 1, 0.0), y(m + 1, 0.0);
  auto RHO = [&](int i, int j) -> double& { return rho[(i - 1) + m * (j - 1)]; };
  auto H = [&](int i, int j) -> double& { return h[(i - 1) + (m + 1) * (j - 1)]; };
  if (dir) orc::cg_set_dirichlet(p, solution, dir);
  int ioerr = -2;
  int rc = orc_cg_residual(p, source, solution, dir, r.data());
  if (rc) return rc;
  double r0 = std::sqrt(orc_cg_dot(p, r.data(), r.data()));
  int l = 0;
  for (int k = 0; k <= maxIters; ++k) resi[k] = 0.0;
  resi[0] = r0;
  double rcur = r0;
  *iters = 0;
  if (r0 == 0.0) return 0;
  for (int j = 1; j <= maxIters; ++j) {
    double b = std::sqrt(orc_cg_dot(p, r.data(), r.data()));
    for (size_t k = 0; k < nl; ++k) V[k] = r[k] / b;
    bhat[0] = b;
    int nr = 0;
    for (int i = 1; i <= m; ++i) {
      l = l + 1;
      nr = i;
      double* vi = &V[nl * (i - 1)];
      orc_cg_matrix_action(p, vi, w.data());
      for (int k = 1; k <= i; ++k) {
        double* vk = &V[nl * (k - 1)];
        H(k, i) = orc_cg_dot(p, vk, w.data());
        double hk = H(k, i);
        for (size_t q = 0; q < nl; ++q) w[q] = w[q] - hk * vk[q];
      }
      H(i + 1, i) = std::sqrt(orc_cg_dot(p, w.data(), w.data()));
      if (orc::almost_equal(H(i + 1, i), 0.0)) break;
      double* vn = &V[nl * i];
      double hn = H(i + 1, i);
      for (size_t q = 0; q < nl; ++q) vn[q] = w[q] / hn;
      RHO(1, i) = H(1, i);
      for (int k = 2; k <= i; ++k) {
        double g = c[k - 2] * RHO(k - 1, i) + s[k - 2] * H(k, i);
        RHO(k, i) = -s[k - 2] * RHO(k - 1, i) + c[k - 2] * H(k, i);
        RHO(k - 1, i) = g;
      }
      double d = std::sqrt(std::pow(RHO(i, i), 2) + std::pow(H(i + 1, i), 2));
      c[i - 1] = RHO(i, i) / d;
      s[i - 1] = H(i + 1, i) / d;
      RHO(i, i) = c[i - 1] * RHO(i, i) + s[i - 1] * H(i + 1, i);
      bhat[i] = -s[i - 1] * bhat[i - 1];
      bhat[i - 1] = c[i - 1] * bhat[i - 1];
      rcur = std::fabs(bhat[i]);
      if (l <= maxIters) resi[l] = rcur;
      if (rcur / r0 <= tol) break;
    }
    if (rcur / r0 > tol) nr = m;
    y[nr - 1] = bhat[nr - 1] / RHO(nr, nr);
    for (int k = nr - 1; k >= 1; --k) {
      y[k - 1] = bhat[k - 1];
      for (int i = k + 1; i <= nr; ++i) y[k - 1] = y[k - 1] - RHO(k, i) * y[i - 1];
      y[k - 1] = y[k - 1] / RHO(k, k);
    }
    for (size_t q = 0; q < nl; ++q) {
      double dd = 0.0;
      for (int k = 1; k <= nr; ++k) dd = dd + V[q + nl * (k - 1)] * y[k - 1];
      solution[q] = solution[q] + dd;
    }
    *iters = l;
    if (rcur / r0 <= tol) {
      ioerr = 0;
      break;
    }
    rc = orc_cg_residual(p, source, solution, dir, r.data());
    if (rc) return rc;
  }
  if (rcur / r0 > tol) ioerr = -1;
  orc_cg_unmask(p, solution);
  orc::cg_set_dirichlet(p, solution, dir);
  return ioerr;
}

// Solve_PCGMRES (IterativeSolvers_Class.f90:656-822): flexible GMRES(m) with variable right preconditioning;
// PreconditionInvert = Jacobi (z = v / assembled diagonal, 1 on masked nodes).  The preconditioned basis Z is
// kept and the update is sol += Z y.
int orc_cg_solve_pgmres(const orc_cg_problem* p, const double* source, double* solution, const double* dir, int m,
                        int maxIters, double tol, double* resi, int* iters) {
  const int n = p->N + 1;
  const size_t nl = (size_t)n * n * p->nEl;
  std::vector<double> r(nl, 0.0), w(nl), V(nl * (m + 1), 0.0), Z(nl * (m + 1), 0.0), diag(nl);
  std::vector<double> rho(m * m, 0.0), h((m + 1) * m, 0.0), c(m, 0.0), s(m, 0.0), bhat(m + 1, 0.0), y(m + 1, 0.0);
  auto RHO = [&](int i, int j) -> double& { return rho[(i - 1) + m * (j - 1)]; };
  auto H = [&](int i, int j) -> double& { return h[(i - 1) + (m + 1) * (j - 1)]; };
  orc_cg_jacobi_diagonal(p, diag.data());
  if (dir) orc::cg_set_dirichlet(p, solution, dir);
  int ioerr = -2;
  int rc = orc_cg_residual(p, source, solution, dir, r.data());
  if (rc) return rc;
  double r0 = std::sqrt(orc_cg_dot(p, r.data(), r.data()));
  int l = 0;
  for (int k = 0; k <= maxIters; ++k) resi[k] = 0.0;
  resi[0] = r0;
  double rcur = r0;
  *iters = 0;
  if (r0 == 0.0) return 0;
  for (int j = 1; j <= maxIters; ++j) {
    double b = std::sqrt(orc_cg_dot(p, r.data(), r.data()));
    for (size_t k = 0; k < nl; ++k) V[k] = r[k] / b;
    bhat[0] = b;
    int nr = 0;
    for (int i = 1; i <= m; ++i) {
      l = l + 1;
      nr = i;
      double* vi = &V[nl * (i - 1)];
      double* zi = &Z[nl * (i - 1)];
      for (size_t q = 0; q < nl; ++q) zi[q] = vi[q] / diag[q];  // PreconditionInvert
      orc_cg_matrix_action(p, zi, w.data());
      for (int k = 1; k <= i; ++k) {
        double* vk = &V[nl * (k - 1)];
        H(k, i) = orc_cg_dot(p, vk, w.data());
        double hk = H(k, i);
        for (size_t q = 0; q < nl; ++q) w[q] = w[q] - hk * vk[q];
      }
      H(i + 1, i) = std::sqrt(orc_cg_dot(p, w.data(), w.data()));
      if (orc::almost_equal(H(i + 1, i), 0.0)) break;
      double* vn = &V[nl * i];
      double hn = H(i + 1, i);
      for (size_t q = 0; q < nl; ++q) vn[q] = w[q] / hn;
      RHO(1, i) = H(1, i);
      for (int k = 2; k <= i; ++k) {
        double g = c[k - 2] * RHO(k - 1, i) + s[k - 2] * H(k, i);
        RHO(k, i) = -s[k - 2] * RHO(k - 1, i) + c[k - 2] * H(k, i);
        RHO(k - 1, i) = g;
      }
      double d = std::sqrt(std::pow(RHO(i, i), 2) + std::pow(H(i + 1, i), 2));
      c[i - 1] = RHO(i, i) / d;
      s[i - 1] = H(i + 1, i) / d;
      RHO(i, i) = c[i - 1] * RHO(i, i) + s[i - 1] * H(i + 1, i);
      bhat[i] = -s[i - 1] * bhat[i - 1];
      bhat[i - 1] = c[i - 1] * bhat[i - 1];
      rcur = std::fabs(bhat[i]);
      if (l <= maxIters) resi[l] = rcur;
      if (rcur / r0 <= tol) break;
    }
    if (rcur / r0 > tol) nr = m;
    y[nr - 1] = bhat[nr - 1] / RHO(nr, nr);
    for (int k = nr - 1; k >= 1; --k) {
      y[k - 1] = bhat[k - 1];
      for (int i = k + 1; i <= nr; ++i) y[k - 1] = y[k - 1] - RHO(k, i) * y[i - 1];
      y[k - 1] = y[k - 1] / RHO(k, k);
    }
    for (size_t q = 0; q < nl; ++q) {
      double dd = 0.0;
      for (int k = 1; k <= nr; ++k) dd = dd + Z[q + nl * (k - 1)] * y[k - 1];
      solution[q] = solution[q] + dd;
    }
    *iters = l;
    if (rcur / r0 <= tol) {
      ioerr = 0;
      break;
    }
    rc = orc_cg_residual(p, source, solution, dir, r.data());
    if (rc) return rc;
  }
  if (rcur / r0 > tol) ioerr = -1;
  orc_cg_unmask(p, solution);
  orc::cg_set_dirichlet(p, solution, dir);
  return ioerr;
}

}  // extern "C"
