// CPU oracle (test infrastructure): helpers shared by the oracle translation units.
#pragma once

#include <cmath>
#include <vector>

#include "oracle.h"

namespace orc {
bool almost_equal(double a, double b);
void barycentric(int nP, const double* x, double* bw);
void lagrange_at(int nP, const double* x, const double* bw, double xe, double* l);
double lagrange_eval(int nP, const double* x, const double* bw, double xe, const double* f);
double lagrange_deriv(int nP, const double* x, const double* bw, double xe, const double* f);
void derivative_matrix(int nP, const double* x, const double* bw, double* D);
// SetDirichletBoundaryCondition (CGsemElliptic_2D_Class.f90:234-301): dir values (0 when dir is null)
void cg_set_dirichlet(const orc_cg_problem* p, double* sol, const double* dir);

// CurveClass_2D of degree g on Chebyshev-Gauss-Lobatto nodes (CurveClass_2D.f90 Evaluate, EvaluateSlope)
struct CurveG {
  int g = 1;
  std::vector<double> s, bw, x, y;
  void nodes(int deg) {
    g = deg;
    s.assign(g + 1, 0.0);
    bw.assign(g + 1, 0.0);
    for (int j = 0; j <= g; ++j) s[j] = -std::cos((double)j * ((4.0 * std::atan(1.0)) / (double)g));
    barycentric(g, s.data(), bw.data());
    x.assign(g + 1, 0.0);
    y.assign(g + 1, 0.0);
  }
  void eval(double a, double& ox, double& oy) const {
    ox = lagrange_eval(g, s.data(), bw.data(), a, x.data());
    oy = lagrange_eval(g, s.data(), bw.data(), a, y.data());
  }
  void slope(double a, double& ox, double& oy) const {
    ox = lagrange_deriv(g, s.data(), bw.data(), a, x.data());
    oy = lagrange_deriv(g, s.data(), bw.data(), a, y.data());
  }
};

// TransfiniteInterpolation_2D / TransfiniteInterpolationMetrics_2D (GeometrySupportRoutines.f90) over four
// side curves (south, east, north, west); cov = dxds, dxdp, dyds, dydp
void tfi(const CurveG* c, double a, double b, double* P);
void tfi_metrics(const CurveG* c, double a, double b, double* cov);
}  // namespace orc
