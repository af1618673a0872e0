// CPU oracle (test infrastructure): helpers shared by the oracle translation units.
#pragma once

namespace orc {
bool almost_equal(double a, double b);
void barycentric(int nP, const double* x, double* bw);
void lagrange_at(int nP, const double* x, const double* bw, double xe, double* l);
double lagrange_eval(int nP, const double* x, const double* bw, double xe, const double* f);
double lagrange_deriv(int nP, const double* x, const double* bw, double xe, const double* f);
void derivative_matrix(int nP, const double* x, const double* bw, double* D);
}  // namespace orc
