// CPU oracle (test infrastructure): quadrature, Lagrange interpolation and the 2-D nodal storage.
// Restates src/interp/Legendre.f90, src/interp/Lagrange_1D_Class.f90 and
// src/nodal/NodalStorage_2D_Class.f90 of the reference, statement for statement.
#include <cmath>
#include <vector>

#include "oracle.h"
#include "oracle_internal.hpp"

namespace orc {

// ConstantsDictionary.f90:30-35,45
static const double kPi = 4.0 * std::atan(1.0);
static const double kTol = 2.220446049250313e-16;  // epsilon(1.0_prec)
static const int kItMax = 50;

// CommonRoutines.f90:58-96 AlmostEqual
bool almost_equal(double a, double b) {
  const double eps = 2.220446049250313e-16;
  if (a == 0.0 || b == 0.0) return std::fabs(a - b) <= eps;
  return (std::fabs(a - b) <= eps * std::fabs(a)) || (std::fabs(a - b) <= eps * std::fabs(b));
}

// Legendre.f90:63-114 LegendrePolynomial
static void legendre_polynomial(int nP, double x, double& l, double& dl) {
  if (nP == 0) {
    l = 1.0;
    dl = 0.0;
  } else if (nP == 1) {
    l = x;
    dl = 1.0;
  } else {
    double lm2 = 1.0, lm1 = x, dlm2 = 0.0, dlm1 = 1.0;
    for (int iP = 2; iP <= nP; ++iP) {
      double r = (double)iP;
      l = ((2.0 * r - 1.0) * x * lm1 - (r - 1.0) * lm2) / r;
      dl = dlm2 + (2.0 * r - 1.0) * lm1;
      lm2 = lm1;
      lm1 = l;
      dlm2 = dlm1;
      dlm1 = dl;
    }
  }
}

// Legendre.f90:118-172 LegendreQandL
static void legendre_q_and_l(int nP, double x, double& q, double& qprime, double& lN) {
  double lNm2 = 1.0, lNm1 = x, dlNm2 = 0.0, dlNm1 = 1.0, dlN = 0.0;
  lN = x;
  for (int iP = 2; iP <= nP; ++iP) {
    double r = (double)iP;
    lN = (2.0 * iP - 1.0) / r * x * lNm1 - (r - 1.0) / r * lNm2;
    dlN = dlNm2 + (2.0 * r - 1.0) * lNm1;
    lNm2 = lNm1;
    lNm1 = lN;
    dlNm2 = dlNm1;
    dlNm1 = dlN;
  }
  int iP = nP + 1;
  double r = (double)iP;
  double lNp1 = (2.0 * iP - 1.0) / r * x * lN - (r - 1.0) / r * lNm2;
  double dlNp1 = dlNm2 + (2.0 * r - 1.0) * lNm1;
  q = lNp1 - lNm2;
  qprime = dlNp1 - dlNm2;
}

// Legendre.f90:216-308 LegendreGauss.  The Newton stop test never fires for negative roots, so
// those always run kItMax iterations (reproduced as written).
static void legendre_gauss(int nP, double* x, double* w) {
  double l, dl;
  if (nP == 0) {
    x[0] = 0.0;
    w[0] = 2.0;
  } else if (nP == 1) {
    x[0] = -std::sqrt(1.0 / 3.0);
    w[0] = 1.0;
    x[1] = -x[0];
    w[1] = w[0];
  } else {
    for (int jX = 0; jX <= (nP + 1) / 2; ++jX) {
      x[jX] = -std::cos((2.0 * jX + 1.0) * kPi / (2.0 * nP + 1.0));
      for (int kIt = 1; kIt <= kItMax; ++kIt) {
        legendre_polynomial(nP + 1, x[jX], l, dl);
        double delta = -l / dl;
        x[jX] = x[jX] + delta;
        if (std::fabs(delta) <= kTol * x[jX]) break;
      }
      legendre_polynomial(nP + 1, x[jX], l, dl);
      w[jX] = 2.0 / ((1.0 - x[jX] * x[jX]) * dl * dl);
      w[nP - jX] = w[jX];
      x[nP - jX] = -x[jX];
    }
  }
  if (std::fmod((double)nP, 2.0) == 0.0) {
    legendre_polynomial(nP + 1, 0.0, l, dl);
    x[nP / 2] = 0.0;
    w[nP / 2] = 2.0 / (dl * dl);
  }
}

// Legendre.f90:312-405 LegendreGaussLobatto
static void legendre_gauss_lobatto(int nP, double* x, double* w) {
  double q, qp, lN;
  if (nP == 1) {
    x[0] = -1.0;
    w[0] = 1.0;
    x[1] = 1.0;
    w[1] = 1.0;
  } else {
    x[0] = -1.0;
    w[0] = 2.0 / ((double)nP * ((double)nP + 1.0));
    x[nP] = 1.0;
    w[nP] = w[0];
    for (int jX = 1; jX <= (nP + 1) / 2 - 1; ++jX) {
      x[jX] = -std::cos((jX + 0.25) * kPi / nP - 3.0 / (8.0 * nP * kPi * (jX + 0.25)));
      for (int kIt = 1; kIt <= kItMax; ++kIt) {
        legendre_q_and_l(nP, x[jX], q, qp, lN);
        double delta = -q / qp;
        x[jX] = x[jX] + delta;
        if (std::fabs(delta) <= kTol * x[jX]) break;
      }
      legendre_q_and_l(nP, x[jX], q, qp, lN);
      w[jX] = 2.0 / ((double)nP * ((double)nP + 1.0) * lN * lN);
      w[nP - jX] = w[jX];
      x[nP - jX] = -x[jX];
    }
  }
  if (std::fmod((double)nP, 2.0) == 0.0) {
    legendre_q_and_l(nP, 0.0, q, qp, lN);
    x[nP / 2] = 0.0;
    w[nP / 2] = 2.0 / ((double)nP * ((double)nP + 1.0) * lN * lN);
  }
}

// Lagrange_1D_Class.f90:349-392 CalculateBarycentricWeights_1D
void barycentric(int nP, const double* x, double* bw) {
  for (int j = 0; j <= nP; ++j) bw[j] = 1.0;
  for (int jP = 1; jP <= nP; ++jP)
    for (int kP = 0; kP <= jP - 1; ++kP) {
      bw[kP] = bw[kP] * (x[kP] - x[jP]);
      bw[jP] = bw[jP] * (x[jP] - x[kP]);
    }
  for (int jP = 0; jP <= nP; ++jP) bw[jP] = 1.0 / bw[jP];
}

// Lagrange_1D_Class.f90:448-515 EvaluateLagrangePolynomial_1D
void lagrange_at(int nP, const double* x, const double* bw, double xe, double* l) {
  bool match = false;
  for (int j = 0; j <= nP; ++j) {
    l[j] = 0.0;
    if (almost_equal(xe, x[j])) {
      l[j] = 1.0;
      match = true;
    }
  }
  if (match) return;
  double t1 = 0.0;
  for (int j = 0; j <= nP; ++j) {
    double t2 = bw[j] / (xe - x[j]);
    l[j] = t2;
    t1 = t1 + t2;
  }
  for (int j = 0; j <= nP; ++j) l[j] = l[j] / t1;
}

// Lagrange_1D_Class.f90:400-444 EvaluateLagrange_1D (interpolant value)
double lagrange_eval(int nP, const double* x, const double* bw, double xe, const double* f) {
  double num = 0.0, den = 0.0;
  for (int j = 0; j <= nP; ++j) {
    if (almost_equal(xe, x[j])) return f[j];
    double t = bw[j] / (xe - x[j]);
    num = num + t * f[j];
    den = den + t;
  }
  return num / den;
}

// Lagrange_1D_Class.f90:519-606 EvaluateDerivative_1D (interpolant derivative)
double lagrange_deriv(int nP, const double* x, const double* bw, double xe, const double* f) {
  double num = 0.0, den = 0.0, p = 0.0;
  int jS = -1;
  bool atNode = false;
  for (int j = 0; j <= nP; ++j) {
    if (almost_equal(xe, x[j])) {
      atNode = true;
      p = f[j];
      den = -bw[j];
      jS = j;
    }
  }
  if (atNode) {
    for (int j = 0; j <= nP; ++j)
      if (j != jS) num = num + bw[j] * (p - f[j]) / (xe - x[j]);
  } else {
    den = 0.0;
    p = lagrange_eval(nP, x, bw, xe, f);
    for (int j = 0; j <= nP; ++j) {
      double t = bw[j] / (xe - x[j]);
      num = num + t * (p - f[j]) / (xe - x[j]);
      den = den + t;
    }
  }
  return num / den;
}

// Lagrange_1D_Class.f90:612-689 CalculateDerivativeMatrix_1D (native nodes, negative sum trick)
void derivative_matrix(int nP, const double* x, const double* bw, double* D) {
  int n = nP + 1;
  for (int k = 0; k <= nP; ++k) {
    D[k + k * n] = 0.0;
    for (int j = 0; j <= nP; ++j) {
      if (j != k) {
        D[k + j * n] = bw[j] / (bw[k] * (x[k] - x[j]));
        D[k + k * n] = D[k + k * n] - D[k + j * n];
      }
    }
  }
}

}  // namespace orc

extern "C" {

int orc_legendre_quadrature(int N, int quad, double* x, double* w) {
  if (N < 0) return -1;
  if (quad == ORC_GAUSS_LOBATTO) {
    if (N < 1) return -1;
    orc::legendre_gauss_lobatto(N, x, w);
  } else if (quad == ORC_GAUSS) {
    orc::legendre_gauss(N, x, w);
  } else {
    return -1;
  }
  return 0;
}

int orc_barycentric_weights(int N, const double* x, double* bw) {
  orc::barycentric(N, x, bw);
  return 0;
}

int orc_derivative_matrix(int N, const double* x, double* D) {
  std::vector<double> bw(N + 1);
  orc::barycentric(N, x, bw.data());
  orc::derivative_matrix(N, x, bw.data(), D);
  return 0;
}

int orc_lagrange_at(int N, const double* x, double xe, double* l) {
  std::vector<double> bw(N + 1);
  orc::barycentric(N, x, bw.data());
  orc::lagrange_at(N, x, bw.data(), xe, l);
  return 0;
}

// NodalStorage_2D_Class.f90:101-230 BuildNodalStorage_2D (nS = nP = N)
int orc_nodal_build(int N, int quad, int form, int quirk_dmatp, double* x, double* w, double* dmatS,
                    double* dmatP, double* lW, double* lE, double* lS, double* lN) {
  int n = N + 1;
  if (orc_legendre_quadrature(N, quad, x, w) != 0) return -1;
  std::vector<double> bw(n), D(n * n);
  orc::barycentric(N, x, bw.data());
  orc::lagrange_at(N, x, bw.data(), -1.0, lW);
  orc::lagrange_at(N, x, bw.data(), 1.0, lE);
  orc::lagrange_at(N, x, bw.data(), -1.0, lS);
  orc::lagrange_at(N, x, bw.data(), 1.0, lN);
  orc::derivative_matrix(N, x, bw.data(), D.data());
  if (form == ORC_CG) {
    for (int k = 0; k < n * n; ++k) {
      dmatS[k] = D[k];
      dmatP[k] = D[k];
    }
  } else if (form == ORC_DG) {
    // dMatS(i,j) = -D(j,i) w_j / w_i   (:199-207)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) dmatS[i + j * n] = -D[j + i * n] * w[j] / w[i];
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        if (quirk_dmatp) {
          // :209-218 as shipped: dMatP(j,i) = -D(j,i) w_j / w_i  (transpose of the s-direction matrix)
          dmatP[j + i * n] = -D[j + i * n] * w[j] / w[i];
        } else {
          // the weak-derivative matrix of the 1-D and 3-D classes (NodalStorage_1D_Class.f90:175)
          dmatP[i + j * n] = -D[j + i * n] * w[j] / w[i];
        }
      }
  } else {
    return -1;
  }
  return 0;
}

}  // extern "C"
