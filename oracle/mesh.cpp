// CPU oracle (test infrastructure): structured quadrilateral mesh, edge table and mapped geometry.
// Restates src/geom/QuadMeshClass.f90 (LoadDefaultMesh :1718-1859, ConstructEdges :1489-1627,
// GetNodeToElementConnectivity, ScaleTheMesh :1691-1714), src/geom/MappedGeometryClass_2D.f90
// (GenerateMesh :536-607, GenerateMetrics :611-710, GenerateBoundaryMetrics :714-788,
// CalculateMetrics :813-833, ScaleGeometry :921-948), src/geom/GeometrySupportRoutines.f90
// (TransfiniteInterpolation_2D :60-105, TransfiniteInterpolationMetrics_2D :109-158) and
// src/geom/CurveClass_2D.f90 (Evaluate/EvaluateSlope with Chebyshev-Gauss-Lobatto curve nodes).
//
// Additions that the reference does not have (documented decisions, not restatements):
//  * periodic connectivity: opposite boundary corner nodes share an ID, so ConstructEdges pairs the
//    opposite sides exactly as it pairs interior sides;
//  * a smooth warp x <- x + A sin(2 pi x) sin(2 pi y), y <- y + A sin(2 pi x) sin(2 pi y) of the unit
//    square.  For a warped mesh the interior covariant metrics are the derivative of the degree-N
//    interpolant of the node positions (the INTERP_METRICS option of ModelFlags.f90); the
//    straight-sided mesh keeps the reference's transfinite metrics.
#include <cmath>
#include <cstring>
#include <map>
#include <utility>
#include <vector>

#include "oracle.h"
#include "oracle_internal.hpp"

namespace {

const double kPi = 4.0 * std::atan(1.0);
// QuadMeshClass.f90:191-195
const int kEdgeMap[2][4] = {{1, 2, 4, 1}, {2, 3, 3, 4}};

struct Curve {  // CurveClass_2D with gPolyDeg = 1 and Chebyshev-Gauss-Lobatto nodes (-1, 1)
  double s[2], bw[2], x[2], y[2];
  void build(double x1, double y1, double x2, double y2) {
    s[0] = -std::cos(0.0 * (kPi / 1.0));  // Chebyshev.f90:124-130
    s[1] = -std::cos(1.0 * (kPi / 1.0));
    orc::barycentric(1, s, bw);
    for (int i = 0; i < 2; ++i) {
      x[i] = x1 + (x2 - x1) * 0.5 * (s[i] + 1.0);
      y[i] = y1 + (y2 - y1) * 0.5 * (s[i] + 1.0);
    }
  }
  void eval(double a, double& ox, double& oy) const {
    ox = orc::lagrange_eval(1, s, bw, a, x);
    oy = orc::lagrange_eval(1, s, bw, a, y);
  }
  void slope(double a, double& ox, double& oy) const {
    ox = orc::lagrange_deriv(1, s, bw, a, x);
    oy = orc::lagrange_deriv(1, s, bw, a, y);
  }
};

inline void uni(const double* l, const double* r, double a, double* p) {  // Unidirectional_2D
  p[0] = 0.5 * ((1.0 - a) * l[0] + (1.0 + a) * r[0]);
  p[1] = 0.5 * ((1.0 - a) * l[1] + (1.0 + a) * r[1]);
}
inline void unid(const double* l, const double* r, double* p) {  // UnidirectionalDerivative_2D
  p[0] = 0.5 * (r[0] - l[0]);
  p[1] = 0.5 * (r[1] - l[1]);
}

void tfi(const Curve* c, double a, double b, double* P) {
  double c1[2], c2[2], c3[2], c4[2], lc[2], rc[2], P1[2], P2[2], Ps[2], Pn[2], Q[2];
  c[0].eval(-1.0, c1[0], c1[1]);
  c[0].eval(1.0, c2[0], c2[1]);
  c[2].eval(-1.0, c3[0], c3[1]);
  c[2].eval(1.0, c4[0], c4[1]);
  c[3].eval(b, lc[0], lc[1]);
  c[1].eval(b, rc[0], rc[1]);
  uni(lc, rc, a, P1);
  c[0].eval(a, lc[0], lc[1]);
  c[2].eval(a, rc[0], rc[1]);
  uni(lc, rc, b, P2);
  uni(c1, c2, a, Ps);
  uni(c3, c4, a, Pn);
  uni(Ps, Pn, b, Q);
  P[0] = P1[0] + P2[0] - Q[0];
  P[1] = P1[1] + P2[1] - Q[1];
}

// returns covT: [0]=dxds [1]=dxdp [2]=dyds [3]=dydp
void tfi_metrics(const Curve* c, double a, double b, double* cov) {
  double wc[2], ec[2], sc[2], nc[2], dw[2], de[2], ds[2], dn[2], c1[2], c2[2], c3[2], c4[2];
  double P1[2], P2[2], Ps[2], Pn[2], Pw[2], Pe[2], t1[2], t2[2], U[2];
  c[3].eval(b, wc[0], wc[1]);
  c[1].eval(b, ec[0], ec[1]);
  c[0].eval(a, sc[0], sc[1]);
  c[2].eval(a, nc[0], nc[1]);
  c[3].slope(b, dw[0], dw[1]);
  c[1].slope(b, de[0], de[1]);
  c[0].slope(a, ds[0], ds[1]);
  c[2].slope(a, dn[0], dn[1]);
  c[0].eval(-1.0, c1[0], c1[1]);
  c[0].eval(1.0, c2[0], c2[1]);
  c[2].eval(-1.0, c3[0], c3[1]);
  c[2].eval(1.0, c4[0], c4[1]);
  unid(wc, ec, P1);
  unid(c1, c2, Ps);
  unid(c3, c4, Pn);
  t1[0] = ds[0] - Ps[0];
  t1[1] = ds[1] - Ps[1];
  t2[0] = dn[0] - Pn[0];
  t2[1] = dn[1] - Pn[1];
  uni(t1, t2, b, U);
  cov[0] = P1[0] + U[0];
  cov[2] = P1[1] + U[1];
  unid(sc, nc, P2);
  unid(c1, c3, Pw);
  unid(c2, c4, Pe);
  t1[0] = dw[0] - Pw[0];
  t1[1] = dw[1] - Pw[1];
  t2[0] = de[0] - Pe[0];
  t2[1] = de[1] - Pe[1];
  uni(t1, t2, a, U);
  cov[1] = P2[0] + U[0];
  cov[3] = P2[1] + U[1];
}

}  // namespace

extern "C" {

int orc_mesh_counts(int nx, int ny, int px, int py, int* nEl, int* nEdges, int* nNodes) {
  if (nx < 1 || ny < 1) return -1;
  if ((px && nx < 3) || (py && ny < 3)) return -1;
  int NX = px ? nx : nx + 1, NY = py ? ny : ny + 1;
  *nEl = nx * ny;
  *nNodes = NX * NY;
  *nEdges = (px ? nx : nx + 1) * ny + nx * (py ? ny : ny + 1);
  return 0;
}

int orc_mesh_build(int nx, int ny, int px, int py, int N, int quad, double warp, double xscale, double yscale,
                   int boundary_flag, int* edges, int* elemNodes, int* nodeType, int* n2e_ptr, int* n2e_elem,
                   int* n2e_local, double* x, double* y, double* dxds, double* dxdp, double* dyds, double* dydp,
                   double* J, double* nhx, double* nhy, double* nlen, double* bx, double* by) {
  int nEl, nEdges, nNodes;
  if (orc_mesh_counts(nx, ny, px, py, &nEl, &nEdges, &nNodes) != 0) return -1;
  const int n = N + 1;
  const int NX = px ? nx : nx + 1;
  auto nodeid = [&](int iX, int iY) {  // 1-based corner grid indices -> 1-based node ID
    int ix = px ? ((iX - 1) % nx) + 1 : iX;
    int iy = py ? ((iY - 1) % ny) + 1 : iY;
    return ix + (iy - 1) * NX;
  };
  std::vector<double> xq(n), wq(n), bw(n);
  if (orc_legendre_quadrature(N, quad, xq.data(), wq.data()) != 0) return -1;
  orc::barycentric(N, xq.data(), bw.data());
  std::vector<double> D(n * n);
  orc::derivative_matrix(N, xq.data(), bw.data(), D.data());

  const double dxE = 1.0 / nx, dyE = 1.0 / ny;
  for (int k = 0; k < nNodes; ++k) nodeType[k] = 0;

  // elements, geometry
  for (int iY = 1; iY <= ny; ++iY)
    for (int iX = 1; iX <= nx; ++iX) {
      int iEl = iX + (iY - 1) * nx;
      int e = iEl - 1;
      int nd[4] = {nodeid(iX, iY), nodeid(iX + 1, iY), nodeid(iX + 1, iY + 1), nodeid(iX, iY + 1)};
      double cx[4] = {dxE * (iX - 1), dxE * iX, dxE * iX, dxE * (iX - 1)};
      double cy[4] = {dyE * (iY - 1), dyE * (iY - 1), dyE * iY, dyE * iY};
      for (int k = 0; k < 4; ++k) elemNodes[4 * e + k] = nd[k];
      Curve cur[4];
      for (int s = 0; s < 4; ++s) {
        int l1 = kEdgeMap[0][s] - 1, l2 = kEdgeMap[1][s] - 1;
        cur[s].build(cx[l1], cy[l1], cx[l2], cy[l2]);
      }
      // GenerateMesh / GenerateMetrics on the unit square, then the warp, then ScaleGeometry
      double* X = x + (size_t)n * n * e;
      double* Y = y + (size_t)n * n * e;
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
          double P[2], cov[4];
          tfi(cur, xq[i], xq[j], P);
          tfi_metrics(cur, xq[i], xq[j], cov);
          int id = i + n * j;
          double sw = warp * std::sin(2.0 * kPi * P[0]) * std::sin(2.0 * kPi * P[1]);
          X[id] = xscale * (P[0] + sw);
          Y[id] = yscale * (P[1] + sw);
          double Jl = cov[0] * cov[3] - cov[1] * cov[2];  // Determinant( covT, 2 )
          dxds[(size_t)n * n * e + id] = xscale * cov[0];
          dxdp[(size_t)n * n * e + id] = xscale * cov[1];
          dyds[(size_t)n * n * e + id] = yscale * cov[2];
          dydp[(size_t)n * n * e + id] = yscale * cov[3];
          J[(size_t)n * n * e + id] = xscale * yscale * Jl;
        }
      if (warp != 0.0) {
        // interpolant-derivative metrics of the warped node positions
        for (int i = 0; i < n; ++i)
          for (int j = 0; j < n; ++j) {
            double xs = 0, xp = 0, ys = 0, yp = 0;
            for (int k = 0; k < n; ++k) {
              xs = xs + D[i + k * n] * X[k + n * j];
              ys = ys + D[i + k * n] * Y[k + n * j];
              xp = xp + D[j + k * n] * X[i + n * k];
              yp = yp + D[j + k * n] * Y[i + n * k];
            }
            size_t id = (size_t)n * n * e + i + n * j;
            dxds[id] = xs;
            dxdp[id] = xp;
            dyds[id] = ys;
            dydp[id] = yp;
            J[id] = xs * yp - xp * ys;
          }
      }
      // boundary locations (GenerateMesh :570-604) and normals (GenerateBoundaryMetrics :714-788)
      auto boundary_point = [&](double a, double b, double& ox, double& oy) {
        double P[2];
        tfi(cur, a, b, P);
        double sw = warp * std::sin(2.0 * kPi * P[0]) * std::sin(2.0 * kPi * P[1]);
        ox = xscale * (P[0] + sw);
        oy = yscale * (P[1] + sw);
      };
      // EvaluateDerivative_2D of the node positions (Lagrange_2D_Class.f90:396-440)
      auto calc_metrics = [&](double a, double b, double* cov) {
        std::vector<double> lS(n), lP(n), f1(n), f2(n);
        orc::lagrange_at(N, xq.data(), bw.data(), a, lS.data());
        orc::lagrange_at(N, xq.data(), bw.data(), b, lP.data());
        const double* F[2] = {X, Y};
        for (int c = 0; c < 2; ++c) {
          double dfds = 0.0, dfdp = 0.0;
          for (int jP = 0; jP < n; ++jP) {
            for (int i = 0; i < n; ++i) f1[i] = F[c][i + n * jP];
            dfds = dfds + orc::lagrange_deriv(N, xq.data(), bw.data(), a, f1.data()) * lP[jP];
          }
          for (int jS = 0; jS < n; ++jS) {
            for (int j = 0; j < n; ++j) f2[j] = F[c][jS + n * j];
            dfdp = dfdp + orc::lagrange_deriv(N, xq.data(), bw.data(), b, f2.data()) * lS[jS];
          }
          cov[2 * c + 0] = dfds;
          cov[2 * c + 1] = dfdp;
        }
      };
      auto set_normal = [&](int side, int i, double d0, double d1) {
        size_t id = (size_t)i + n * (side + 4 * (size_t)e);
        double len = std::sqrt(d0 * d0 + d1 * d1);
        double nrm = std::sqrt(d0 * d0 + d1 * d1);  // Normalize_Vector (VectorClass.f90:236-246)
        nhx[id] = d0 / nrm;
        nhy[id] = d1 / nrm;
        nlen[id] = len;
      };
      for (int i = 0; i < n; ++i) {
        double cov[4], Jl, sJ;
        double s = xq[i];
        boundary_point(s, -1.0, bx[(size_t)i + n * (0 + 4 * (size_t)e)], by[(size_t)i + n * (0 + 4 * (size_t)e)]);
        boundary_point(s, 1.0, bx[(size_t)i + n * (2 + 4 * (size_t)e)], by[(size_t)i + n * (2 + 4 * (size_t)e)]);
        calc_metrics(s, -1.0, cov);
        Jl = cov[0] * cov[3] - cov[1] * cov[2];
        sJ = std::fabs(Jl) / Jl;
        set_normal(0, i, -sJ * (-cov[2]), -sJ * cov[0]);
        calc_metrics(s, 1.0, cov);
        Jl = cov[0] * cov[3] - cov[1] * cov[2];
        sJ = std::fabs(Jl) / Jl;
        set_normal(2, i, sJ * (-cov[2]), sJ * cov[0]);
      }
      for (int j = 0; j < n; ++j) {
        double cov[4], Jl, sJ;
        double p = xq[j];
        boundary_point(-1.0, p, bx[(size_t)j + n * (3 + 4 * (size_t)e)], by[(size_t)j + n * (3 + 4 * (size_t)e)]);
        boundary_point(1.0, p, bx[(size_t)j + n * (1 + 4 * (size_t)e)], by[(size_t)j + n * (1 + 4 * (size_t)e)]);
        calc_metrics(-1.0, p, cov);
        Jl = cov[0] * cov[3] - cov[1] * cov[2];
        sJ = std::fabs(Jl) / Jl;
        set_normal(3, j, -sJ * cov[3], -sJ * (-cov[1]));
        calc_metrics(1.0, p, cov);
        Jl = cov[0] * cov[3] - cov[1] * cov[2];
        sJ = std::fabs(Jl) / Jl;
        set_normal(1, j, sJ * cov[3], sJ * (-cov[1]));
      }
    }

  // ConstructEdges (second pass; edge IDs in order of first appearance)
  std::map<std::pair<int, int>, int> table;
  int ne = 0;
  for (int iEl = 1; iEl <= nEl; ++iEl)
    for (int k = 1; k <= 4; ++k) {
      int startID = elemNodes[4 * (iEl - 1) + kEdgeMap[0][k - 1] - 1];
      int endID = elemNodes[4 * (iEl - 1) + kEdgeMap[1][k - 1] - 1];
      std::pair<int, int> key(std::min(startID, endID), std::max(startID, endID));
      auto it = table.find(key);
      if (it != table.end()) {
        int id = it->second;
        int e1 = edges[6 * (id - 1) + 0], s1 = edges[6 * (id - 1) + 1];
        int n1 = elemNodes[4 * (e1 - 1) + kEdgeMap[0][s1 - 1] - 1];
        edges[6 * (id - 1) + 2] = iEl;
        edges[6 * (id - 1) + 3] = (startID == n1) ? k : -k;
      } else {
        ++ne;
        if (ne > nEdges) return -2;
        table[key] = ne;
        int* E = edges + 6 * (ne - 1);
        E[0] = iEl;
        E[1] = k;
        E[2] = boundary_flag;
        E[3] = 0;
        E[4] = startID;  // temporarily hold node IDs for the node-type pass
        E[5] = endID;
      }
    }
  if (ne != nEdges) return -3;
  // start / increment and boundary node types (LoadDefaultMesh :1828-1847)
  for (int id = 0; id < nEdges; ++id) {
    int* E = edges + 6 * id;
    int n1 = E[4], n2 = E[5];
    if (E[2] < 0) {
      nodeType[n1 - 1] = E[2];
      nodeType[n2 - 1] = E[2];
    }
    if (E[3] < 0) {
      E[4] = N - 1;
      E[5] = -1;
    } else {
      E[4] = 1;
      E[5] = 1;
    }
  }
  // GetNodeToElementConnectivity: tail insertion, element order, key = local corner 1..4
  std::vector<int> cnt(nNodes, 0);
  for (int e = 0; e < nEl; ++e)
    for (int k = 0; k < 4; ++k) cnt[elemNodes[4 * e + k] - 1]++;
  n2e_ptr[0] = 0;
  for (int i = 0; i < nNodes; ++i) n2e_ptr[i + 1] = n2e_ptr[i] + cnt[i];
  std::vector<int> pos(n2e_ptr, n2e_ptr + nNodes);
  for (int e = 0; e < nEl; ++e)
    for (int k = 0; k < 4; ++k) {
      int nd = elemNodes[4 * e + k] - 1;
      n2e_elem[pos[nd]] = e + 1;
      n2e_local[pos[nd]] = k + 1;
      pos[nd]++;
    }
  return 0;
}

}  // extern "C"
