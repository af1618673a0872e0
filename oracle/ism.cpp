// CPU oracle (test infrastructure): ISM-V2 (SpecMesh) unstructured quadrilateral mesh files.
// Restates src/geom/QuadMeshClass.f90 ReadSpecMeshFile_QuadMesh :2100-2475 (file layout, straight interior
// sides, boundary curves through the file's Chebyshev-Gauss-Lobatto points, side names -> boundary flags,
// start/increment from the secondary side's sign), ConstructEdges :1489-1627 and GetNodeToElementConnectivity,
// with the element geometry of MappedGeometryClass_2D.f90 Build :105-144 (GenerateMesh :536-607 and
// GenerateMetrics :611-710: transfinite positions, transfinite covariant metrics and boundary normals) and
// src/geom/GeometrySupportRoutines.f90 (TransfiniteInterpolation_2D, TransfiniteInterpolationMetrics_2D),
// src/geom/CurveClass_2D.f90 (Evaluate, EvaluateSlope) and src/interp/Chebyshev.f90 (ChebyshevGaussLobatto).
// Only the text of the file is read: no SpecMesh program is run.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

#include "oracle.h"
#include "oracle_internal.hpp"

namespace {

const double kPiI = 4.0 * std::atan(1.0);
const int kMap[2][4] = {{1, 2, 4, 1}, {2, 3, 3, 4}};  // QuadMeshClass.f90:194-195

// ModelFlags.f90:80-97
int flag_of(const std::string& s) {
  if (s == "DIRICHLET") return -200;
  if (s == "ROBIN") return -202;
  if (s == "ROBIN_FORCED") return -204;
  if (s == "HOMOGENEOUS_NEUMANN") return -201;
  if (s == "NEUMANN_WALL") return -206;
  if (s == "NEUMANN") return -100;
  if (s == "NO_NORMAL_FLOW") return -100;
  if (s == "PRESCRIBED") return -102;
  if (s == "RADIATION") return -101;
  if (s == "InflowOne") return -103;
  if (s == "InflowTwo") return -104;
  return 1;  // INTERIOR (unrecognised names keep the default)
}

}  // namespace

namespace orc {

inline void uni(const double* l, const double* r, double a, double* p) {
  p[0] = 0.5 * ((1.0 - a) * l[0] + (1.0 + a) * r[0]);
  p[1] = 0.5 * ((1.0 - a) * l[1] + (1.0 + a) * r[1]);
}
inline void unid(const double* l, const double* r, double* p) {
  p[0] = 0.5 * (r[0] - l[0]);
  p[1] = 0.5 * (r[1] - l[1]);
}

void tfi(const CurveG* c, double a, double b, double* P) {
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

void tfi_metrics(const CurveG* c, double a, double b, double* cov) {  // dxds dxdp dyds dydp
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

}  // namespace orc

namespace {

using orc::CurveG;
using orc::tfi;
using orc::tfi_metrics;

struct IsmFile {
  int nNodes = 0, nEdges = 0, nElems = 0, gdeg = 1;
  std::vector<double> nx, ny;
  std::vector<int> nodes;                 // 4 per element (1-based)
  std::vector<int> bflags;                // 4 per element
  std::vector<std::vector<double>> cx, cy;  // 4 per element: curve points (boundary sides)
  std::vector<int> sideFlags;             // 4 per element
};

bool read_ism(const char* path, IsmFile& f, bool header_only) {
  std::ifstream in(path);
  if (!in) return false;
  std::string line;
  if (!std::getline(in, line)) return false;  // ISM version
  if (!(in >> f.nNodes >> f.nEdges >> f.nElems >> f.gdeg)) return false;
  if (header_only) return true;
  f.nx.resize(f.nNodes);
  f.ny.resize(f.nNodes);
  for (int i = 0; i < f.nNodes; ++i) {
    double z;
    if (!(in >> f.nx[i] >> f.ny[i] >> z)) return false;
  }
  for (int i = 0; i < f.nEdges; ++i) {  // edge records are read and not used (:2178-2187)
    int a, b, c, d, e, g;
    if (!(in >> a >> b >> c >> d >> e >> g)) return false;
  }
  f.nodes.resize(4 * f.nElems);
  f.bflags.resize(4 * f.nElems);
  f.cx.assign(4 * f.nElems, {});
  f.cy.assign(4 * f.nElems, {});
  f.sideFlags.assign(4 * f.nElems, 1);
  for (int e = 0; e < f.nElems; ++e) {
    for (int k = 0; k < 4; ++k)
      if (!(in >> f.nodes[4 * e + k])) return false;
    for (int k = 0; k < 4; ++k)
      if (!(in >> f.bflags[4 * e + k])) return false;
    for (int k = 0; k < 4; ++k) {
      if (f.bflags[4 * e + k] != 1) continue;
      f.cx[4 * e + k].resize(f.gdeg + 1);
      f.cy[4 * e + k].resize(f.gdeg + 1);
      for (int j = 0; j <= f.gdeg; ++j) {
        double z;
        if (!(in >> f.cx[4 * e + k][j] >> f.cy[4 * e + k][j] >> z)) return false;
      }
    }
    std::getline(in, line);  // rest of the flag / curve line
    if (!std::getline(in, line)) return false;
    std::istringstream names(line);  // four names separated by blanks
    for (int k = 0; k < 4; ++k) {
      std::string w;
      if (!(names >> w)) return false;
      f.sideFlags[4 * e + k] = flag_of(w);
    }
  }
  return true;
}

}  // namespace

extern "C" {

int orc_ism_counts(const char* path, int* nEl, int* nEdges, int* nNodes, int* geomDegree) {
  IsmFile f;
  if (!read_ism(path, f, true)) return -1;
  *nEl = f.nElems;
  *nEdges = f.nEdges;
  *nNodes = f.nNodes;
  *geomDegree = f.gdeg;
  return 0;
}

int orc_ism_build(const char* path, int N, int quad, int* edges, int* elemNodes, int* nodeType, int* n2e_ptr,
                  int* n2e_elem, int* n2e_local, double* x, double* y, double* dxds, double* dxdp, double* dyds,
                  double* dydp, double* J, double* nhx, double* nhy, double* nlen, double* bx, double* by) {
  IsmFile f;
  if (!read_ism(path, f, false)) return -1;
  const int n = N + 1, nEl = f.nElems, nNodes = f.nNodes, nEdges = f.nEdges;
  std::vector<double> xq(n), wq(n);
  if (orc_legendre_quadrature(N, quad, xq.data(), wq.data()) != 0) return -1;
  for (int k = 0; k < nNodes; ++k) nodeType[k] = 0;
  for (int e = 0; e < nEl; ++e) {
    for (int k = 0; k < 4; ++k) elemNodes[4 * e + k] = f.nodes[4 * e + k];
    CurveG cur[4];
    for (int side = 0; side < 4; ++side) {
      cur[side].nodes(f.gdeg);
      if (f.bflags[4 * e + side] == 0) {  // straight side between its two corner nodes
        const int n1 = f.nodes[4 * e + kMap[0][side] - 1], n2 = f.nodes[4 * e + kMap[1][side] - 1];
        const double x1 = f.nx[n1 - 1], y1 = f.ny[n1 - 1], x2 = f.nx[n2 - 1], y2 = f.ny[n2 - 1];
        for (int j = 0; j <= f.gdeg; ++j) {
          cur[side].x[j] = x1 + (x2 - x1) * 0.5 * (cur[side].s[j] + 1.0);
          cur[side].y[j] = y1 + (y2 - y1) * 0.5 * (cur[side].s[j] + 1.0);
        }
      } else {
        cur[side].x = f.cx[4 * e + side];
        cur[side].y = f.cy[4 * e + side];
      }
    }
    const size_t o = (size_t)n * n * e;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        double P[2], cov[4];
        tfi(cur, xq[i], xq[j], P);
        tfi_metrics(cur, xq[i], xq[j], cov);
        const size_t id = o + i + n * j;
        x[id] = P[0];
        y[id] = P[1];
        dxds[id] = cov[0];
        dxdp[id] = cov[1];
        dyds[id] = cov[2];
        dydp[id] = cov[3];
        J[id] = cov[0] * cov[3] - cov[1] * cov[2];
      }
    auto set_normal = [&](int side, int i, double d0, double d1, double a, double b) {
      const size_t id = (size_t)i + n * (side + 4 * (size_t)e);
      const double len = std::sqrt(d0 * d0 + d1 * d1);
      nhx[id] = d0 / len;
      nhy[id] = d1 / len;
      nlen[id] = len;
      double P[2];
      tfi(cur, a, b, P);
      bx[id] = P[0];
      by[id] = P[1];
    };
    for (int i = 0; i < n; ++i) {
      double cov[4], Jl, sJ;
      const double s = xq[i];
      tfi_metrics(cur, s, -1.0, cov);
      Jl = cov[0] * cov[3] - cov[1] * cov[2];
      sJ = std::fabs(Jl) / Jl;
      set_normal(0, i, -sJ * (-cov[2]), -sJ * cov[0], s, -1.0);
      tfi_metrics(cur, s, 1.0, cov);
      Jl = cov[0] * cov[3] - cov[1] * cov[2];
      sJ = std::fabs(Jl) / Jl;
      set_normal(2, i, sJ * (-cov[2]), sJ * cov[0], s, 1.0);
    }
    for (int j = 0; j < n; ++j) {
      double cov[4], Jl, sJ;
      const double p = xq[j];
      tfi_metrics(cur, -1.0, p, cov);
      Jl = cov[0] * cov[3] - cov[1] * cov[2];
      sJ = std::fabs(Jl) / Jl;
      set_normal(3, j, -sJ * cov[3], -sJ * (-cov[1]), -1.0, p);
      tfi_metrics(cur, 1.0, p, cov);
      Jl = cov[0] * cov[3] - cov[1] * cov[2];
      sJ = std::fabs(Jl) / Jl;
      set_normal(1, j, sJ * cov[3], sJ * (-cov[1]), 1.0, p);
    }
  }
  // ConstructEdges: IDs in order of first appearance, secondary side negative for opposite orientation
  std::map<std::pair<int, int>, int> table;
  std::vector<int> en1(nEdges + 1), en2(nEdges + 1);
  int ne = 0;
  for (int iEl = 1; iEl <= nEl; ++iEl)
    for (int k = 1; k <= 4; ++k) {
      const int startID = elemNodes[4 * (iEl - 1) + kMap[0][k - 1] - 1];
      const int endID = elemNodes[4 * (iEl - 1) + kMap[1][k - 1] - 1];
      const std::pair<int, int> key(std::min(startID, endID), std::max(startID, endID));
      auto it = table.find(key);
      if (it != table.end()) {
        const int id = it->second;
        const int e1 = edges[6 * (id - 1) + 0], s1 = edges[6 * (id - 1) + 1];
        const int n1 = elemNodes[4 * (e1 - 1) + kMap[0][s1 - 1] - 1];
        edges[6 * (id - 1) + 2] = iEl;
        edges[6 * (id - 1) + 3] = (startID == n1) ? k : -k;
      } else {
        ++ne;
        if (ne > nEdges) return -2;
        table[key] = ne;
        int* E = edges + 6 * (ne - 1);
        E[0] = iEl;
        E[1] = k;
        E[2] = -100;  // BoundaryFlagDefault = NO_NORMAL_FLOW
        E[3] = 0;
        en1[ne] = startID;
        en2[ne] = endID;
      }
    }
  if (ne != nEdges) return -3;
  // boundary flags of the primary side (:2336-2418), then start / increment (:2420-2430)
  for (int id = 1; id <= nEdges; ++id) {
    int* E = edges + 6 * (id - 1);
    const int fl = f.sideFlags[4 * (E[0] - 1) + E[1] - 1];
    if (fl < 0) {
      E[2] = fl;
      nodeType[en1[id] - 1] = fl;
      nodeType[en2[id] - 1] = fl;
    }
    if (E[3] < 0) {
      E[4] = N - 1;
      E[5] = -1;
    } else {
      E[4] = 1;
      E[5] = 1;
    }
  }
  std::vector<int> cnt(nNodes, 0);
  for (int e = 0; e < nEl; ++e)
    for (int k = 0; k < 4; ++k) cnt[elemNodes[4 * e + k] - 1]++;
  n2e_ptr[0] = 0;
  for (int i = 0; i < nNodes; ++i) n2e_ptr[i + 1] = n2e_ptr[i] + cnt[i];
  std::vector<int> pos(n2e_ptr, n2e_ptr + nNodes);
  for (int e = 0; e < nEl; ++e)
    for (int k = 0; k < 4; ++k) {
      const int nd = elemNodes[4 * e + k] - 1;
      n2e_elem[pos[nd]] = e + 1;
      n2e_local[pos[nd]] = k + 1;
      pos[nd]++;
    }
  return 0;
}

}  // extern "C"
