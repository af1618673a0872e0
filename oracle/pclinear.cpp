// CPU oracle (test infrastructure): the reference's linear-FEM preconditioner of the CGSEM 2-D solve.
// Restates
//  * src/geom/QuadMeshClass.f90 ConstructLinearMeshFromOther_QuadMesh :1863-2092 -- the GLL nodes of the
//    original mesh become the corner nodes of nEl*N*N bilinear elements; unique nodes by position
//    (AlmostEqual, first earlier match), element / node maps linToOther and otherToLin, straight side curves
//    through the corner nodes, MappedGeometry_2D Build (transfinite covariant metrics, Determinant for J),
//    ConstructEdges :1489-1627 (an unmatched side gets BoundaryFlagDefault = NO_NORMAL_FLOW and marks its two
//    nodes) and GetNodeToElementConnectivity :1631-1658 (tail insertion, element order);
//  * src/cgsem/CGsemPreconditioner_2D_Class.f90 -- Build :88-128 (N = 1 Gauss-Lobatto CG storage,
//    NO_NORMAL_FLOW nodes -> DIRICHLET, fluxCoeff = 1), MapFromOrigToPC / MapFromPCToOrig :160-226, Mask /
//    UnMask / GlobalSum :230-420 (corner-node lists only), FluxDivergence / MatrixAction :424-598, DotProduct
//    :602-642 (masks copies of its arguments) and Solve :646-746 (CG from u = 0, stop at ||r||/||r0|| < TOL or
//    after maxIters, u = r when maxIters = 0);
//  * src/cgsem/CGsemElliptic_2D_Class.f90 Solve_PCConjugateGradient :1114-1207 with the preconditioner call
//    w = preconditioner%Solve(UnMask(r)) and Build :146-152 (the preconditioner's fluxCoeff is mapped while the
//    solver's own fluxCoeff still holds ONE, so the linear operator always has k = 1).
// Decisions: the unique-node search uses a hash grid of cell size 1e-9 x the mesh extent, which finds the same
// first earlier AlmostEqual match as the reference's all-pairs loop (AlmostEqual's tolerance is ~1e-16
// relative); ioerr = 0 on convergence as in the other oracle solvers.  Extension: with `ids` (one node id per
// local node, equal ids = one node) the nodes are identified by those ids instead of by position, numbered in
// the same first-appearance order.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "oracle.h"
#include "oracle_internal.hpp"

namespace {

const int kEdgeMap[2][4] = {{1, 2, 4, 1}, {2, 3, 3, 4}};  // QuadMeshClass.f90:194-195
constexpr int kNoNormalFlow = -100;                        // ModelFlags.f90:80

struct LinearPC {
  int nEl = 0, nNodes = 0;
  std::vector<int> linToOther;  // 4 per linear element: original local index of corner (i, j), i + 2 j
  std::vector<int> otherToLin;  // 1 per original local node: linear local index (last assignment wins)
  std::vector<int> nodeType, n2e_ptr, n2e_elem, n2e_local;
  std::vector<double> dxds, dxdp, dyds, dydp, J, kcoef, dmat, qw;
  orc_cg_problem p{};
  int maxIters = 0;
  double tol = 0;
};

double extent(const double* x, size_t n) {
  double lo = x[0], hi = x[0];
  for (size_t k = 1; k < n; ++k) {
    lo = std::min(lo, x[k]);
    hi = std::max(hi, x[k]);
  }
  return hi - lo;
}

// uniqueNids of ConstructLinearMeshFromOther: node i takes the ID of the first j < i at the same position
// (AlmostEqual in x and y), else the next new ID.
int unique_ids(const double* x, const double* y, size_t n, std::vector<int>& uid) {
  const double ext = std::max({extent(x, n), extent(y, n), 1e-300});
  const double h = ext * 1e-9;
  auto cell = [&](double v) { return (int64_t)std::floor(v / h); };
  auto key = [](int64_t a, int64_t b) { return (uint64_t)a * 0x9E3779B97F4A7C15ull ^ (uint64_t)b; };
  std::unordered_map<uint64_t, std::vector<int>> grid;
  grid.reserve(n);
  uid.assign(n, 0);
  int nUnique = 0;
  for (size_t i = 0; i < n; ++i) {
    const int64_t cx = cell(x[i]), cy = cell(y[i]);
    int best = -1;
    for (int64_t dx = -1; dx <= 1; ++dx)
      for (int64_t dy = -1; dy <= 1; ++dy) {
        auto it = grid.find(key(cx + dx, cy + dy));
        if (it == grid.end()) continue;
        for (int j : it->second)
          if ((best < 0 || j < best) && orc::almost_equal(x[i], x[j]) && orc::almost_equal(y[i], y[j])) best = j;
      }
    if (best >= 0) {
      uid[i] = uid[best];
    } else {
      uid[i] = ++nUnique;
    }
    grid[key(cx, cy)].push_back((int)i);
  }
  return nUnique;
}

int ids_in_order(const int* ids, size_t n, std::vector<int>& uid) {
  std::unordered_map<int, int> seen;
  uid.assign(n, 0);
  int nUnique = 0;
  for (size_t i = 0; i < n; ++i) {
    auto it = seen.find(ids[i]);
    if (it == seen.end()) it = seen.emplace(ids[i], ++nUnique).first;
    uid[i] = it->second;
  }
  return nUnique;
}

void build(const orc_cg_problem* p, const double* x, const double* y, const int* ids, LinearPC& L) {
  const int N = p->N, n = N + 1;
  const size_t nl = (size_t)n * n * p->nEl;
  std::vector<int> uid;
  L.nNodes = ids ? ids_in_order(ids, nl, uid) : unique_ids(x, y, nl, uid);
  L.nEl = p->nEl * N * N;
  // node positions: every original node writes its position to its unique ID (the last write stays)
  std::vector<double> nx(L.nNodes + 1), ny(L.nNodes + 1);
  for (size_t k = 0; k < nl; ++k) {
    nx[uid[k]] = x[k];
    ny[uid[k]] = y[k];
  }
  L.linToOther.assign((size_t)4 * L.nEl, 0);
  L.otherToLin.assign(nl, 0);
  std::vector<int> nodes((size_t)4 * L.nEl);
  const size_t ne = (size_t)L.nEl * 4;
  L.dxds.assign(ne, 0.0);
  L.dxdp.assign(ne, 0.0);
  L.dyds.assign(ne, 0.0);
  L.dydp.assign(ne, 0.0);
  L.J.assign(ne, 0.0);
  L.kcoef.assign(ne, 1.0);
  orc::CurveG cur[4];
  for (auto& c : cur) c.nodes(1);
  const double s[2] = {-1.0, 1.0};
  for (int e = 0; e < p->nEl; ++e)
    for (int iP = 1; iP <= N; ++iP)
      for (int iS = 1; iS <= N; ++iS) {
        const int eid = (iS - 1) + N * ((iP - 1) + e * N);  // 0-based linear element ID
        auto orig = [&](int i, int j) { return (int)((size_t)i + n * (j + (size_t)n * e)); };
        const int c00 = orig(iS - 1, iP - 1), c10 = orig(iS, iP - 1), c11 = orig(iS, iP), c01 = orig(iS - 1, iP);
        int* lo = &L.linToOther[(size_t)4 * eid];
        lo[0] = c00;
        lo[1] = c10;
        lo[3] = c11;
        lo[2] = c01;
        L.otherToLin[c00] = 4 * eid + 0;
        L.otherToLin[c10] = 4 * eid + 1;
        L.otherToLin[c11] = 4 * eid + 3;
        L.otherToLin[c01] = 4 * eid + 2;
        int* nd = &nodes[(size_t)4 * eid];
        nd[0] = uid[c00];  // southwest
        nd[1] = uid[c10];  // southeast
        nd[2] = uid[c11];  // northeast
        nd[3] = uid[c01];  // northwest
        for (int side = 0; side < 4; ++side) {
          const int n1 = nd[kEdgeMap[0][side] - 1], n2 = nd[kEdgeMap[1][side] - 1];
          const double x1 = nx[n1], y1 = ny[n1], x2 = nx[n2], y2 = ny[n2];
          for (int k = 0; k < 2; ++k) {
            cur[side].x[k] = x1 + (x2 - x1) * 0.5 * (s[k] + 1.0);
            cur[side].y[k] = y1 + (y2 - y1) * 0.5 * (s[k] + 1.0);
          }
        }
        for (int i = 0; i < 2; ++i)
          for (int j = 0; j < 2; ++j) {
            double cov[4];
            orc::tfi_metrics(cur, s[i], s[j], cov);
            const size_t id = (size_t)i + 2 * (j + (size_t)2 * eid);
            L.dxds[id] = cov[0];
            L.dxdp[id] = cov[1];
            L.dyds[id] = cov[2];
            L.dydp[id] = cov[3];
            L.J[id] = cov[0] * cov[3] - cov[1] * cov[2];
          }
      }
  // ConstructEdges: a side whose (min, max) node pair no other side has is a boundary edge; its nodes get
  // NO_NORMAL_FLOW, which the preconditioner's Build turns into DIRICHLET.
  L.nodeType.assign(L.nNodes, 1);
  std::unordered_map<uint64_t, int> sides;
  sides.reserve(ne);
  for (int e = 0; e < L.nEl; ++e)
    for (int k = 0; k < 4; ++k) {
      const int a = nodes[(size_t)4 * e + kEdgeMap[0][k] - 1], b = nodes[(size_t)4 * e + kEdgeMap[1][k] - 1];
      sides[((uint64_t)std::min(a, b) << 32) | (uint64_t)std::max(a, b)] += 1;
    }
  for (int e = 0; e < L.nEl; ++e)
    for (int k = 0; k < 4; ++k) {
      const int a = nodes[(size_t)4 * e + kEdgeMap[0][k] - 1], b = nodes[(size_t)4 * e + kEdgeMap[1][k] - 1];
      if (sides[((uint64_t)std::min(a, b) << 32) | (uint64_t)std::max(a, b)] == 1) {
        L.nodeType[a - 1] = kNoNormalFlow;
        L.nodeType[b - 1] = kNoNormalFlow;
      }
    }
  for (int& t : L.nodeType)
    if (t == kNoNormalFlow) t = ORC_DIRICHLET;
  // GetNodeToElementConnectivity
  std::vector<int> cnt(L.nNodes, 0);
  for (int e = 0; e < L.nEl; ++e)
    for (int k = 0; k < 4; ++k) cnt[nodes[(size_t)4 * e + k] - 1]++;
  L.n2e_ptr.assign(L.nNodes + 1, 0);
  for (int i = 0; i < L.nNodes; ++i) L.n2e_ptr[i + 1] = L.n2e_ptr[i] + cnt[i];
  L.n2e_elem.assign(ne, 0);
  L.n2e_local.assign(ne, 0);
  std::vector<int> pos(L.n2e_ptr.begin(), L.n2e_ptr.end() - 1);
  for (int e = 0; e < L.nEl; ++e)
    for (int k = 0; k < 4; ++k) {
      const int nd = nodes[(size_t)4 * e + k] - 1;
      L.n2e_elem[pos[nd]] = e + 1;
      L.n2e_local[pos[nd]] = k + 1;
      pos[nd]++;
    }
  // N = 1 Gauss-Lobatto CG storage
  double xg[2], wg[2];
  orc_legendre_quadrature(1, ORC_GAUSS_LOBATTO, xg, wg);
  L.qw.assign(wg, wg + 2);
  L.dmat.assign(4, 0.0);
  orc_derivative_matrix(1, xg, L.dmat.data());
  orc_cg_problem& q = L.p;
  q.N = 1;
  q.nEl = L.nEl;
  q.nEdges = 0;  // N = 1: no edge-interior nodes, shared nodes are all corner nodes
  q.nNodes = L.nNodes;
  q.dmat = L.dmat.data();
  q.qw = L.qw.data();
  q.edges = nullptr;
  q.nodeType = L.nodeType.data();
  q.n2e_ptr = L.n2e_ptr.data();
  q.n2e_elem = L.n2e_elem.data();
  q.n2e_local = L.n2e_local.data();
  q.dxds = L.dxds.data();
  q.dxdp = L.dxdp.data();
  q.dyds = L.dyds.data();
  q.dydp = L.dydp.data();
  q.J = L.J.data();
  q.kcoef = L.kcoef.data();
  q.lambda = 0.0;
  q.op = 0;
}

// DotProduct_CGsemPreconditioner_2D: masks copies of its arguments
double pc_dot(const LinearPC& L, const std::vector<double>& u, const std::vector<double>& v) {
  std::vector<double> uu(u), vv(v);
  return orc_cg_dot(&L.p, uu.data(), vv.data());
}

// Solve_CGsemPreconditioner_2D: x (original mesh, unmasked) from b (original mesh)
int pc_solve(const LinearPC& L, const double* b, double* x, int* iters_out) {
  const size_t nl = (size_t)4 * L.nEl;
  std::vector<double> u(nl, 0.0), r(nl), v(nl, 0.0), z(nl, 0.0), w(nl);
  for (size_t k = 0; k < nl; ++k) r[k] = b[L.linToOther[k]];
  const double r0 = std::sqrt(pc_dot(L, r, r));
  double num = 0, den = 0, rNorm = 0;
  int it = 0;
  for (int iter = 1; iter <= L.maxIters; ++iter) {
    w = r;
    num = pc_dot(L, r, w);
    if (iter == 1) {
      v = w;
    } else {
      const double c = num / den;
      for (size_t k = 0; k < nl; ++k) v[k] = w[k] + c * v[k];
    }
    orc_cg_matrix_action(&L.p, v.data(), z.data());
    const double a = num / pc_dot(L, v, z);
    for (size_t k = 0; k < nl; ++k) u[k] = u[k] + a * v[k];
    for (size_t k = 0; k < nl; ++k) r[k] = r[k] - a * z[k];
    den = num;
    rNorm = std::sqrt(pc_dot(L, r, r));
    it = iter;
    if (rNorm / r0 < L.tol) break;
  }
  if (L.maxIters == 0) u = r;
  orc_cg_unmask(&L.p, u.data());
  const size_t no = L.otherToLin.size();
  for (size_t k = 0; k < no; ++k) x[k] = u[L.otherToLin[k]];
  if (iters_out) *iters_out = it;
  return 0;
}

}  // namespace

extern "C" {

int orc_pc_linear_info(const orc_cg_problem* p, const double* x, const double* y, const int* ids, int* nUnique,
                       int* nDirichlet) {
  if (p->N < 1) return -1;
  LinearPC L;
  build(p, x, y, ids, L);
  *nUnique = L.nNodes;
  int nd = 0;
  for (int t : L.nodeType) nd += t == ORC_DIRICHLET;
  *nDirichlet = nd;
  return 0;
}

int orc_pc_linear_apply(const orc_cg_problem* p, const double* x, const double* y, const int* ids, int pcIters,
                        double pcTol, const double* b, double* out, int* iters) {
  if (p->N < 1 || pcIters < 0) return -1;
  LinearPC L;
  build(p, x, y, ids, L);
  L.maxIters = pcIters;
  L.tol = pcTol;
  return pc_solve(L, b, out, iters);
}

int orc_cg_solve_pcg_linear(const orc_cg_problem* p, const double* x, const double* y, const int* ids,
                            const double* source, double* solution, const double* dir, int maxIters, double tol,
                            int pcIters, double pcTol, double* resi, int* iters) {
  if (p->N < 1 || pcIters < 0) return -1;
  LinearPC L;
  build(p, x, y, ids, L);
  L.maxIters = pcIters;
  L.tol = pcTol;
  const int n = p->N + 1;
  const size_t nl = (size_t)n * n * p->nEl;
  std::vector<double> u(nl), r(nl), v(nl), z(nl), w(nl);
  if (dir) orc::cg_set_dirichlet(p, solution, dir);
  int ioerr = -2;
  std::memcpy(u.data(), solution, nl * sizeof(double));
  int rc = orc_cg_residual(p, source, solution, dir, r.data());
  if (rc) return rc;
  const double r0 = std::sqrt(orc_cg_dot(p, r.data(), r.data()));
  for (int k = 0; k <= maxIters; ++k) resi[k] = 0.0;
  resi[0] = r0;
  double rNorm = r0, num = 0, den = 0;
  *iters = 0;
  if (r0 < tol) return 0;
  for (int iter = 1; iter <= maxIters; ++iter) {
    orc_cg_unmask(p, r.data());
    pc_solve(L, r.data(), w.data(), nullptr);
    num = orc_cg_dot(p, r.data(), w.data());
    if (iter == 1) {
      std::memcpy(v.data(), w.data(), nl * sizeof(double));
    } else {
      const double b = num / den;
      for (size_t k = 0; k < nl; ++k) v[k] = w[k] + b * v[k];
    }
    orc_cg_matrix_action(p, v.data(), z.data());
    const double a = num / orc_cg_dot(p, v.data(), z.data());
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

}  // extern "C"
