/*
 * CPU ORACLE for the SELF spectral-element hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * This library is a plain C++ restatement of the reference Fortran routines
 * (lileipku00/SELF, src/...) that the GPU path replaces.  It exists to check
 * the GPU library and to provide the timed CPU baseline.  Only tests/,
 * __graft_entry__.smoke() and bench.py (cpu_baseline leg and --impl reference)
 * may load it.  The product library (self_gb300, libselfgpu.so) never links,
 * loads or calls it.
 *
 * Parity pins:
 *   - 1-D CGSEM elliptic example (examples/elliptic1d/parabola/run/residual.curve,
 *     elliptic.curve) reproduces Solve_ConjugateGradient, GLL nodes/weights,
 *     derivative matrix and the mask/global-sum semantics;
 *   - spectral convergence of the derivative matrices
 *     (testing/interp/Lagrange1D_Convergence/TestLagrangeInterpolation_1D.f90);
 *   - analytic known answers: lake at rest, periodic translation of a Gaussian,
 *     manufactured solutions.  The 2-D routines have no reference-shipped
 *     golden vectors: their parity with the Fortran is by restatement.
 *
 * Arithmetic follows the Fortran statement order left to right, with no FMA
 * contraction (built with -ffp-contract=off), so that results are identical on
 * x86-64 and aarch64 hosts.
 *
 * Index conventions (match the Fortran storage so arrays pass unchanged):
 *   nodal matrices  D(i,j) at D[i + j*n], n = N+1 (column major)
 *   element arrays  f(i,j,e) at f[i + n*(j + n*e)]      (i = s index, j = p index)
 *   E-vectors       q(i,j,v,e) at q[i + n*(j + n*(v + nEq*e))]
 *   side arrays     b(i,v,side,e) at b[i + n*(v + nEq*(side + 4*e))], side 0..3 = S,E,N,W
 *   normals         nhat(i,side,e) at [i + n*(side + 4*e)]
 *   edge table      edges[6*k + {0..5}] = e1, s1, e2, s2, start, inc (1-based
 *                   elements and sides as in QuadMeshClass.f90; e2 < 0 is a boundary flag)
 */
#ifndef SELF_ORACLE_H
#define SELF_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* ModelFlags.f90:80-137 */
#define ORC_NO_NORMAL_FLOW (-100)
#define ORC_RADIATION (-101)
#define ORC_INFLOW_ONE (-103)
#define ORC_INFLOW_TWO (-104)
#define ORC_DIRICHLET (-200)
#define ORC_GAUSS 1
#define ORC_GAUSS_LOBATTO (-1)
#define ORC_DG 2000
#define ORC_CG 2001

/* ---------------- nodal storage (Legendre.f90, Lagrange_1D_Class.f90, NodalStorage_2D_Class.f90) */
int orc_legendre_quadrature(int N, int quad, double* x, double* w);
int orc_barycentric_weights(int N, const double* x, double* bw);
int orc_derivative_matrix(int N, const double* x, double* D);
int orc_lagrange_at(int N, const double* x, double xe, double* l);
/* quirk_dmatp = 1 reproduces the transposed p-direction DG matrix of NodalStorage_2D_Class.f90:209-218 */
int orc_nodal_build(int N, int quad, int form, int quirk_dmatp, double* x, double* w, double* dmatS,
                    double* dmatP, double* lW, double* lE, double* lS, double* lN);

/* ---------------- structured quad mesh (QuadMeshClass.f90 LoadDefaultMesh/ConstructEdges/ScaleTheMesh)
 * periodic_x/y identify the boundary corner nodes so that ConstructEdges pairs the opposite sides
 * (periodic connectivity does not exist in the reference; it is the new mesh-layer feature).
 * warp: x <- x + warp*sin(2 pi x)sin(2 pi y), y likewise, on the unit square before scaling. */
int orc_mesh_counts(int nx, int ny, int periodic_x, int periodic_y, int* nEl, int* nEdges, int* nNodes);
int orc_mesh_build(int nx, int ny, int periodic_x, int periodic_y, int N, int quad, double warp,
                   double xscale, double yscale, int boundary_flag,
                   int* edges, int* elemNodes, int* nodeType, int* n2e_ptr, int* n2e_elem, int* n2e_local,
                   double* x, double* y, double* dxds, double* dxdp, double* dyds, double* dydp, double* J,
                   double* nhx, double* nhy, double* nlen, double* bx, double* by);

/* ---------------- ISM-V2 (SpecMesh) mesh files: ReadSpecMeshFile_QuadMesh (QuadMeshClass.f90:2100-2475) with
 * transfinite element geometry; the same output arrays as orc_mesh_build. */
int orc_ism_counts(const char* path, int* nEl, int* nEdges, int* nNodes, int* geomDegree);
int orc_ism_build(const char* path, int N, int quad, int* edges, int* elemNodes, int* nodeType, int* n2e_ptr,
                  int* n2e_elem, int* n2e_local, double* x, double* y, double* dxds, double* dxdp, double* dyds,
                  double* dydp, double* J, double* nhx, double* nhy, double* nlen, double* bx, double* by);

/* ---------------- DGSEM 2-D (ConservativeShallowWaterClass.f90, AdvectionClass.f90) */
typedef struct {
  int N, nEl, nEdges, nEq;
  int model;                  /* 1 = conservative SW, 2 = advection, 3 = linear SW, 4 = skew-symmetric SW (nEq 4) */
  const double *dmatS, *dmatP, *qw, *lW, *lE, *lS, *lN;
  const int* edges;
  const double *dxds, *dxdp, *dyds, *dydp, *J;
  const double *nhx, *nhy, *nlen;
  const double *h, *dhdx, *dhdy, *fcor; /* shallow water: bathymetry, gradient, planetary vorticity */
  const double* relax;                  /* NULL or relaxation field (i,j,v,e), nEq variables */
  const double* rfac;                   /* NULL or relaxation rate: SW timescale (i,j,e); advection (i,j,v,e) */
  const double *u, *v;                  /* advection velocity (i,j,e) */
  double g, drag, dt, kappa;
} orc_dg_problem;

int orc_dg_traces(const orc_dg_problem* p, const double* q, double* bsol);
int orc_dg_edge_flux(const orc_dg_problem* p, double t, const double* bsol, double* bflux);
int orc_dg_tendency(const orc_dg_problem* p, double t, const double* q, double* tend);
int orc_dg_rk3(const orc_dg_problem* p, double tn, int nsteps, double* q);
int orc_sw_bathymetry_gradient(const orc_dg_problem* p, double* dhdx, double* dhdy);
int orc_set_threads(int n);

/* ---------------- CGSEM 2-D (CGsemElliptic_2D_Class.f90) and solvers (IterativeSolvers_Class.f90) */
typedef struct {
  int N, nEl, nEdges, nNodes;
  const double *dmat, *qw;                    /* GLL CG derivative matrix and weights */
  const int* edges;                           /* e2 = ORC_DIRICHLET on boundary edges */
  const int* nodeType;
  const int *n2e_ptr, *n2e_elem, *n2e_local;  /* corner node -> (element, local corner 1..4) in list order */
  const double *dxds, *dxdp, *dyds, *dydp, *J;
  const double* kcoef;                        /* fluxCoeff (i,j,e) */
  double lambda;                              /* Helmholtz mass coefficient, operator -(K + lambda M) */
  int op;                                     /* 0 = -(div k grad) - lambda, 1 = advection-diffusion */
  double vx, vy;
} orc_cg_problem;

int orc_cg_mask(const orc_cg_problem* p, double* u);
int orc_cg_unmask(const orc_cg_problem* p, double* u);
int orc_cg_global_sum(const orc_cg_problem* p, double* u);
int orc_cg_local_operator(const orc_cg_problem* p, const double* u, double* Lu);
int orc_cg_matrix_action(const orc_cg_problem* p, double* u, double* Au);
int orc_cg_residual(const orc_cg_problem* p, const double* source, double* solution, const double* dirichlet,
                    double* r);
double orc_cg_dot(const orc_cg_problem* p, double* u, double* v);
int orc_cg_jacobi_diagonal(const orc_cg_problem* p, double* diag);
/* precond: 0 none, 1 Jacobi.  Stops at ||r||/||r0|| < tol (CGsemElliptic_2D_Class.f90:1188-1193).
 * Returns ioerr (0 converged, -1 not converged); resi has maxIters+1 entries. */
int orc_cg_solve_pcg(const orc_cg_problem* p, const double* source, double* solution, const double* dirichlet,
                     int maxIters, double tol, int precond, double* resi, int* iters);
int orc_cg_solve_gmres(const orc_cg_problem* p, const double* source, double* solution, const double* dirichlet,
                       int m, int maxIters, double tol, double* resi, int* iters);
/* Solve_PCGMRES (IterativeSolvers_Class.f90:656-822): flexible GMRES(m), right preconditioning by Jacobi. */
int orc_cg_solve_pgmres(const orc_cg_problem* p, const double* source, double* solution, const double* dirichlet,
                        int m, int maxIters, double tol, double* resi, int* iters);

/* The reference's linear-FEM preconditioner (CGsemPreconditioner_2D_Class.f90 on the mesh of
 * QuadMeshClass.f90 ConstructLinearMeshFromOther :1863-2092); x, y = GLL node positions of the problem; ids =
 * NULL (nodes identified by position, as the reference) or one node id per local node (equal ids = one node).
 * info: unique corner nodes of the linear mesh and how many of them are DIRICHLET.
 * apply: out (unmasked, original layout) = preconditioner%Solve(b) with pcIters / pcTol, iters = CG steps run.
 * solve: Solve_PCConjugateGradient (CGsemElliptic_2D_Class.f90:1114-1207) with that preconditioner. */
int orc_pc_linear_info(const orc_cg_problem* p, const double* x, const double* y, const int* ids, int* nUnique,
                       int* nDirichlet);
int orc_pc_linear_apply(const orc_cg_problem* p, const double* x, const double* y, const int* ids, int pcIters,
                        double pcTol, const double* b, double* out, int* iters);
int orc_cg_solve_pcg_linear(const orc_cg_problem* p, const double* x, const double* y, const int* ids,
                            const double* source, double* solution, const double* dirichlet, int maxIters, double tol,
                            int pcIters, double pcTol, double* resi, int* iters);

/* ---------------- 1-D CGSEM elliptic example (examples/elliptic1d/parabola/localmods/Elliptic1D_Class.f90) */
int orc_elliptic1d_solve(int N, int nEl, int maxIters, double tol, int cg_quirk, double* x, double* u,
                         double* resi, int* iters);

#ifdef __cplusplus
}
#endif
#endif
