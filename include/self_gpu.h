/*
 * self_gpu.h -- C ABI of the GB300 (sm_103a) spectral-element library (libselfgpu.so).
 *
 * It replaces the compute procedures of SELF's Fortran types (lileipku00/SELF) on the
 * spectral-element hot path.  Every entry point is extern "C", takes plain pointers and sizes,
 * and returns an int status (SELF_OK = 0, negative = error; self_last_error() gives the text).
 * A Fortran ISO_C_BINDING module binds these functions one to one.
 *
 * Array conventions are the Fortran ones, so arrays pass without reordering:
 *   matrices     D(i,j) at D[i + j*n], n = N+1 (column major, as DOUBLE D(0:N,0:N))
 *   element data f(i,j,e) at f[i + n*(j + n*e)]            (Fortran f(0:N,0:N,1:nEl))
 *   E-vectors    q(i,j,v,e) at q[i + n*(j + n*(v + nEq*e))] (Fortran G2D(0:N,0:N,1:nEq,1:nEl))
 *   side data    b(i,side,e) at b[i + n*(side + 4*e)], side 0..3 = south, east, north, west
 *   edge table   edges[6*k + 0..5] = e1, s1, e2, s2, start, inc with 1-based element and side
 *                IDs (QuadMeshClass.f90 Edge: e2 < 0 is a boundary flag, s2 < 0 reversed)
 * Handles are not thread safe; distinct handles may be used from distinct threads.  Host arrays
 * are read or written synchronously.  The library owns all device memory it allocates.
 */
#ifndef SELF_GPU_H
#define SELF_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status codes */
#define SELF_OK 0
#define SELF_ERR_INVALID (-1)       /* bad argument or size */
#define SELF_ERR_CUDA (-2)          /* a CUDA runtime call failed */
#define SELF_ERR_ALLOC (-3)         /* device or host allocation failed */
#define SELF_ERR_UNSUPPORTED (-4)   /* option outside the implemented path */
#define SELF_ERR_TIMEOUT (-5)       /* a bounded device wait ran out */
#define SELF_ERR_NOT_CONVERGED (-6) /* iterative solver hit maxIters (ioerr = -1) */
#define SELF_ERR_NONFINITE (-7)     /* NaN or Inf met in a residual */

/* ---------------------------------------------------------------- flags (ModelFlags.f90:80-137) */
#define SELF_NO_NORMAL_FLOW (-100)
#define SELF_INFLOW_ONE (-103)
#define SELF_INFLOW_TWO (-104)
#define SELF_DIRICHLET (-200)
#define SELF_GAUSS 1
#define SELF_GAUSS_LOBATTO (-1)
#define SELF_DG 2000
#define SELF_CG 2001

#define SELF_MODEL_SW_CONSERVATIVE 1 /* ConservativeShallowWaterClass.f90 */
#define SELF_MODEL_ADVECTION 2       /* AdvectionClass.f90 (kappa = 0) */
#define SELF_MODEL_SW_LINEAR 3       /* ShallowWaterClass.f90, ModelFormulation LINEAR: state (u, v, eta) */
/* ShallowWaterClass.f90, ModelFormulation SKEW_SYMMETRIC: nEq = 4, state (u, v, eta, zeta) with the relative
 * vorticity zeta (the reference's vorticity(:)%solution(:,:,2)) advanced by RelativeVorticityEdgeFlux and
 * VorticityTimeDerivative in the same RK3 steps */
#define SELF_MODEL_SW_SKEW 4

#define SELF_PREC_FP64 0 /* plain FP64 drop-in */
#define SELF_PREC_FP32 1 /* FP32 arithmetic; shallow water in perturbation form about the lake at rest */
#define SELF_PREC_FP64_EXACT 2 /* FP64 in the reference's statement order, no FMA contraction, true divisions */

/* ---------------------------------------------------------------- context */
typedef struct self_ctx self_ctx;

/* One context per (process, device).  Replaces nothing in the reference (its drivers run on the
 * host); it carries the CUDA device, stream and the last error text. */
int self_ctx_create(int device, self_ctx** out);
/* Destroy every handle created on a context before the context itself. */
int self_ctx_destroy(self_ctx* ctx);
int self_last_error(const self_ctx* ctx, char* buf, size_t len);
const char* self_status_string(int status);
int self_ctx_synchronize(self_ctx* ctx);
/* 1 when all work enqueued on the context's stream has completed, 0 otherwise (cudaStreamQuery). */
int self_ctx_query(self_ctx* ctx);
/* Page-locked, device-mapped host memory for host<->device transfers at full link speed.  State arrays in such a
 * block are read and written by the conversion kernels directly (no staging copy). */
int self_host_alloc(size_t bytes, void** ptr);
int self_host_free(void* ptr);

/* ---------------------------------------------------------------- host set-up (Build procedures)
 * NodalStorage_2D%Build (NodalStorage_2D_Class.f90:101-230).  form = SELF_DG gives the weak
 * derivative matrix -M^-1 D^T M in both directions; dmatS/dmatP/lag*: n*n and n doubles. */
int self_nodal_build(int N, int quadrature, int form, double* nodes, double* qweights, double* dmatS,
                     double* dmatP, double* lagW, double* lagE, double* lagS, double* lagN);

/* QuadMesh%LoadDefaultMesh + ConstructEdges + ScaleTheMesh (QuadMeshClass.f90:1489-1627,1691-1859)
 * on nx*ny elements of the unit square, with optional periodic connectivity, an optional warp
 * x,y += warp*sin(2 pi x)sin(2 pi y) before scaling by (xscale, yscale), and boundary edges
 * flagged boundary_flag.  Sizes: self_mesh_counts.  Outputs as in the conventions above:
 * edges 6*nEdges; elemNodes 4*nEl; nodeType nNodes; node->element lists n2e_ptr (nNodes+1),
 * n2e_elem/n2e_local (4*nEl); x,y,dxds,dxdp,dyds,dydp,J n*n*nEl; nhx,nhy,nlen,bx,by n*4*nEl. */
int self_mesh_counts(int nx, int ny, int periodic_x, int periodic_y, int* nEl, int* nEdges, int* nNodes);
int self_mesh_build(int nx, int ny, int periodic_x, int periodic_y, int N, int quadrature, double warp,
                    double xscale, double yscale, int boundary_flag, int* edges, int* elemNodes, int* nodeType,
                    int* n2e_ptr, int* n2e_elem, int* n2e_local, double* x, double* y, double* dxds,
                    double* dxdp, double* dyds, double* dydp, double* J, double* nhx, double* nhy,
                    double* nlen, double* bx, double* by);

/* ---------------------------------------------------------------- DGSEM 2-D
 * Replaces ShallowWater (ConservativeShallowWaterClass.f90:71-151) and Advection
 * (AdvectionClass.f90:84-164) compute procedures:
 *   self_dg2d_tendency == %GlobalTimeDerivative(t)        (:1222-1262)  [+ %GetTendency]
 *   self_dg2d_rk3      == nsteps x %ForwardStepRK3(tn)    (:1173-1218)
 *   self_dg2d_set_state/get_state == %SetSolution/%GetSolution for all elements
 * All pointers in the descriptor are host arrays read once at create time. */
typedef struct {
  int N, nEl, nEdges, nEq;
  int model;     /* SELF_MODEL_* */
  int precision; /* SELF_PREC_* */
  const double *dmatS, *dmatP, *qweight, *lagW, *lagE, *lagS, *lagN;
  const int* edges;
  const double *dxds, *dxdp, *dyds, *dydp, *J;
  const double *nhx, *nhy, *nlen;
  const double *h, *dhdx, *dhdy, *fcor; /* shallow water: bathymetry(:,:,1:3), planetary vorticity */
  const double* relax;                  /* optional relaxation field (i,j,v,e) or NULL */
  const double* rfac;                   /* optional: SW relaxation timescale (i,j,e); advection (i,j,v,e) */
  const double *u, *v;                  /* advection velocity (i,j,e) */
  double g, linear_drag, dt;
  /* advection only: diffusivity kappa >= 0; kappa > 0 adds the BR1 passes of AdvectionClass.f90 (gradient by the
   * DG weak derivative with central fluxes, :1123-1264 and :1482-1563; flux c u - kappa grad c; FP64 forms) */
  double kappa;
} self_dg2d_desc;

typedef struct self_dg2d self_dg2d;
int self_dg2d_create(self_ctx* ctx, const self_dg2d_desc* desc, self_dg2d** out);
int self_dg2d_destroy(self_dg2d* h);
int self_dg2d_set_state(self_dg2d* h, const double* q);
int self_dg2d_get_state(self_dg2d* h, double* q);
int self_dg2d_tendency(self_dg2d* h, double t, double* dqdt);
int self_dg2d_rk3(self_dg2d* h, double tn, int nsteps);
/* Same as self_dg2d_rk3 but enqueued only (no host synchronisation); pair with self_ctx_synchronize. */
int self_dg2d_rk3_async(self_dg2d* h, double tn, int nsteps);
/* Device bytes held by the handle (admission control of the serving loop). */
long long self_dg2d_bytes(const self_dg2d* h);
/* Device address of the resident state (FP64: double, FP32: float perturbation form). */
int self_dg2d_state_device(self_dg2d* h, void** dptr, size_t* bytes);

/* Known answer helpers for the shallow-water set-up (host, FP64):
 * CalculateBathymetryGradient (ConservativeShallowWaterClass.f90:1733-1868). */
/* ReadSpecMeshFile_QuadMesh (QuadMeshClass.f90:2100-2475): an ISM-V2 (SpecMesh) file.  counts first, then
 * build into arrays of the sizes self_mesh_build uses; corner nodes, transfinite element geometry from the
 * file's side curves, edges rebuilt from the elements (first-appearance order), boundary flags from the side
 * names (unnamed boundary sides are SELF_NO_NORMAL_FLOW). */
int self_mesh_ism_counts(const char* path, int* nEl, int* nEdges, int* nNodes, int* geomDegree);
int self_mesh_ism_build(const char* path, int N, int quadrature, int* edges, int* elemNodes, int* nodeType,
                        int* n2e_ptr, int* n2e_elem, int* n2e_local, double* x, double* y, double* dxds,
                        double* dxdp, double* dyds, double* dydp, double* J, double* nhx, double* nhy,
                        double* nlen, double* bx, double* by);

int self_sw_bathymetry_gradient(int N, int nEl, const double* dmatS, const double* dmatP, const double* qweight,
                                const double* lagW, const double* lagE, const double* lagS, const double* lagN,
                                const double* dxds, const double* dxdp, const double* dyds, const double* dydp,
                                const double* J, const double* nhx, const double* nhy, const double* nlen,
                                const double* h, double* dhdx, double* dhdy);

/* ---------------------------------------------------------------- pickup (checkpoint) files
 * The reference's restart format (WritePickup/ReadPickup_ShallowWater, ConservativeShallowWaterClass.f90:
 * 2013-2130; _Advection, AdvectionClass.f90:2040-2171): direct-access, big-endian, unformatted records of
 * (N+1)^2 doubles, no record markers.  For every element, for every field f in order, recs[f] records come
 * from fields[f] + (e * recs[f] + r) * (N+1)^2.  Shallow water: {state (3), bathymetry h (1), f (1)};
 * advection: {state (nEq), relaxation field (nEq), relaxation factor (nEq), u (1), v (1)}.  On read a null
 * field is skipped. */
int self_pickup_write(const char* path, int N, int nEl, int nfields, const double* const* fields, const int* recs);
int self_pickup_read(const char* path, int N, int nEl, int nfields, double* const* fields, const int* recs);

/* ---------------------------------------------------------------- CGSEM 2-D
 * Replaces CGsemElliptic_2D (CGsemElliptic_2D_Class.f90:57-93) compute procedures on element-local
 * ("L-vector") arrays u(0:N,0:N,1:nEl) with GLL nodes:
 *   self_cg2d_matrix_action == %MatrixAction(u, Au)   (:930-976)  u is not modified
 *   self_cg2d_residual      == %Residual(dirF, r)      (:980-1068) with source(:,:,:) given
 *   self_cg2d_dot           == %DotProduct(u, v)       (:1072-1110)
 *   self_cg2d_mask/unmask   == %Mask / %UnMask         (:350-542)
 *   self_cg2d_solve         == %Solve (PCG, :1114-1207) and IterativeSolver GMRES (IterativeSolvers_Class.f90:493-652)
 *   self_cg2d_precondition  == %preconditioner%Solve (CGsemPreconditioner_2D_Class.f90:646-746)
 * Operator: op 0 = FluxDivergence - lambda*J*w_i*w_j (weak form of div(k grad u) - lambda u, the reference's
 * sign); op 1 adds the advection term -J*w_i*w_j*(vx du/dx + vy du/dy) (nonsymmetric; use GMRES). */
typedef struct {
  int N, nEl, nEdges, nNodes;
  const double *dmat, *qweight; /* GLL derivative matrix (CG form) and weights */
  const int* edges;             /* e2 = SELF_DIRICHLET on Dirichlet edges */
  const int* nodeType;          /* corner node types (SELF_DIRICHLET marks prescribed nodes) */
  const int *n2e_ptr, *n2e_elem, *n2e_local; /* corner node -> (element, local corner 1..4), list order */
  const double *dxds, *dxdp, *dyds, *dydp, *J;
  const double* fluxCoeff; /* k(i,j,e) */
  double lambda;
  int op;
  double vx, vy;
  /* GLL node positions x(i,j,e), y(i,j,e): only SELF_SOLVE_PCG_LINEAR needs them (NULL otherwise), to build the
   * bilinear sub-quads of the reference's preconditioner mesh (QuadMeshClass.f90 ConstructLinearMeshFromOther
   * :1863-2092). */
  const double *x, *y;
} self_cg2d_desc;

#define SELF_SOLVE_CG 0           /* conjugate gradient, no preconditioner */
#define SELF_SOLVE_PCG_JACOBI 1   /* conjugate gradient, assembled-diagonal (Jacobi) preconditioner */
#define SELF_SOLVE_GMRES 2        /* GMRES(m), modified Gram-Schmidt + Givens */
#define SELF_SOLVE_PGMRES_JACOBI 3 /* flexible right-preconditioned GMRES(m) (Solve_PCGMRES), Jacobi */
/* conjugate gradient preconditioned by the reference's linear-FEM inner CG (CGsemElliptic_2D %Solve =
 * Solve_PCConjugateGradient :1114-1207 with CGsemPreconditioner_2D %Solve :646-746): w = pc_iterations CG steps
 * (or fewer, to ||r||/||r0|| < pc_tolerance) on the N = 1 mesh of the GLL nodes (nodes identified by position as
 * the reference does), k = 1, the nodes of unshared sub-quad sides Dirichlet; pc_iterations = 0 makes w = r.
 * Needs desc x, y. */
#define SELF_SOLVE_PCG_LINEAR 4

typedef struct {
  int method;             /* SELF_SOLVE_* */
  int precision;          /* SELF_PREC_FP64: plain; SELF_PREC_FP32: FP32 inner CG under FP64 iterative refinement */
  int maxIters;           /* iteration cap (total inner iterations for FP32 refinement) */
  int m;                  /* GMRES restart length */
  double tolerance;       /* stop at ||r|| / ||r0|| < tolerance (FP64 residual) */
  double inner_tolerance; /* FP32 inner solve: relative reduction per refinement step (default 1e-4) */
  int max_outer;          /* refinement steps cap (default 30) */
  int pc_iterations;      /* SELF_SOLVE_PCG_LINEAR: inner CG steps per application (CGsemParams pcIterates, 50) */
  double pc_tolerance;    /* SELF_SOLVE_PCG_LINEAR: inner stop ||r||/||r0|| < pc_tolerance (pcTolerance, 1e-4) */
  int pc_nodes;           /* SELF_SOLVE_PCG_LINEAR: SELF_PC_NODES_POSITION or SELF_PC_NODES_CONNECTIVITY */
  /* FP32 inner CG at N = 7: nonzero runs the element operator's derivative contractions on the tensor cores
   * (tcgen05 GEMMs of 32-element tiles, compensated TF32 products); 0 uses the CUDA-core line form */
  int tensor_cores;
  /* storage of the (P)CG vectors (the FP32 inner iterations and the FP64 solve): SELF_LAYOUT_COMPACT (default)
   * one value per unknown, grouped by mesh entity (element interiors, edges, corners), when the mesh is conforming
   * (FP64: and N >= 5, the even-odd operator; else the element-local form); SELF_LAYOUT_LOCAL the masked
   * element-local L-vectors.  The linear-FEM preconditioner and the tensor-core apply run on the element-local form;
   * GMRES always does. */
  int inner_layout;
} self_solve_opts;
#define SELF_LAYOUT_COMPACT 0
#define SELF_LAYOUT_LOCAL 1
/* How the preconditioner mesh identifies shared GLL nodes.  POSITION is the reference (AlmostEqual positions,
 * ~1 ulp): where positions of one node computed in different elements differ by more (transfinite elements, e.g.
 * SpecMesh files), the node stays split, the split sub-quad sides become Dirichlet and the PCG can stall, as the
 * reference's does.  CONNECTIVITY takes the spectral mesh's own shared copies (no split nodes). */
#define SELF_PC_NODES_POSITION 0
#define SELF_PC_NODES_CONNECTIVITY 1

typedef struct {
  int ioerr;            /* 0 converged, -1 not converged (reference meanings), -2 other */
  int iterations;       /* CG iterations / GMRES Arnoldi steps (sum over refinement steps) */
  int outer_iterations; /* refinement steps (1 for FP64) */
  double r0;            /* ||r0|| (masked FP64 residual of the initial guess) */
  double rel_residual;  /* final ||r|| / ||r0|| */
} self_solve_report;

typedef struct self_cg2d self_cg2d;
int self_cg2d_create(self_ctx* ctx, const self_cg2d_desc* desc, self_cg2d** out);
int self_cg2d_destroy(self_cg2d* h);
int self_cg2d_matrix_action(self_cg2d* h, const double* u, double* Au);
/* The FP32 form of MatrixAction that the FP32 inner solves use (u and Au masked L-vectors in FP64 on the host, the
 * operator in FP32), in one of the inner solves' forms: SELF_F32_LOCAL (element-local L-vectors, CUDA-core line
 * contractions), SELF_F32_TENSOR_CORES (N = 7 only: the derivative contractions on the tensor cores with compensated
 * TF32 products, as self_solve_opts.tensor_cores), SELF_F32_COMPACT (the compact node layout of
 * self_solve_opts.inner_layout; SELF_ERR_UNSUPPORTED on a mesh it does not cover). */
#define SELF_F32_LOCAL 0
#define SELF_F32_TENSOR_CORES 1
#define SELF_F32_COMPACT 2
int self_cg2d_matrix_action_f32(self_cg2d* h, const double* u, double* Au, int form);
int self_cg2d_residual(self_cg2d* h, const double* source, const double* solution, double* r);
int self_cg2d_dot(self_cg2d* h, const double* u, const double* v, double* out);
int self_cg2d_mask(self_cg2d* h, double* u);
int self_cg2d_unmask(self_cg2d* h, double* u);
/* solution: initial guess in, solution out (unmasked, Dirichlet values from `dirichlet` or 0 when NULL).
 * resi: NULL or maxIters+1 doubles (||r|| per iteration; per refinement step for the FP32 form). */
int self_cg2d_solve(self_cg2d* h, const self_solve_opts* opts, const double* source, const double* dirichlet,
                    double* solution, double* resi, self_solve_report* report);
/* == preconditioner%Solve(w, UnMask(r)) of Solve_PCConjugateGradient (CGsemPreconditioner_2D_Class.f90:646-746):
 * one application of the linear-FEM preconditioner in FP64 with opts.pc_iterations / opts.pc_tolerance.
 * r: residual L-vector (masked or unmasked); w: result, unmasked; iterations: inner CG steps run (may be NULL). */
int self_cg2d_precondition(self_cg2d* h, const self_solve_opts* opts, const double* r, double* w, int* iterations);

/* ---------------------------------------------------------------- batched uneven CGSEM solves
 * Many independent Helmholtz problems (op 0; different meshes and degrees N = 2..9) solved together: one
 * launch per phase covers every problem, inner iterations replay as CUDA graphs, converged problems skip their
 * work.  Each problem is the PCG-Jacobi of self_cg2d_solve from a zero initial guess with homogeneous
 * Dirichlet values; opts.precision = SELF_PREC_FP32 runs FP32 inner solves under FP64 iterative refinement. */
typedef struct self_cgbatch self_cgbatch;
/* nprob problems in slots 0..nprob-1 (nprob may be 0 for an empty pool filled by self_cgbatch_add) */
int self_cgbatch_create(self_ctx* ctx, int nprob, const self_cg2d_desc* descs, self_cgbatch** out);
int self_cgbatch_destroy(self_cgbatch* b);
/* set the source of slot p and restart its solve from a zero initial guess */
int self_cgbatch_set_source(self_cgbatch* b, int p, const double* source);
int self_cgbatch_problem_size(self_cgbatch* b, int p, long long* nlocal);
/* solve every problem in the pool in one launch of a graph whose conditional while node repeats the tick on the
 * device until every problem finished; reports in slot order */
int self_cgbatch_solve(self_cgbatch* b, const self_solve_opts* opts, self_solve_report* reports);
int self_cgbatch_get_solution(self_cgbatch* b, int p, double* solution);
/* continuous batching: add a problem to a free slot (its solve starts at the next step), remove a slot,
 * advance every unfinished problem by one step (outer updates + graph-captured inner iterations), read a
 * slot's report; footprint = device bytes a problem would take (admission control). */
int self_cgbatch_add(self_cgbatch* b, const self_cg2d_desc* desc, const double* source, int* slot);
int self_cgbatch_remove(self_cgbatch* b, int slot);
int self_cgbatch_step(self_cgbatch* b, const self_solve_opts* opts, int* nfinished);
int self_cgbatch_report(self_cgbatch* b, int slot, self_solve_report* report, int* finished);
int self_cgbatch_footprint(const self_cg2d_desc* desc, long long* bytes);
long long self_cgbatch_bytes(const self_cgbatch* b);
/* Project autotuner: times element-tile sizes of the element operator (1, 2, 4, ... 32 rounds of one node per
 * thread) per (N, element-count bucket: <=256, <=1024, <=4096, larger) and keeps the fastest; cache_path (JSON)
 * is read first and written after.  self_cgbatch_tuning returns the elements per tile in use. */
int self_cgbatch_autotune(self_cgbatch* b, const char* cache_path);
int self_cgbatch_tuning(self_cgbatch* b, int N, int bucket, int* elements_per_tile);

/* ---------------------------------------------------------------- continuous-batching request loop
 * No counterpart in the reference (its drivers run one model at a time).  A worker thread inside the library owns
 * every CUDA call of the loop; submit / poll / result / cancel / stats may be called from any thread.  Requests are
 * admitted in arrival order while their device footprint fits hbm_budget_bytes (and while fewer than max_active
 * run, when max_active > 0):
 *   solve requests (Helmholtz, op 0) join one batched slot pool: each tick advances every admitted solve -- outer
 *   FP64 residual step, outer decision and inner PCG iterations, all on the device -- with one synchronisation;
 *   shallow-water requests run their RK3 steps on their own handle on one of sw_streams extra streams, in chunks
 *   of sw_chunk steps enqueued asynchronously (kernels overlap the solves).
 * A result is bit-identical to the same request served alone.  The caller keeps every array the descriptor points
 * to, and the source / initial state, alive until poll reports the request done, failed or cancelled.  The ctx
 * must not be used by the caller while the loop exists. */
typedef struct self_serve self_serve;
typedef struct {
  double hbm_budget_bytes; /* admission limit: device bytes of the requests on the GPU */
  int precision;           /* solves: SELF_PREC_FP32 (FP32 inner / FP64 refinement) or SELF_PREC_FP64 */
  double tolerance;        /* solves stop at ||r||/||r0|| < tolerance (FP64 residual) */
  double inner_tolerance;  /* FP32 inner solves: relative reduction per refinement step (default 1e-4) */
  int max_outer;           /* refinement steps cap (default 30) */
  int maxIters;            /* inner iterations cap per solve (default 100000) */
  int sw_streams;          /* extra streams for shallow-water requests (default 4) */
  int sw_chunk;            /* RK3 steps enqueued per chunk (default 10) */
  int max_active;          /* requests on the GPU at once; 0 = no cap, 1 = one request at a time */
} self_serve_opts;
#define SELF_SERVE_SOLVE 0
#define SELF_SERVE_SW 1
#define SELF_SERVE_QUEUED 0
#define SELF_SERVE_RUNNING 1
#define SELF_SERVE_DONE 2
#define SELF_SERVE_CANCELLED 3
#define SELF_SERVE_FAILED 4
typedef struct {
  int state, kind, status;            /* SELF_SERVE_*, status of a failed request */
  int steps_done;                     /* shallow-water request: RK3 steps enqueued so far */
  double submit_s, admit_s, done_s;   /* seconds since the loop was created (-1: not yet) */
  self_solve_report report;           /* solve request: as self_cg2d_solve reports it */
} self_serve_info;
typedef struct {
  long long submitted, admitted, finished, cancelled, failed, queued, running, bytes_in_use;
  double p50_ms, p99_ms, mean_ms;     /* latency (done - submit) of the finished requests */
  double throughput_per_s;            /* finished / (last done - first submit) */
  double elapsed_s;
} self_serve_statistics;
int self_serve_create(self_ctx* ctx, const self_serve_opts* opts, self_serve** out);
/* stops the worker (requests still queued or running are cancelled) and frees everything */
int self_serve_destroy(self_serve* s);
/* Helmholtz solve (desc as self_cg2d_create, op 0; source as self_cg2d_solve; zero initial guess, homogeneous
 * Dirichlet values): returns a ticket */
int self_serve_submit_solve(self_serve* s, const self_cg2d_desc* desc, const double* source, long long* ticket);
/* shallow-water ensemble member: `steps` RK3 steps from the state q0 (desc as self_dg2d_create) */
int self_serve_submit_sw(self_serve* s, const self_dg2d_desc* desc, const double* q0, int steps, long long* ticket);
int self_serve_poll(self_serve* s, long long ticket, self_serve_info* info);
/* result of a done request: the solve's solution (L-vector, unmasked) or the member's final state; n values */
int self_serve_result(self_serve* s, long long ticket, double* out, size_t n);
/* forget a finished / cancelled / failed request (its result) */
int self_serve_release(self_serve* s, long long ticket);
int self_serve_cancel(self_serve* s, long long ticket);
/* wait until nothing is queued or running (SELF_ERR_TIMEOUT after timeout_s seconds) */
int self_serve_wait(self_serve* s, double timeout_s);
int self_serve_stats(self_serve* s, self_serve_statistics* st);

/* ---------------------------------------------------------------- dot product without allocation
 * No counterpart in the reference.  For callers that cannot allocate device memory where they need an inner
 * product -- Fortran codes whose device arrays live in their own OpenACC / CUDA Fortran data regions and forbid
 * allocation inside the time loop, latency-bound loops that cannot take an allocation stall -- this computes
 * result = sum_k x[k]*y[k] in FP64 on the current device: a two-pass reduction over contiguous tiles of 16384
 * elements, deterministic for a given n and equal to self_cg2d_dot up to rounding, whose partial sums live in a
 * fixed static device array (32 KiB, held by every GPU that loads the library until exit) instead of
 * cudaMalloc'd memory.  x, y (n doubles) and result (one double) are device pointers; stream may be NULL.
 * n <= 67,108,864 (4096 partials x 16384 elements); larger n returns SELF_ERR_INVALID.  The call allocates
 * nothing; its first call in a CUDA context looks up the array's address there (a new context, e.g. after
 * cudaDeviceReset, looks it up again).  Calls that overlap on the GPU share the array and race; serialise them.
 * An error left pending by earlier work is reported, not cleared.  Errors: self_last_error(NULL, ...). */
int self_dot_noalloc(const double* x, const double* y, long long n, double* result, void* stream);

/* ---------------------------------------------------------------- measurement helpers
 * Not part of the drop-in (no reference counterpart): launch accounting, timers, L2 eviction and peak probes used
 * to measure the entry points above. */
/* number of kernels this context launched so far (for launch accounting) */
long long self_ctx_kernel_launches(const self_ctx* ctx);
/* CUDA-event timer on the context's stream: start records an event, stop records a second one,
 * synchronises and returns the elapsed milliseconds between them. */
int self_ctx_timer_start(self_ctx* ctx);
int self_ctx_timer_stop(self_ctx* ctx, double* ms);
/* Overwrite a scratch buffer of `bytes` on the context's stream (evicts L2 between timed steps). */
int self_ctx_flush_l2(self_ctx* ctx, size_t bytes);
/* host_loop != 0: the context's single-problem (P)CG solves repeat their captured 16-iteration graph from the host
 * (one synchronisation per graph) instead of one launch of a conditional-while graph, so that kernel profilers,
 * which do not list kernels inside conditional graph nodes, see every launch.  The same kernels and iterations;
 * 0 (the default) restores the device-side loop. */
int self_ctx_host_loop(self_ctx* ctx, int host_loop);
/* Measured fused-multiply-add rate of the device (TFLOP/s, FP64 when fp64 != 0 else FP32): the compute
 * roofline used for kernels bound by the FP64 pipe. */
int self_probe_fma_peak(self_ctx* ctx, int fp64, double* tflops);
/* Average CUDA-event time (ms) of one launch of each kernel of an RK stage, each launch preceded by an L2 flush
 * of flush_bytes; the resident state is restored afterwards.  ms[0] = edge-flux kernel, ms[1] = volume +
 * RK-update kernel. */
int self_dg2d_time_kernels(self_dg2d* h, int reps, size_t flush_bytes, double* ms);
/* Failure-detection test hook (no reference counterpart): arms the bounded bulk-copy waits of the fused FP32
 * shallow-water stage (N = 7) for the next self_dg2d_rk3 call only.  In that call the first wait of every warp
 * polls a shared-memory barrier that nothing arrives on, gives up after `polls` polls, drains the warp's copies in
 * flight with the normal limit and returns without writing; self_dg2d_rk3 then returns SELF_ERR_TIMEOUT and the
 * handle's state is unchanged.  Other handles: SELF_ERR_UNSUPPORTED. */
int self_dg2d_test_wait_timeout(self_dg2d* h, int polls);

#ifdef __cplusplus
}
#endif
#endif /* SELF_GPU_H */
