"""Host-side mirror of SELF's CGsemElliptic_2D and its iterative solvers over the C ABI.

Method names follow CGsemElliptic_2D_Class.f90:57-93 and IterativeSolvers_Class.f90:55-186:

    cg = CGsemElliptic_2D(ctx, nodal, mesh, fluxCoeff, lam=0.1)  # %Build (mesh with DIRICHLET boundary)
    Au = cg.MatrixAction(u)                                       # %MatrixAction
    r = cg.Residual(source, solution)                             # %Residual
    d = cg.DotProduct(u, v)                                       # %DotProduct
    sol, rep = cg.Solve(source, method="pcg")                     # %Solve  (or "cg", "gmres", "pgmres")
    sol, rep = cg.Solve(source, method="pcg_linear")              # %Solve with the reference's linear-FEM
                                                                  # preconditioner (pcIterates / pcTolerance)
    w, its = cg.Precondition(r)                                   # %preconditioner%Solve

Arrays are element-local float64 vectors u(0:N,0:N,1:nEl) flattened in Fortran order.
"""
import ctypes as C

import numpy as np

from . import _native as nat

SOLVE_CG, SOLVE_PCG_JACOBI, SOLVE_GMRES, SOLVE_PGMRES_JACOBI, SOLVE_PCG_LINEAR = 0, 1, 2, 3, 4
PC_NODES = {"position": 0, "connectivity": 1}  # how the linear-FEM preconditioner mesh finds shared nodes


class CG2DDesc(C.Structure):
    _fields_ = [("N", C.c_int), ("nEl", C.c_int), ("nEdges", C.c_int), ("nNodes", C.c_int),
                ("dmat", nat.dp), ("qweight", nat.dp), ("edges", nat.ip), ("nodeType", nat.ip),
                ("n2e_ptr", nat.ip), ("n2e_elem", nat.ip), ("n2e_local", nat.ip),
                ("dxds", nat.dp), ("dxdp", nat.dp), ("dyds", nat.dp), ("dydp", nat.dp), ("J", nat.dp),
                ("fluxCoeff", nat.dp), ("lam", C.c_double), ("op", C.c_int), ("vx", C.c_double), ("vy", C.c_double),
                ("x", nat.dp), ("y", nat.dp)]


class SolveOpts(C.Structure):
    _fields_ = [("method", C.c_int), ("precision", C.c_int), ("maxIters", C.c_int), ("m", C.c_int),
                ("tolerance", C.c_double), ("inner_tolerance", C.c_double), ("max_outer", C.c_int),
                ("pc_iterations", C.c_int), ("pc_tolerance", C.c_double), ("pc_nodes", C.c_int),
                ("tensor_cores", C.c_int), ("inner_layout", C.c_int)]

    def __init__(self, *a, **kw):
        super().__init__(*a, **kw)
        if "pc_iterations" not in kw:  # CGsemParams defaults (pcIterates = 50, pcTolerance = 1e-4)
            self.pc_iterations, self.pc_tolerance = 50, 1e-4


class SolveReport(C.Structure):
    _fields_ = [("ioerr", C.c_int), ("iterations", C.c_int), ("outer_iterations", C.c_int), ("r0", C.c_double),
                ("rel_residual", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


INNER_LAYOUTS = {"compact": 0, "local": 1}  # SELF_LAYOUT_COMPACT, SELF_LAYOUT_LOCAL
F32_FORMS = {"local": 0, "tensor_cores": 1, "compact": 2}  # SELF_F32_LOCAL, _TENSOR_CORES, _COMPACT
_METHODS = {"cg": SOLVE_CG, "pcg": SOLVE_PCG_JACOBI, "pcg_jacobi": SOLVE_PCG_JACOBI, "gmres": SOLVE_GMRES,
            "pgmres": SOLVE_PGMRES_JACOBI, "pcg_linear": SOLVE_PCG_LINEAR}


def cg2d_desc(nodal, mesh, fluxCoeff, lam=0.0, op=0, vel=(0.0, 0.0)):
    """self_cg2d_desc over the arrays of a NodalStorage_2D (GLL, CG form) and a QuadMesh; returns (desc, keep):
    `keep` holds the arrays the descriptor points to and must outlive every use of it."""
    s = CG2DDesc()
    s.N, s.nEl, s.nEdges, s.nNodes = nodal.N, mesh.nEl, mesh.nEdges, mesh.nNodes
    s.dmat, s.qweight = nat.d(nodal.dmatS), nat.d(nodal.w)
    s.edges, s.nodeType = nat.i(mesh.edges), nat.i(mesh.nodeType)
    s.n2e_ptr, s.n2e_elem, s.n2e_local = nat.i(mesh.n2e_ptr), nat.i(mesh.n2e_elem), nat.i(mesh.n2e_local)
    s.dxds, s.dxdp, s.dyds, s.dydp, s.J = (nat.d(getattr(mesh, k)) for k in ("dxds", "dxdp", "dyds", "dydp", "J"))
    fluxCoeff = np.ascontiguousarray(fluxCoeff, dtype=np.float64)
    s.fluxCoeff = nat.d(fluxCoeff)
    s.lam, s.op, s.vx, s.vy = lam, op, vel[0], vel[1]
    s.x, s.y = nat.d(mesh.x), nat.d(mesh.y)  # node positions: the linear-FEM preconditioner's mesh
    return s, (nodal, mesh, fluxCoeff)


class CGsemElliptic_2D:
    """op=0: weak -div(k grad u) + lam u with the reference's sign (MatrixAction = -(K + lam M) u);
    op=1: advection-diffusion -kappa Lap u + v.grad u (kappa in fluxCoeff), same sign convention."""

    def __init__(self, ctx, nodal, mesh, fluxCoeff, lam=0.0, op=0, vel=(0.0, 0.0)):
        s, self._keep = cg2d_desc(nodal, mesh, fluxCoeff, lam, op, vel)
        self.ctx, self.nodal, self.mesh = ctx, nodal, mesh
        self.nl = nodal.n * nodal.n * mesh.nEl
        p = C.c_void_p()
        nat.check(nat.lib().self_cg2d_create(ctx.ptr, C.byref(s), C.byref(p)), ctx.ptr)
        self.ptr = p
        ctx.adopt(self)

    def _chk(self, st):
        return nat.check(st, self.ctx.ptr)

    @staticmethod
    def _vec(a):
        return np.ascontiguousarray(a, dtype=np.float64).ravel()

    def MatrixAction(self, u):
        u = self._vec(u)
        out = np.zeros(self.nl)
        self._chk(nat.lib().self_cg2d_matrix_action(self.ptr, nat.d(u), nat.d(out)))
        return out

    def MatrixAction32(self, u, tensor_cores=False, form=None):
        """MatrixAction with the FP32 operator of the inner solves, on masked L-vectors: form "local" (element-local
        vectors, CUDA-core contractions), "tensor_cores" (N = 7; also tensor_cores=True) or "compact" (the compact
        node layout)."""
        form = form or ("tensor_cores" if tensor_cores else "local")
        u = self._vec(u)
        out = np.zeros(self.nl)
        self._chk(nat.lib().self_cg2d_matrix_action_f32(self.ptr, nat.d(u), nat.d(out), F32_FORMS[form]))
        return out

    def Residual(self, source, solution):
        out = np.zeros(self.nl)
        self._chk(nat.lib().self_cg2d_residual(self.ptr, nat.d(self._vec(source)), nat.d(self._vec(solution)),
                                               nat.d(out)))
        return out

    def DotProduct(self, u, v):
        out = C.c_double()
        self._chk(nat.lib().self_cg2d_dot(self.ptr, nat.d(self._vec(u)), nat.d(self._vec(v)), C.byref(out)))
        return out.value

    def Mask(self, u):
        u = self._vec(u).copy()
        self._chk(nat.lib().self_cg2d_mask(self.ptr, nat.d(u)))
        return u

    def UnMask(self, u):
        u = self._vec(u).copy()
        self._chk(nat.lib().self_cg2d_unmask(self.ptr, nat.d(u)))
        return u

    def Solve(self, source, solution=None, method="pcg", precision="fp64", maxIters=20000, tolerance=1e-10, m=30,
              inner_tolerance=1e-4, max_outer=30, dirichlet=None, return_resi=False, pc_iterations=50,
              pc_tolerance=1e-4, pc_nodes="position", tensor_cores=False, inner_layout="compact"):
        o = SolveOpts()
        o.tensor_cores = 1 if tensor_cores else 0
        o.inner_layout = INNER_LAYOUTS[inner_layout]
        o.method = _METHODS[method]
        o.precision = nat.PREC_FP32 if precision == "fp32" else nat.PREC_FP64
        o.maxIters, o.m, o.tolerance = maxIters, m, tolerance
        o.inner_tolerance, o.max_outer = inner_tolerance, max_outer
        o.pc_iterations, o.pc_tolerance, o.pc_nodes = pc_iterations, pc_tolerance, PC_NODES[pc_nodes]
        sol = np.zeros(self.nl) if solution is None else self._vec(solution).copy()
        resi = np.zeros(maxIters + 1) if return_resi else None
        rep = SolveReport()
        self._chk(nat.lib().self_cg2d_solve(self.ptr, C.byref(o), nat.d(self._vec(source)),
                                            nat.d(None if dirichlet is None else self._vec(dirichlet)), nat.d(sol),
                                            nat.d(resi), C.byref(rep)))
        out = rep.as_dict()
        if return_resi:
            out["resi"] = resi
        return sol, out

    def Precondition(self, r, pc_iterations=50, pc_tolerance=1e-4, pc_nodes="position"):
        """preconditioner%Solve(w, UnMask(r)): the linear-FEM inner CG (FP64).  Returns (w unmasked, CG steps).
        pc_nodes "position" finds shared nodes by position as the reference does, "connectivity" by the mesh's
        own shared copies."""
        o = SolveOpts()
        o.pc_iterations, o.pc_tolerance, o.pc_nodes = pc_iterations, pc_tolerance, PC_NODES[pc_nodes]
        w = np.zeros(self.nl)
        its = C.c_int()
        self._chk(nat.lib().self_cg2d_precondition(self.ptr, C.byref(o), nat.d(self._vec(r)), nat.d(w), C.byref(its)))
        return w, its.value

    def Trash(self):
        if getattr(self, "ptr", None):
            nat.lib().self_cg2d_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.Trash()
        except Exception:
            pass
