"""ctypes front end of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py (cpu_baseline leg and --impl reference) import this
module.  It loads oracle/_build/liboracle.so (built by oracle/Makefile) and exposes the restated
reference routines on numpy arrays laid out exactly like the Fortran storage (see oracle.h).
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "liboracle.so")

NO_NORMAL_FLOW = -100
INFLOW_ONE = -103
INFLOW_TWO = -104
DIRICHLET = -200
GAUSS = 1
GAUSS_LOBATTO = -1
DG = 2000
CG = 2001

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def build():
    subprocess.check_call(["make", "-s", "-C", _HERE])


def _load():
    if not os.path.exists(_LIB):
        build()
    return C.CDLL(_LIB)


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = _load()
    return _lib


def _d(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"], (a.dtype, a.flags)
    return a.ctypes.data_as(_dp)


def _i(a):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_ip)


def set_threads(n):
    lib().orc_set_threads(int(n))


# --------------------------------------------------------------------------- nodal
def quadrature(N, quad):
    x = np.zeros(N + 1)
    w = np.zeros(N + 1)
    rc = lib().orc_legendre_quadrature(N, quad, _d(x), _d(w))
    assert rc == 0
    return x, w


def derivative_matrix(N, x):
    D = np.zeros((N + 1) * (N + 1))
    lib().orc_derivative_matrix(N, _d(np.ascontiguousarray(x, dtype=np.float64)), _d(D))
    return D.reshape(N + 1, N + 1, order="F")


class Nodal:
    """NodalStorage_2D: nodes, weights, derivative matrices (column-major flat), boundary interpolants."""

    def __init__(self, N, quad, form, quirk_dmatp=0):
        n = N + 1
        self.N, self.n = N, n
        self.x = np.zeros(n)
        self.w = np.zeros(n)
        self.dmatS = np.zeros(n * n)
        self.dmatP = np.zeros(n * n)
        self.lW, self.lE, self.lS, self.lN = (np.zeros(n) for _ in range(4))
        rc = lib().orc_nodal_build(N, quad, form, quirk_dmatp, _d(self.x), _d(self.w), _d(self.dmatS),
                                   _d(self.dmatP), _d(self.lW), _d(self.lE), _d(self.lS), _d(self.lN))
        assert rc == 0


# --------------------------------------------------------------------------- mesh
class Mesh:
    """Structured quad mesh with edge table, corner-node lists and mapped geometry."""

    def __init__(self, nx, ny, N, quad, periodic=(False, False), warp=0.0, scale=(1.0, 1.0),
                 boundary_flag=NO_NORMAL_FLOW):
        nEl, nEd, nNo = C.c_int(), C.c_int(), C.c_int()
        rc = lib().orc_mesh_counts(nx, ny, int(periodic[0]), int(periodic[1]), C.byref(nEl), C.byref(nEd),
                                   C.byref(nNo))
        assert rc == 0, "bad mesh size"
        self.nEl, self.nEdges, self.nNodes = nEl.value, nEd.value, nNo.value
        n = N + 1
        self.N, self.n = N, n
        ne = self.nEl
        self.edges = np.zeros(6 * self.nEdges, np.int32)
        self.elemNodes = np.zeros(4 * ne, np.int32)
        self.nodeType = np.zeros(self.nNodes, np.int32)
        self.n2e_ptr = np.zeros(self.nNodes + 1, np.int32)
        self.n2e_elem = np.zeros(4 * ne, np.int32)
        self.n2e_local = np.zeros(4 * ne, np.int32)
        f = lambda: np.zeros(n * n * ne)
        self.x, self.y, self.dxds, self.dxdp, self.dyds, self.dydp, self.J = (f() for _ in range(7))
        b = lambda: np.zeros(n * 4 * ne)
        self.nhx, self.nhy, self.nlen, self.bx, self.by = (b() for _ in range(5))
        rc = lib().orc_mesh_build(nx, ny, int(periodic[0]), int(periodic[1]), N, quad, C.c_double(warp),
                                  C.c_double(scale[0]), C.c_double(scale[1]), boundary_flag, _i(self.edges),
                                  _i(self.elemNodes), _i(self.nodeType), _i(self.n2e_ptr), _i(self.n2e_elem),
                                  _i(self.n2e_local), _d(self.x), _d(self.y), _d(self.dxds), _d(self.dxdp),
                                  _d(self.dyds), _d(self.dydp), _d(self.J), _d(self.nhx), _d(self.nhy),
                                  _d(self.nlen), _d(self.bx), _d(self.by))
        assert rc == 0, rc


class IsmMesh:
    """Mesh read from an ISM-V2 file (ReadSpecMeshFile_QuadMesh): same attributes as Mesh."""

    def __init__(self, path, N, quad):
        nEl, nEd, nNo, g = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        rc = lib().orc_ism_counts(str(path).encode(), C.byref(nEl), C.byref(nEd), C.byref(nNo), C.byref(g))
        assert rc == 0, "unreadable mesh file"
        self.nEl, self.nEdges, self.nNodes, self.geomDegree = nEl.value, nEd.value, nNo.value, g.value
        n = N + 1
        self.N, self.n = N, n
        ne = self.nEl
        self.edges = np.zeros(6 * self.nEdges, np.int32)
        self.elemNodes = np.zeros(4 * ne, np.int32)
        self.nodeType = np.zeros(self.nNodes, np.int32)
        self.n2e_ptr = np.zeros(self.nNodes + 1, np.int32)
        self.n2e_elem = np.zeros(4 * ne, np.int32)
        self.n2e_local = np.zeros(4 * ne, np.int32)
        f = lambda: np.zeros(n * n * ne)
        self.x, self.y, self.dxds, self.dxdp, self.dyds, self.dydp, self.J = (f() for _ in range(7))
        b = lambda: np.zeros(n * 4 * ne)
        self.nhx, self.nhy, self.nlen, self.bx, self.by = (b() for _ in range(5))
        rc = lib().orc_ism_build(str(path).encode(), N, quad, _i(self.edges), _i(self.elemNodes),
                                 _i(self.nodeType), _i(self.n2e_ptr), _i(self.n2e_elem), _i(self.n2e_local),
                                 _d(self.x), _d(self.y), _d(self.dxds), _d(self.dxdp), _d(self.dyds), _d(self.dydp),
                                 _d(self.J), _d(self.nhx), _d(self.nhy), _d(self.nlen), _d(self.bx), _d(self.by))
        assert rc == 0, rc


# --------------------------------------------------------------------------- DG
class _DGProblem(C.Structure):
    _fields_ = [("N", C.c_int), ("nEl", C.c_int), ("nEdges", C.c_int), ("nEq", C.c_int), ("model", C.c_int),
                ("dmatS", _dp), ("dmatP", _dp), ("qw", _dp), ("lW", _dp), ("lE", _dp), ("lS", _dp), ("lN", _dp),
                ("edges", _ip), ("dxds", _dp), ("dxdp", _dp), ("dyds", _dp), ("dydp", _dp), ("J", _dp),
                ("nhx", _dp), ("nhy", _dp), ("nlen", _dp), ("h", _dp), ("dhdx", _dp), ("dhdy", _dp),
                ("fcor", _dp), ("relax", _dp), ("rfac", _dp), ("u", _dp), ("v", _dp),
                ("g", C.c_double), ("drag", C.c_double), ("dt", C.c_double), ("kappa", C.c_double)]


class DGProblem:
    """Shallow water (model=1, nEq=3) or linear advection (model=2) on a Mesh with a Nodal (DG, GAUSS)."""

    def __init__(self, nodal, mesh, model, nEq, dt, g=9.81, drag=0.0, h=None, dhdx=None, dhdy=None, fcor=None,
                 u=None, v=None, relax=None, rfac=None, kappa=0.0):
        self.keep = [nodal, mesh, h, dhdx, dhdy, fcor, u, v, relax, rfac]
        s = _DGProblem()
        s.N, s.nEl, s.nEdges, s.nEq, s.model = nodal.N, mesh.nEl, mesh.nEdges, nEq, model
        s.dmatS, s.dmatP, s.qw = _d(nodal.dmatS), _d(nodal.dmatP), _d(nodal.w)
        s.lW, s.lE, s.lS, s.lN = _d(nodal.lW), _d(nodal.lE), _d(nodal.lS), _d(nodal.lN)
        s.edges = _i(mesh.edges)
        s.dxds, s.dxdp, s.dyds, s.dydp, s.J = (_d(getattr(mesh, k)) for k in ("dxds", "dxdp", "dyds", "dydp", "J"))
        s.nhx, s.nhy, s.nlen = _d(mesh.nhx), _d(mesh.nhy), _d(mesh.nlen)
        s.h, s.dhdx, s.dhdy, s.fcor = _d(h), _d(dhdx), _d(dhdy), _d(fcor)
        s.relax, s.rfac = _d(relax), _d(rfac)
        s.u, s.v = _d(u), _d(v)
        s.g, s.drag, s.dt, s.kappa = g, drag, dt, kappa
        self.s = s
        self.nodal, self.mesh, self.nEq = nodal, mesh, nEq
        self.nq = nodal.n * nodal.n * nEq * mesh.nEl
        self.nb = nodal.n * nEq * 4 * mesh.nEl

    def traces(self, q):
        bs = np.zeros(self.nb)
        lib().orc_dg_traces(C.byref(self.s), _d(q), _d(bs))
        return bs

    def edge_flux(self, t, bs):
        bf = np.zeros(self.nb)
        rc = lib().orc_dg_edge_flux(C.byref(self.s), C.c_double(t), _d(bs), _d(bf))
        assert rc == 0
        return bf

    def tendency(self, q, t=0.0):
        out = np.zeros(self.nq)
        rc = lib().orc_dg_tendency(C.byref(self.s), C.c_double(t), _d(q), _d(out))
        assert rc == 0, rc
        return out

    def rk3(self, q, nsteps, tn=0.0):
        q = np.array(q, dtype=np.float64, copy=True)
        rc = lib().orc_dg_rk3(C.byref(self.s), C.c_double(tn), int(nsteps), _d(q))
        assert rc == 0, rc
        return q

    def bathymetry_gradient(self):
        n = self.nodal.n
        dx = np.zeros(n * n * self.mesh.nEl)
        dy = np.zeros_like(dx)
        lib().orc_sw_bathymetry_gradient(C.byref(self.s), _d(dx), _d(dy))
        return dx, dy


# --------------------------------------------------------------------------- CG
class _CGProblem(C.Structure):
    _fields_ = [("N", C.c_int), ("nEl", C.c_int), ("nEdges", C.c_int), ("nNodes", C.c_int),
                ("dmat", _dp), ("qw", _dp), ("edges", _ip), ("nodeType", _ip),
                ("n2e_ptr", _ip), ("n2e_elem", _ip), ("n2e_local", _ip),
                ("dxds", _dp), ("dxdp", _dp), ("dyds", _dp), ("dydp", _dp), ("J", _dp), ("kcoef", _dp),
                ("lam", C.c_double), ("op", C.c_int), ("vx", C.c_double), ("vy", C.c_double)]


class CGProblem:
    """CGSEM 2-D on a Mesh built with GAUSS_LOBATTO and boundary_flag = DIRICHLET."""

    def __init__(self, nodal, mesh, kcoef, lam=0.0, op=0, vel=(0.0, 0.0)):
        self.keep = [nodal, mesh, kcoef]
        s = _CGProblem()
        s.N, s.nEl, s.nEdges, s.nNodes = nodal.N, mesh.nEl, mesh.nEdges, mesh.nNodes
        s.dmat, s.qw = _d(nodal.dmatS), _d(nodal.w)
        s.edges, s.nodeType = _i(mesh.edges), _i(mesh.nodeType)
        s.n2e_ptr, s.n2e_elem, s.n2e_local = _i(mesh.n2e_ptr), _i(mesh.n2e_elem), _i(mesh.n2e_local)
        s.dxds, s.dxdp, s.dyds, s.dydp, s.J = (_d(getattr(mesh, k)) for k in ("dxds", "dxdp", "dyds", "dydp", "J"))
        s.kcoef = _d(kcoef)
        s.lam, s.op, s.vx, s.vy = lam, op, vel[0], vel[1]
        self.s = s
        self.nl = nodal.n * nodal.n * mesh.nEl

    def mask(self, u):
        lib().orc_cg_mask(C.byref(self.s), _d(u))

    def unmask(self, u):
        lib().orc_cg_unmask(C.byref(self.s), _d(u))

    def global_sum(self, u):
        lib().orc_cg_global_sum(C.byref(self.s), _d(u))

    def local_operator(self, u):
        out = np.zeros(self.nl)
        lib().orc_cg_local_operator(C.byref(self.s), _d(u), _d(out))
        return out

    def matrix_action(self, u):
        u = np.array(u, dtype=np.float64, copy=True)
        out = np.zeros(self.nl)
        rc = lib().orc_cg_matrix_action(C.byref(self.s), _d(u), _d(out))
        assert rc == 0
        return out

    def residual(self, source, solution, dirichlet=None):
        r = np.zeros(self.nl)
        sol = np.array(solution, dtype=np.float64, copy=True)
        lib().orc_cg_residual(C.byref(self.s), _d(source), _d(sol), _d(dirichlet), _d(r))
        return r

    def dot(self, u, v):
        u = np.array(u, dtype=np.float64, copy=True)
        v = np.array(v, dtype=np.float64, copy=True)
        f = lib().orc_cg_dot
        f.restype = C.c_double
        return f(C.byref(self.s), _d(u), _d(v))

    def jacobi_diagonal(self):
        d = np.zeros(self.nl)
        lib().orc_cg_jacobi_diagonal(C.byref(self.s), _d(d))
        return d

    def solve_pcg(self, source, solution=None, maxIters=5000, tol=1e-10, precond=1, dirichlet=None):
        sol = np.zeros(self.nl) if solution is None else np.array(solution, dtype=np.float64, copy=True)
        resi = np.zeros(maxIters + 1)
        it = C.c_int()
        ioerr = lib().orc_cg_solve_pcg(C.byref(self.s), _d(source), _d(sol), _d(dirichlet), maxIters,
                                       C.c_double(tol), precond, _d(resi), C.byref(it))
        return sol, ioerr, it.value, resi[: it.value + 1]

    def solve_pgmres(self, source, solution=None, m=30, maxIters=2000, tol=1e-10, dirichlet=None):
        """Solve_PCGMRES with the Jacobi preconditioner."""
        sol = np.zeros(self.nl) if solution is None else np.array(solution, dtype=np.float64, copy=True)
        resi = np.zeros(maxIters + 1)
        it = C.c_int()
        ioerr = lib().orc_cg_solve_pgmres(C.byref(self.s), _d(source), _d(sol), _d(dirichlet), m, maxIters,
                                          C.c_double(tol), _d(resi), C.byref(it))
        return sol, ioerr, it.value, resi[: min(it.value, maxIters) + 1]

    def _xy(self):
        mesh = self.keep[1]
        return _d(mesh.x), _d(mesh.y)

    @staticmethod
    def _ids(ids):
        return None if ids is None else _i(np.ascontiguousarray(ids, dtype=np.int32))

    def pc_linear_info(self, ids=None):
        """(unique corner nodes, DIRICHLET nodes) of the reference's linear preconditioner mesh (nodes by position,
        or by the given per-node ids)."""
        nu, nd = C.c_int(), C.c_int()
        x, y = self._xy()
        ids = None if ids is None else np.ascontiguousarray(ids, dtype=np.int32)
        assert lib().orc_pc_linear_info(C.byref(self.s), x, y, self._ids(ids), C.byref(nu), C.byref(nd)) == 0
        return nu.value, nd.value

    def pc_linear_apply(self, b, pcIters=50, pcTol=1e-4, ids=None):
        """preconditioner%Solve(b): the linear-FEM inner CG, output unmasked on the original nodes."""
        out = np.zeros(self.nl)
        it = C.c_int()
        x, y = self._xy()
        b = np.ascontiguousarray(b, dtype=np.float64)
        ids = None if ids is None else np.ascontiguousarray(ids, dtype=np.int32)
        assert lib().orc_pc_linear_apply(C.byref(self.s), x, y, self._ids(ids), pcIters, C.c_double(pcTol), _d(b),
                                         _d(out), C.byref(it)) == 0
        return out, it.value

    def solve_pcg_linear(self, source, solution=None, maxIters=2000, tol=1e-10, pcIters=50, pcTol=1e-4,
                         dirichlet=None, ids=None):
        """Solve_PCConjugateGradient with the reference's linear-FEM preconditioner."""
        sol = np.zeros(self.nl) if solution is None else np.array(solution, dtype=np.float64, copy=True)
        resi = np.zeros(maxIters + 1)
        it = C.c_int()
        x, y = self._xy()
        ids = None if ids is None else np.ascontiguousarray(ids, dtype=np.int32)
        ioerr = lib().orc_cg_solve_pcg_linear(C.byref(self.s), x, y, self._ids(ids), _d(source), _d(sol),
                                              _d(dirichlet), maxIters, C.c_double(tol), pcIters, C.c_double(pcTol),
                                              _d(resi), C.byref(it))
        return sol, ioerr, it.value, resi[: it.value + 1]

    def solve_gmres(self, source, solution=None, m=30, maxIters=2000, tol=1e-10, dirichlet=None):
        sol = np.zeros(self.nl) if solution is None else np.array(solution, dtype=np.float64, copy=True)
        resi = np.zeros(maxIters + 1)
        it = C.c_int()
        ioerr = lib().orc_cg_solve_gmres(C.byref(self.s), _d(source), _d(sol), _d(dirichlet), m, maxIters,
                                         C.c_double(tol), _d(resi), C.byref(it))
        return sol, ioerr, it.value, resi[: min(it.value, maxIters) + 1]


def elliptic1d(N=5, nEl=10, maxIters=1000, tol=1e-8, cg_quirk=1):
    nd = (N + 1) * nEl
    x = np.zeros(nd)
    u = np.zeros(nd)
    resi = np.zeros(maxIters + 1)
    it = C.c_int()
    ioerr = lib().orc_elliptic1d_solve(N, nEl, maxIters, C.c_double(tol), cg_quirk, _d(x), _d(u), _d(resi),
                                       C.byref(it))
    return x, u, resi, it.value, ioerr


def pickup_bytes(N, nEl, fields):
    """Bytes of a pickup file as WritePickup_ShallowWater / WritePickup_Advection write it
    (ConservativeShallowWaterClass.f90:2013-2064, AdvectionClass.f90:2040-2098): ACCESS='direct',
    CONVERT='big_endian', RECL = 8 (N+1)^2 bytes, records in the order element -> field -> record, each record
    the (N+1)^2 values of sol(:,:,iEq) with iS fastest.  fields: [(array, records per element), ...]."""
    nn = (N + 1) ** 2
    out = []
    for e in range(nEl):
        for a, r in fields:
            a = np.asarray(a, dtype=np.float64).reshape(nEl, r, nn)
            for k in range(r):
                out.append(a[e, k].astype(">f8").tobytes())
    return b"".join(out)
