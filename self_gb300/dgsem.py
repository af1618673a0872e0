"""Host-side mirror of SELF's DGSEM 2-D types over the C ABI.

Names follow the reference's type-bound procedures (ConservativeShallowWaterClass.f90:71-151,
AdvectionClass.f90:84-164, NodalStorage_2D_Class.f90, QuadMeshClass.f90) so that a driver written
against the Fortran types reads the same:

    sw = ShallowWater(ctx, nodal, mesh, h, fcor, dt=dt)     # %Build
    sw.SetSolution(q)                                        # %SetSolution for every element
    sw.ForwardStepRK3(tn, nsteps)                            # nsteps x %ForwardStepRK3
    dqdt = sw.GlobalTimeDerivative(t)                        # %GlobalTimeDerivative + %GetTendency
    q = sw.GetSolution()

Arrays are numpy float64 in the Fortran storage order (element-contiguous, i fastest).
"""
import ctypes as C
import os
import weakref

import numpy as np

from . import _native as nat


class Context:
    """One CUDA device + stream (self_ctx)."""

    def __init__(self, device=0):
        p = C.c_void_p()
        nat.check(nat.lib().self_ctx_create(int(device), C.byref(p)))
        self.ptr = p
        self._handles = weakref.WeakSet()  # handles created on this context, released before it

    def adopt(self, handle):
        self._handles.add(handle)

    def synchronize(self):
        nat.check(nat.lib().self_ctx_synchronize(self.ptr), self.ptr)

    def kernel_launches(self):
        return int(nat.lib().self_ctx_kernel_launches(self.ptr))

    def host_loop(self, on=True):
        """(P)CG solves repeat their 16-iteration graph from the host (for kernel profilers) instead of one
        conditional-while graph launch (self_ctx_host_loop)."""
        nat.check(nat.lib().self_ctx_host_loop(self.ptr, 1 if on else 0), self.ptr)

    def close(self):
        if self.ptr:
            for h in list(getattr(self, "_handles", ())):
                h.Trash()
            nat.lib().self_ctx_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class NodalStorage_2D:
    """NodalStorage_2D%Build(N, N, quadrature, form): nodes, weights, derivative matrices, interpolants."""

    def __init__(self, N, quadrature=nat.GAUSS, form=nat.DG):
        n = N + 1
        self.N, self.n, self.quadrature, self.form = N, n, quadrature, form
        self.x, self.w = np.zeros(n), np.zeros(n)
        self.dmatS, self.dmatP = np.zeros(n * n), np.zeros(n * n)
        self.lW, self.lE, self.lS, self.lN = (np.zeros(n) for _ in range(4))
        nat.check(nat.lib().self_nodal_build(N, quadrature, form, nat.d(self.x), nat.d(self.w), nat.d(self.dmatS),
                                             nat.d(self.dmatP), nat.d(self.lW), nat.d(self.lE), nat.d(self.lS),
                                             nat.d(self.lN)))


class QuadMesh:
    """QuadMesh%LoadDefaultMesh + ConstructEdges + ScaleTheMesh on nx x ny elements (optionally periodic and
    warped).  Geometry arrays follow MappedGeometry_2D."""

    def __init__(self, nx, ny, N, quadrature=nat.GAUSS, periodic=(False, False), warp=0.0, scale=(1.0, 1.0),
                 boundary_flag=nat.NO_NORMAL_FLOW):
        nEl, nEd, nNo = C.c_int(), C.c_int(), C.c_int()
        nat.check(nat.lib().self_mesh_counts(nx, ny, int(periodic[0]), int(periodic[1]), C.byref(nEl), C.byref(nEd),
                                             C.byref(nNo)))
        self.nx, self.ny, self.N, self.n = nx, ny, N, N + 1
        self.nEl, self.nEdges, self.nNodes = nEl.value, nEd.value, nNo.value
        n, ne = N + 1, self.nEl
        self.edges = np.zeros(6 * self.nEdges, np.int32)
        self.elemNodes = np.zeros(4 * ne, np.int32)
        self.nodeType = np.zeros(self.nNodes, np.int32)
        self.n2e_ptr = np.zeros(self.nNodes + 1, np.int32)
        self.n2e_elem = np.zeros(4 * ne, np.int32)
        self.n2e_local = np.zeros(4 * ne, np.int32)
        self.x, self.y, self.dxds, self.dxdp, self.dyds, self.dydp, self.J = (np.zeros(n * n * ne) for _ in range(7))
        self.nhx, self.nhy, self.nlen, self.bx, self.by = (np.zeros(n * 4 * ne) for _ in range(5))
        nat.check(nat.lib().self_mesh_build(
            nx, ny, int(periodic[0]), int(periodic[1]), N, quadrature, C.c_double(warp), C.c_double(scale[0]),
            C.c_double(scale[1]), boundary_flag, nat.i(self.edges), nat.i(self.elemNodes), nat.i(self.nodeType),
            nat.i(self.n2e_ptr), nat.i(self.n2e_elem), nat.i(self.n2e_local), nat.d(self.x), nat.d(self.y),
            nat.d(self.dxds), nat.d(self.dxdp), nat.d(self.dyds), nat.d(self.dydp), nat.d(self.J), nat.d(self.nhx),
            nat.d(self.nhy), nat.d(self.nlen), nat.d(self.bx), nat.d(self.by)))


def read_ism_mesh(path, N, quadrature=nat.GAUSS):
    """QuadMesh%ReadSpecMeshFile (QuadMeshClass.f90:2100-2475): a QuadMesh from an ISM-V2 (SpecMesh) file."""
    nEl, nEd, nNo, g = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    bpath = str(path).encode()
    nat.check(nat.lib().self_mesh_ism_counts(bpath, C.byref(nEl), C.byref(nEd), C.byref(nNo), C.byref(g)))
    m = QuadMesh.__new__(QuadMesh)
    m.nx = m.ny = None
    m.N, m.n = N, N + 1
    m.nEl, m.nEdges, m.nNodes, m.geomDegree = nEl.value, nEd.value, nNo.value, g.value
    n, ne = N + 1, m.nEl
    m.edges = np.zeros(6 * m.nEdges, np.int32)
    m.elemNodes = np.zeros(4 * ne, np.int32)
    m.nodeType = np.zeros(m.nNodes, np.int32)
    m.n2e_ptr = np.zeros(m.nNodes + 1, np.int32)
    m.n2e_elem = np.zeros(4 * ne, np.int32)
    m.n2e_local = np.zeros(4 * ne, np.int32)
    m.x, m.y, m.dxds, m.dxdp, m.dyds, m.dydp, m.J = (np.zeros(n * n * ne) for _ in range(7))
    m.nhx, m.nhy, m.nlen, m.bx, m.by = (np.zeros(n * 4 * ne) for _ in range(5))
    nat.check(nat.lib().self_mesh_ism_build(
        bpath, N, quadrature, nat.i(m.edges), nat.i(m.elemNodes), nat.i(m.nodeType), nat.i(m.n2e_ptr),
        nat.i(m.n2e_elem), nat.i(m.n2e_local), nat.d(m.x), nat.d(m.y), nat.d(m.dxds), nat.d(m.dxdp), nat.d(m.dyds),
        nat.d(m.dydp), nat.d(m.J), nat.d(m.nhx), nat.d(m.nhy), nat.d(m.nlen), nat.d(m.bx), nat.d(m.by)))
    return m


def bathymetry_gradient(nodal, mesh, h):
    """CalculateBathymetryGradient for every element (host, FP64)."""
    dhdx, dhdy = np.zeros_like(h), np.zeros_like(h)
    nat.check(nat.lib().self_sw_bathymetry_gradient(
        nodal.N, mesh.nEl, nat.d(nodal.dmatS), nat.d(nodal.dmatP), nat.d(nodal.w), nat.d(nodal.lW),
        nat.d(nodal.lE), nat.d(nodal.lS), nat.d(nodal.lN), nat.d(mesh.dxds), nat.d(mesh.dxdp), nat.d(mesh.dyds),
        nat.d(mesh.dydp), nat.d(mesh.J), nat.d(mesh.nhx), nat.d(mesh.nhy), nat.d(mesh.nlen), nat.d(h),
        nat.d(dhdx), nat.d(dhdy)))
    return dhdx, dhdy


def dg2d_desc(nodal, mesh, model, nEq, dt, precision, g=9.81, linear_drag=0.0, h=None, dhdx=None, dhdy=None,
              fcor=None, u=None, v=None, relax=None, rfac=None, kappa=0.0):
    """self_dg2d_desc over the arrays of a NodalStorage_2D and a QuadMesh; returns (desc, keep): `keep` holds the
    arrays the descriptor points to and must outlive every use of it."""
    s = nat.DG2DDesc()
    s.N, s.nEl, s.nEdges, s.nEq, s.model, s.precision = nodal.N, mesh.nEl, mesh.nEdges, nEq, model, precision
    s.dmatS, s.dmatP, s.qweight = nat.d(nodal.dmatS), nat.d(nodal.dmatP), nat.d(nodal.w)
    s.lagW, s.lagE, s.lagS, s.lagN = nat.d(nodal.lW), nat.d(nodal.lE), nat.d(nodal.lS), nat.d(nodal.lN)
    s.edges = nat.i(mesh.edges)
    s.dxds, s.dxdp, s.dyds, s.dydp, s.J = (nat.d(getattr(mesh, k)) for k in ("dxds", "dxdp", "dyds", "dydp", "J"))
    s.nhx, s.nhy, s.nlen = nat.d(mesh.nhx), nat.d(mesh.nhy), nat.d(mesh.nlen)
    s.h, s.dhdx, s.dhdy, s.fcor = nat.d(h), nat.d(dhdx), nat.d(dhdy), nat.d(fcor)
    s.relax, s.rfac, s.u, s.v = nat.d(relax), nat.d(rfac), nat.d(u), nat.d(v)
    s.g, s.linear_drag, s.dt, s.kappa = g, linear_drag, dt, kappa
    return s, (nodal, mesh, h, dhdx, dhdy, fcor, u, v, relax, rfac)


class _DG2D:
    def __init__(self, ctx, nodal, mesh, model, nEq, dt, precision, g=9.81, linear_drag=0.0, h=None, dhdx=None,
                 dhdy=None, fcor=None, u=None, v=None, relax=None, rfac=None, kappa=0.0):
        s, self._keep = dg2d_desc(nodal, mesh, model, nEq, dt, precision, g, linear_drag, h, dhdx, dhdy, fcor, u, v,
                                  relax, rfac, kappa)
        self.ctx = ctx
        self.nodal, self.mesh, self.nEq, self.dt, self.precision = nodal, mesh, nEq, dt, precision
        self.nq = nodal.n * nodal.n * nEq * mesh.nEl
        p = C.c_void_p()
        nat.check(nat.lib().self_dg2d_create(ctx.ptr, C.byref(s), C.byref(p)), ctx.ptr)
        self.ptr = p
        ctx.adopt(self)

    def _chk(self, st):
        return nat.check(st, self.ctx.ptr)

    def SetSolution(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64).ravel()
        assert q.size == self.nq
        self._chk(nat.lib().self_dg2d_set_state(self.ptr, nat.d(q)))

    def GetSolution(self):
        q = np.zeros(self.nq)
        self._chk(nat.lib().self_dg2d_get_state(self.ptr, nat.d(q)))
        return q

    def GlobalTimeDerivative(self, t=0.0):
        out = np.zeros(self.nq)
        self._chk(nat.lib().self_dg2d_tendency(self.ptr, C.c_double(t), nat.d(out)))
        return out

    def ForwardStepRK3(self, tn=0.0, nsteps=1):
        self._chk(nat.lib().self_dg2d_rk3(self.ptr, C.c_double(tn), int(nsteps)))

    def ForwardStepRK3_async(self, tn=0.0, nsteps=1):
        self._chk(nat.lib().self_dg2d_rk3_async(self.ptr, C.c_double(tn), int(nsteps)))

    def state_device(self):
        p, nb = C.c_void_p(), C.c_size_t()
        self._chk(nat.lib().self_dg2d_state_device(self.ptr, C.byref(p), C.byref(nb)))
        return p.value, nb.value

    def Trash(self):
        if getattr(self, "ptr", None):
            nat.lib().self_dg2d_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.Trash()
        except Exception:
            pass


class ShallowWater(_DG2D):
    """formulation "conservative": ConservativeShallowWater (U=Hu, V=Hv, H) with LLF flux, bathymetry and Coriolis
    sources, mirror walls.  formulation "linear": ShallowWaterClass with ModelFormulation LINEAR (u, v, eta about a
    resting depth h; linear flux with the edge depth, Coriolis, linear drag and relaxation sources).
    formulation "skew_symmetric": ModelFormulation SKEW_SYMMETRIC, 4 state variables (u, v, eta, zeta): the
    relative vorticity zeta is advanced with the state and enters the Coriolis term as f + zeta."""

    def __init__(self, ctx, nodal, mesh, h, fcor, dt, g=9.81, linear_drag=0.0, dhdx=None, dhdy=None,
                 precision=nat.PREC_FP64, relax=None, timescale=None, formulation="conservative"):
        nEq = 3
        if formulation == "linear":
            model = nat.MODEL_SW_LINEAR
        elif formulation == "skew_symmetric":
            model, nEq = nat.MODEL_SW_SKEW, 4
        elif formulation == "conservative":
            model = nat.MODEL_SW_CONSERVATIVE
            if dhdx is None or dhdy is None:
                dhdx, dhdy = bathymetry_gradient(nodal, mesh, h)
        else:
            raise ValueError(f"formulation {formulation!r}")
        super().__init__(ctx, nodal, mesh, model, nEq, dt, precision, g=g, linear_drag=linear_drag,
                         h=h, dhdx=dhdx, dhdy=dhdy, fcor=fcor, relax=relax, rfac=timescale)
        self.h, self.dhdx, self.dhdy, self.fcor = h, dhdx, dhdy, fcor
        self.formulation = formulation

    def WritePickup(self, iteration, directory="."):
        """WritePickup_ShallowWater (ConservativeShallowWaterClass.f90:2013-2064): ShallowWater.<iter>.pickup
        with, per element, the 3 state records, the bathymetry and the planetary vorticity."""
        path = os.path.join(directory, "ShallowWater.%010d.pickup" % iteration)
        q = self.GetSolution()
        h = np.ascontiguousarray(self.h, dtype=np.float64).ravel()
        f = np.ascontiguousarray(self.fcor, dtype=np.float64).ravel()
        write_pickup(path, self.nodal.N, self.mesh.nEl, [(q, 3), (h, 1), (f, 1)])
        return path

    def ReadPickup(self, iteration, directory="."):
        """ReadPickup_ShallowWater (:2068-2126): sets the state from the file and returns (state, h, f).  The
        bathymetry and vorticity define the handle, so a file with other fields needs a new handle."""
        path = os.path.join(directory, "ShallowWater.%010d.pickup" % iteration)
        n2, ne = self.nodal.n * self.nodal.n, self.mesh.nEl
        q, h, f = np.zeros(3 * n2 * ne), np.zeros(n2 * ne), np.zeros(n2 * ne)
        read_pickup(path, self.nodal.N, ne, [(q, 3), (h, 1), (f, 1)])
        self.SetSolution(q)
        return q, h, f


def write_pickup(path, N, nEl, fields):
    """Direct-access big-endian records of (N+1)^2 doubles; fields: [(array, records per element), ...]."""
    arrs = [np.ascontiguousarray(a, dtype=np.float64).ravel() for a, _ in fields]
    recs = (C.c_int * len(fields))(*[r for _, r in fields])
    ptrs = (nat.dp * len(fields))(*[nat.d(a) for a in arrs])
    nat.check(nat.lib().self_pickup_write(path.encode(), N, nEl, len(fields), ptrs, recs))


def read_pickup(path, N, nEl, fields):
    """Fill the given arrays (float64, contiguous; None skips a field) from a pickup file."""
    recs = (C.c_int * len(fields))(*[r for _, r in fields])
    ptrs = (nat.dp * len(fields))(*[nat.d(a) if a is not None else None for a, _ in fields])
    nat.check(nat.lib().self_pickup_read(path.encode(), N, nEl, len(fields), ptrs, recs))


class Advection(_DG2D):
    """Advection(-diffusion) of nTracers with the upwind (Rusanov) flux; kappa > 0 adds the BR1 diffusion passes
    (gradient by the DG weak derivative with central fluxes, flux c u - kappa grad c)."""

    def __init__(self, ctx, nodal, mesh, u, v, dt, nTracers=1, precision=nat.PREC_FP64, relax=None, rfac=None,
                 kappa=0.0):
        super().__init__(ctx, nodal, mesh, nat.MODEL_ADVECTION, nTracers, dt, precision, u=u, v=v, relax=relax,
                         rfac=rfac, kappa=kappa)
        self.kappa = kappa
        self.u, self.v, self.relax, self.rfac = u, v, relax, rfac

    def WritePickup(self, iteration, directory="."):
        """WritePickup_Advection (AdvectionClass.f90:2040-2098): per element the nEq state records, the nEq
        relaxation-field and nEq relaxation-factor records, then u and v."""
        path = os.path.join(directory, "Advection.%010d.pickup" % iteration)
        nq = self.nq
        zero = np.zeros(nq)
        fields = [(self.GetSolution(), self.nEq),
                  (zero if self.relax is None else self.relax, self.nEq),
                  (zero if self.rfac is None else self.rfac, self.nEq),
                  (self.u, 1), (self.v, 1)]
        write_pickup(path, self.nodal.N, self.mesh.nEl, fields)
        return path
