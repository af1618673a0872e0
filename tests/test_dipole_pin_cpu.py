"""Pin of the 2-D set-up against the reference's one shipped 2-D output: the dipole run's energy curve
(examples/shallowwater/dipole/run/Energies.0000000000.curve, made by the dipole example's own integrator:
IntegrateEnergies / CalculateEnergies of examples/shallowwater/dipole/localmods/ConservativeShallowWaterClass.f90
:2091-2161 over box.mesh, N = 10 Legendre-Gauss, ScaleTheMesh by 4e5 m).

PE(t=0) = sum over elements, then nodes (iP outer, iS inner), of 1/2 g eta^2 J w_i w_j with the dipole free surface
of ShallowWater_InitialConditions.f90 (InitialCondition :92-130): eta = dn (exp(-|x-x0|^2/(2L^2)) -
exp(-|x-x1|^2/(2L^2))), dn = f0 vMax L / g.  It depends on the ISM-V2 reader, the transfinite element geometry,
the Jacobians, the mesh scaling and the Gauss quadrature at N = 10, and on nothing in the time stepping.

The shipped namelist (run/shallowwater.params: vMax = 1.75, L = 1e4, iterInit = 600000) cannot have produced this
curve: its PE(0) is 2.17e7, not 1.10e8, and a run from iterInit = 600000 would write Energies.0000600000.curve.
With vMax = 1.5 and L = 2.5e4 (the other dipole parameters as shipped) PE(0) agrees to 16 of the 17 printed digits,
in the oracle's set-up and in the product's.  KE(0) and the values at t = 500, 1000 also depend on the run's
bathymetry, which the shipped files do not determine (the shipped shelf gives KE(0) 29 % low), so they stay
unpinned.
"""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
MESH = os.path.join(HERE, "golden", "box.mesh")
N, SCALE, G, F0 = 10, 4.0e5, 9.81, 1.0e-4
X0, Y0, X1, Y1 = 2.0e5, 205000.0, 2.0e5, 195000.0


def _curve():
    vals = {}
    key = None
    for line in open(os.path.join(HERE, "golden", "dipole_energies.curve")):
        s = line.split()
        if not s:
            continue
        if s[0].startswith("#"):
            key = s[0][1:]
            vals[key] = []
        else:
            vals[key].append((float(s[0]), float(s[1])))
    return vals


def _pe(x, y, J, w, nEl, vmax, L):
    """CalculateEnergies' PE summed per element (iP outer, iS inner), then over elements in order."""
    n = N + 1
    dn = F0 * vmax * L / G
    c0 = (x - X0) ** 2 + (y - Y0) ** 2
    c1 = (x - X1) ** 2 + (y - Y1) ** 2
    eta = dn * (np.exp(-0.5 * c0 / (L * L)) - np.exp(-0.5 * c1 / (L * L)))
    w2 = np.outer(w, w).ravel(order="F")  # w_i w_j at i + n j
    pe = (0.5 * G * eta * eta * J * np.tile(w2, nEl)).reshape(nEl, n * n)
    total = 0.0
    for e in range(nEl):
        loc = 0.0
        for v in pe[e]:
            loc += v
        total += loc
    return total


def test_curve_fixture_shape():
    c = _curve()
    assert [t for t, _ in c["KE"]] == [0.0, 500.0, 1000.0] and [t for t, _ in c["PE"]] == [0.0, 500.0, 1000.0]


@pytest.mark.parametrize("side", ["oracle", "product"])
def test_dipole_pe0_matches_reference_curve(oracle, side):
    pe_ref = _curve()["PE"][0][1]
    if side == "oracle":
        nod = oracle.Nodal(N, oracle.GAUSS, oracle.DG)
        mesh = oracle.IsmMesh(MESH, N, oracle.GAUSS)
    else:
        import self_gb300 as sg
        nod = sg.NodalStorage_2D(N, sg._native.GAUSS, sg._native.DG)
        mesh = sg.read_ism_mesh(MESH, N, sg._native.GAUSS)
    x, y, J = mesh.x * SCALE, mesh.y * SCALE, mesh.J * SCALE * SCALE  # ScaleTheMesh (MappedGeometry_2D :921-948)
    pe = _pe(x, y, J, nod.w, mesh.nEl, vmax=1.5, L=2.5e4)
    assert abs(pe - pe_ref) <= 1e-14 * pe_ref, (pe, pe_ref)
    # the shipped namelist's dipole gives a PE(0) five times smaller: it is not the run that wrote the curve
    pe_shipped = _pe(x, y, J, nod.w, mesh.nEl, vmax=1.75, L=1.0e4)
    assert 0.15 < pe_shipped / pe_ref < 0.25
