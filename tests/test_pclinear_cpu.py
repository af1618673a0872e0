"""The restated linear-FEM preconditioner (oracle only, no GPU).

CGsemPreconditioner_2D (CGsemPreconditioner_2D_Class.f90) on the mesh of ConstructLinearMeshFromOther
(QuadMeshClass.f90:1863-2092): node identification by position, boundary nodes Dirichlet, inner CG, and
Solve_PCConjugateGradient (CGsemElliptic_2D_Class.f90:1114-1207) around it.
"""
import os

import numpy as np

from helpers import connectivity_ids

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _square(oracle, N=5, nx=8, warp=0.03, lam=0.1, flag=None):
    import self_gb300 as sg
    from self_gb300 import workloads as W
    nat = sg._native
    nod = sg.NodalStorage_2D(N, nat.GAUSS_LOBATTO, nat.CG)
    mesh = sg.QuadMesh(nx, nx, N, nat.GAUSS_LOBATTO, warp=warp,
                       boundary_flag=nat.DIRICHLET if flag is None else flag)
    k, f, source = W.helmholtz(mesh, N)
    return nod, mesh, source, oracle.CGProblem(nod, mesh, k, lam=lam)


def test_linear_mesh_of_a_structured_mesh(oracle):
    """Every shared GLL node of the structured (warped) mesh is found by position: (nx N + 1)^2 corner nodes of the
    linear mesh, the 4 nx N boundary nodes Dirichlet."""
    for N, nx in ((5, 8), (2, 5), (9, 3)):
        _, _, _, P = _square(oracle, N, nx)
        assert P.pc_linear_info() == ((nx * N + 1) ** 2, 4 * nx * N)


def test_linear_mesh_of_an_ism_mesh_splits_nodes_like_the_reference(oracle):
    """On the SpecMesh square, GLL positions of a shared node computed from different elements can differ by more
    than AlmostEqual's ~1 ulp, so the reference's position search leaves some shared nodes split (more unique
    nodes than the topology has, and the split sides become boundary sides with Dirichlet nodes)."""
    import self_gb300 as sg
    nat = sg._native
    N = 3
    mesh = sg.read_ism_mesh(os.path.join(ROOT, "tests", "golden", "square.mesh"), N, nat.GAUSS_LOBATTO)
    nod = sg.NodalStorage_2D(N, nat.GAUSS_LOBATTO, nat.CG)
    P = oracle.CGProblem(nod, mesh, np.ones(mesh.x.size), lam=0.1)
    nu, nd = P.pc_linear_info()
    topo = mesh.nNodes + mesh.nEdges * (N - 1) + mesh.nEl * (N - 1) ** 2
    nb = int((mesh.edges.reshape(-1, 6)[:, 2] < 0).sum()) * N
    assert nu > topo
    assert nd > nb


def test_zero_preconditioner_iterations_is_plain_cg(oracle):
    """pcIterates = 0 makes the preconditioner u = r: the PCG is the unpreconditioned CG, iterate for iterate."""
    _, _, source, P = _square(oracle, 3, 4, 0.0)
    s1, e1, it1, r1 = P.solve_pcg_linear(source, maxIters=300, tol=1e-10, pcIters=0)
    s2, e2, it2, r2 = P.solve_pcg(source, maxIters=300, tol=1e-10, precond=0)
    assert (e1, it1) == (e2, it2)
    np.testing.assert_array_equal(r1, r2)
    np.testing.assert_array_equal(s1, s2)


def test_preconditioned_solve_reaches_the_jacobi_solution_in_fewer_iterations(oracle):
    _, _, source, P = _square(oracle)
    s1, e1, it1, r1 = P.solve_pcg_linear(source, maxIters=500, tol=1e-10, pcIters=20, pcTol=1e-4)
    s2, e2, it2, _ = P.solve_pcg(source, maxIters=2000, tol=1e-10, precond=1)
    assert e1 == 0 and e2 == 0
    assert it1 < it2 / 4
    assert r1[-1] / r1[0] < 1e-10
    assert np.abs(s1 - s2).max() <= 1e-8 * np.abs(s2).max()


def test_preconditioner_application_properties(oracle):
    """The inner CG stops at pcTol (or after pcIters), its output is unmasked (every copy of a node equal) and zero
    on the boundary; run to a tight tolerance it solves the linear-FEM system, so it is linear in b."""
    _, mesh, source, P = _square(oracle, 4, 5, 0.02)
    rng = np.random.default_rng(1)
    b = rng.normal(size=P.nl)
    P.mask(b)
    P.unmask(b)
    w, it = P.pc_linear_apply(b, pcIters=400, pcTol=1e-13)
    assert 0 < it < 400
    wm = w.copy()
    P.mask(wm)
    wu = wm.copy()
    P.unmask(wu)
    np.testing.assert_array_equal(w, wu)
    w2, _ = P.pc_linear_apply(2.5 * b, pcIters=400, pcTol=1e-13)
    assert np.abs(w2 - 2.5 * w).max() <= 1e-9 * np.abs(w2).max()
    w3, it3 = P.pc_linear_apply(b, pcIters=5, pcTol=1e-4)
    assert it3 == 5
    w0, it0 = P.pc_linear_apply(b, pcIters=0, pcTol=1e-4)
    assert it0 == 0
    np.testing.assert_array_equal(w0, b)


def test_connectivity_ids_give_the_topological_linear_mesh(oracle):
    """Identified by the mesh's own shared copies, the SpecMesh square's linear mesh has the topology's node count
    and only its physical boundary Dirichlet; the preconditioned solve then converges where the position search
    (the reference) stalls."""
    import self_gb300 as sg
    from self_gb300 import workloads as W
    nat = sg._native
    N = 4
    mesh = sg.read_ism_mesh(os.path.join(ROOT, "tests", "golden", "square.mesh"), N, nat.GAUSS_LOBATTO)
    nod = sg.NodalStorage_2D(N, nat.GAUSS_LOBATTO, nat.CG)
    k, f, source = W.helmholtz(mesh, N)
    P = oracle.CGProblem(nod, mesh, k, lam=0.1)
    ids = connectivity_ids(mesh, N)
    topo = mesh.nNodes + mesh.nEdges * (N - 1) + mesh.nEl * (N - 1) ** 2
    nb = int((mesh.edges.reshape(-1, 6)[:, 2] < 0).sum()) * N
    assert P.pc_linear_info(ids) == (topo, nb)
    s1, e1, it1, r1 = P.solve_pcg_linear(source, maxIters=400, tol=1e-10, pcIters=12, ids=ids)
    s0, e0, it0, r0 = P.solve_pcg_linear(source, maxIters=100, tol=1e-10, pcIters=12)
    s2, e2, it2, _ = P.solve_pcg(source, maxIters=3000, tol=1e-10, precond=1)
    assert e1 == 0 and e2 == 0 and it1 < it2
    assert np.abs(s1 - s2).max() <= 1e-8 * np.abs(s2).max()
    assert e0 == -1 and r0[-1] / r0[0] > 1e-2
    # on a structured mesh both identifications give the same linear mesh and the same iterates
    _, _, src2, Q = _square(oracle, 4, 5, 0.02)
    import self_gb300 as sg2  # noqa: F401
    m2 = Q.keep[1]
    a = Q.solve_pcg_linear(src2, maxIters=300, tol=1e-10, pcIters=10)
    b = Q.solve_pcg_linear(src2, maxIters=300, tol=1e-10, pcIters=10, ids=connectivity_ids(m2, 4))
    assert a[2] == b[2]
    np.testing.assert_array_equal(a[3], b[3])
