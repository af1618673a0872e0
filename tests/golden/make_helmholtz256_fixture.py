"""Makes tests/golden/helmholtz256_n7_pcg.npz: the oracle's converged PCG-Jacobi solution of the 256x256 N=7
Helmholtz problem (k = 1 + 0.5 sin(4 pi x) cos(4 pi y), lambda = 0.1, Dirichlet 0, seeded Fourier right-hand side,
seed 3) to ||r||/||r0|| < 1e-10, sampled at 8192 seeded local nodes, with the solution's max-abs, its iteration
count and residual history every 100 iterations.  The solve takes minutes on a host (too slow for each test run);
the test compares the GPU's FP64 and FP32-refined solutions with it.

    python tests/golden/make_helmholtz256_fixture.py
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

N, NX, SEED, NSAMPLE = 7, 256, 3, 8192


def problem(O):
    from self_gb300 import workloads as W
    nod = O.Nodal(N, O.GAUSS_LOBATTO, O.CG)
    mesh = O.Mesh(NX, NX, N, O.GAUSS_LOBATTO, boundary_flag=O.DIRICHLET)
    k, f, source = W.helmholtz(mesh, N, seed=SEED)
    return nod, mesh, k, source


def sample_index(nl):
    return np.sort(np.random.default_rng(12345).choice(nl, NSAMPLE, replace=False)).astype(np.int64)


if __name__ == "__main__":
    from oracle import oracle as O
    O.build()
    O.set_threads(os.cpu_count())
    nod, mesh, k, source = problem(O)
    P = O.CGProblem(nod, mesh, k, lam=0.1)
    t0 = time.time()
    sol, ioerr, it, resi = P.solve_pcg(source, maxIters=50000, tol=1e-10, precond=1)
    el = time.time() - t0
    assert ioerr == 0, ioerr
    idx = sample_index(sol.size)
    np.savez_compressed(os.path.join(HERE, "helmholtz256_n7_pcg.npz"), idx=idx, u=sol[idx],
                        umax=np.abs(sol).max(), iterations=it, resi_every100=resi[::100],
                        resi_first21=resi[:21])
    print(f"{it} iterations in {el:.0f} s, max |u| = {np.abs(sol).max():.6e}")
