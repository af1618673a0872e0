"""Shared helpers of the parity tests: build identical problems for the oracle and the GPU library."""
import numpy as np


def rel_inf(a, b):
    """max |a-b| / max |b| (per-variable relative error in the infinity norm)."""
    den = np.abs(b).max()
    return np.abs(a - b).max() / (den if den > 0 else 1.0)


def per_var_rel(a, b, nEq, n2):
    a = a.reshape(-1, nEq, n2)
    b = b.reshape(-1, nEq, n2)
    return [rel_inf(a[:, v], b[:, v]) for v in range(nEq)]


def connectivity_ids(mesh, N):
    """One node id per local node from the mesh's own shared copies (edge table with start/increment, corner
    node -> element lists): equal ids = one node.  The test-side statement of "identify by connectivity"."""
    n = N + 1
    nn = n * n
    ids = np.arange(mesh.nEl * nn, dtype=np.int64)

    def side_node(side, k):
        return {1: (k, 0), 2: (N, k), 3: (k, N), 4: (0, k)}[side]

    def lid(e, i, j):
        return (e - 1) * nn + i + n * j

    E = np.asarray(mesh.edges).reshape(-1, 6)
    for e1, s1, e2, s2, start, inc in E:
        if e2 <= 0:
            continue
        nn2 = start
        for m in range(1, N):
            a = lid(e1, *side_node(s1, m))
            b = lid(e2, *side_node(abs(s2), nn2))
            ids[b] = ids[a]
            nn2 += inc
    corner = {1: (0, 0), 2: (N, 0), 3: (N, N), 4: (0, N)}
    ptr, el, loc = mesh.n2e_ptr, mesh.n2e_elem, mesh.n2e_local
    for nd in range(mesh.nNodes):
        a, b = ptr[nd], ptr[nd + 1]
        if b <= a:
            continue
        first = lid(el[a], *corner[loc[a]])
        for c in range(a, b):
            ids[lid(el[c], *corner[loc[c]])] = ids[first]
    return ids.astype(np.int32)
