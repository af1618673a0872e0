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
