"""Small numeric helpers shared by the tests."""
import numpy as np


def rel_l2(a, b):
    """Norm-wise relative L2 error ||a-b|| / ||b|| (Julia's isapprox uses the norm-wise form)."""
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def rand_c(rng, shape, dtype=np.complex64):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(dtype)
