"""Small numeric helpers shared by the tests."""
import numpy as np


def rel_l2(a, b):
    """Norm-wise relative L2 error ||a-b|| / ||b|| (Julia's isapprox uses the norm-wise form)."""
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def rand_c(rng, shape, dtype=np.complex64):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(dtype)


# Modified Shepp-Logan head phantom (Toft, 1996; the published ten-ellipse table):
# intensity, semi-axes a, b, centre x0, y0, rotation (degrees), on [-1, 1]^2.
_SHEPP_LOGAN_MODIFIED = (
    (1.0, 0.69, 0.92, 0.0, 0.0, 0.0),
    (-0.8, 0.6624, 0.874, 0.0, -0.0184, 0.0),
    (-0.2, 0.11, 0.31, 0.22, 0.0, -18.0),
    (-0.2, 0.16, 0.41, -0.22, 0.0, 18.0),
    (0.1, 0.21, 0.25, 0.0, 0.35, 0.0),
    (0.1, 0.046, 0.046, 0.0, 0.1, 0.0),
    (0.1, 0.046, 0.046, 0.0, -0.1, 0.0),
    (0.1, 0.046, 0.023, -0.08, -0.605, 0.0),
    (0.1, 0.023, 0.023, 0.0, -0.606, 0.0),
    (0.1, 0.023, 0.046, 0.06, -0.605, 0.0),
)


def shepp_logan(N, oversample=1):
    """N x N modified Shepp-Logan phantom (first index x, second y, pixels tiling [-1, 1]),
    each pixel the mean over oversample x oversample sub-pixel samples."""
    o = int(oversample)
    c = ((np.arange(N * o) + 0.5) / (N * o)) * 2.0 - 1.0
    X, Y = np.meshgrid(c, -c, indexing="ij")
    img = np.zeros((N * o, N * o))
    for I, a, b, x0, y0, phi in _SHEPP_LOGAN_MODIFIED:
        t = np.deg2rad(phi)
        xr = (X - x0) * np.cos(t) + (Y - y0) * np.sin(t)
        yr = -(X - x0) * np.sin(t) + (Y - y0) * np.cos(t)
        img[(xr / a) ** 2 + (yr / b) ** 2 <= 1.0] += I
    return img.reshape(N, o, N, o).mean(axis=(1, 3))
