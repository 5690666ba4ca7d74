"""Seeded synthetic inputs: random-ellipse phantoms and noisy sinograms.

The ellipse rasterisation follows the reference's phantom code (`exp_shepp.py:44-50`): pixel centres on
`linspace(-1, 1, N)` in both axes (`meshgrid(..., indexing="ij")`, so axis 0 is y and axis 1 is x), a rotated
ellipse indicator `((x-x0)cos p + (y-y0) sin p)^2/a^2 + (-(x-x0) sin p + (y-y0) cos p)^2/b^2 <= 1`, and additive
intensities. Parameters are drawn from one `numpy.random.default_rng(seed)` stream, per ellipse in the order
centre (x0, y0) ~ U[-0.6, 0.6]^2, semi-axes (a, b) ~ U[0.05, 0.4]^2, angle p ~ U[0, pi), intensity ~ U[-0.5, 1.0].
"""

import numpy as np


def ellipse_params(rng, count):
    """(count, 6) array of (x0, y0, a, b, phi, intensity), drawn ellipse by ellipse from `rng`."""
    out = np.empty((count, 6))
    for e in range(count):
        out[e, 0:2] = rng.uniform(-0.6, 0.6, 2)
        out[e, 2:4] = rng.uniform(0.05, 0.4, 2)
        out[e, 4] = rng.uniform(0.0, np.pi)
        out[e, 5] = rng.uniform(-0.5, 1.0)
    return out


def rasterise(N, params):
    """Sum of ellipse indicators times intensities on the N x N grid (float64)."""
    g = np.linspace(-1.0, 1.0, N)
    y, x = np.meshgrid(g, g, indexing="ij")
    img = np.zeros((N, N))
    for x0, y0, a, b, p, amp in params:
        c, s = np.cos(p), np.sin(p)
        xr = (x - x0) * c + (y - y0) * s
        yr = -(x - x0) * s + (y - y0) * c
        img[(xr / a) ** 2 + (yr / b) ** 2 <= 1.0] += amp
    return img


def ellipse_phantom(N, seed, ellipses=10, texture=0.0):
    """One phantom. `texture` > 0 adds texture * (float32 uniform [0, 1) image) drawn after the ellipses from the
    same stream (the large-N workload uses 40 ellipses and texture 0.1)."""
    rng = np.random.default_rng(seed)
    img = rasterise(N, ellipse_params(rng, ellipses))
    if texture:
        img = img + texture * rng.random((N, N), dtype=np.float32).astype(np.float64)
    return img


def add_noise(b, rel_sigma, seed):
    """b + sigma * N(0, 1) on every sinogram entry, sigma = rel_sigma * max|b| (structural zeros included)."""
    rng = np.random.default_rng(seed)
    sigma = rel_sigma * float(np.abs(b).max())
    return b + sigma * rng.standard_normal(b.shape)


def int_image(N, seed, lo=0, hi=255):
    """Integer image with values uniform in [lo, hi] (int32)."""
    return np.random.default_rng(seed).integers(lo, hi + 1, size=(N, N), dtype=np.int32)
