"""Host (FP64 NumPy) forms of the level-1 stencils, used only by the setup's generalised eigenproblem
(the M = P^{-1} operator of the Lanczos run, fastops.py:318-319). The apply path runs these on the GPU."""

import numpy as np


def G1_apply(x):
    """G_1 x = 8x + J(K x) + (J(K x^T))^T, K = tridiag(1, 2, 1) along axis 0, J = column-pair swap
    (fasthybrid.py:81-98)."""
    x = np.asarray(x, dtype=float)

    def k_rows(v):
        y = 2.0 * v
        y[1:] += v[:-1]
        y[:-1] += v[1:]
        return y

    def j_cols(v):
        y = np.empty_like(v)
        y[:, 0::2] = v[:, 1::2]
        y[:, 1::2] = v[:, 0::2]
        return y

    return 8.0 * x + j_cols(k_rows(x)) + j_cols(k_rows(x.T)).T


def Pi_apply(x):
    """2x2-cell averaging (fasthybrid.py:101-105)."""
    N = x.shape[0]
    c = x.reshape(N // 2, 2, N // 2, 2).mean(axis=(1, 3))
    return np.repeat(np.repeat(c, 2, axis=0), 2, axis=1)


def lorr_fwd(y):
    """4y + 8 Pi y (fastops.py:318)."""
    return 4.0 * y + 8.0 * Pi_apply(y)
