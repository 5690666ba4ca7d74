"""Oracle (test infrastructure only): NumPy restatements of the reference's iterative pseudoinverse (pinv.py) and of
the row-wise normal operator of its `adrt` package patch (patches/adrt-gram-freq.patch).

Nothing in the product imports this module; only tests use it, as the checker. Its parity with the reference is
pinned by tests/golden/pinv_gram_vectors.npz (made by tests/golden/make_golden_pinv.py, which runs the reference's
pinv.py and adrtcore.py and compiles the patch's C++ gram_freq).
"""

import numpy as np

from . import adrt_np as A
from .oblique_np import Tq, TqT, bfly_levels, bflyT_levels


def _ip(a, b):
    """pinv.py:19-20."""
    return float(np.vdot(a, b).real)


def cgls(n, b, tol=1e-12, maxit=10000, x0=None):
    """CGLS for min ||R x - b|| (pinv.py:23-48); returns (x, hist)."""
    N = 1 << n
    b = np.asarray(b, dtype=float).reshape(4, 2 * N - 1, N)
    x = np.zeros((N, N)) if x0 is None else np.array(x0, dtype=float)
    r = b - A.adrt(n, x)
    s = A.adrt_T(n, r)
    p = s.copy()
    gamma = _ip(s, s)
    g0 = np.sqrt(gamma)
    hist = [g0]
    for _ in range(maxit):
        q = A.adrt(n, p)
        alpha = gamma / _ip(q, q)
        x += alpha * p
        r -= alpha * q
        s = A.adrt_T(n, r)
        gnew = _ip(s, s)
        hist.append(np.sqrt(gnew))
        if np.sqrt(gnew) <= tol * g0:
            break
        p = s + (gnew / gamma) * p
        gamma = gnew
    return x, np.array(hist)


def pcg_normal(n, b, M, tol=1e-12, maxit=10000, x0=None, rhs=None):
    """PCG for R^T R x = R^T b with preconditioner M (pinv.py:51-82); returns (x, hist of ||r||_2)."""
    N = 1 << n
    if rhs is None:
        rhs = A.adrt_T(n, np.asarray(b, dtype=float).reshape(4, 2 * N - 1, N))

    def G(v):
        return A.adrt_T(n, A.adrt(n, v))

    x = np.zeros((N, N)) if x0 is None else np.array(x0, dtype=float)
    r = rhs - G(x)
    z = M(r)
    p = z.copy()
    rho = _ip(r, z)
    r0 = np.linalg.norm(r)
    hist = [r0]
    for _ in range(maxit):
        q = G(p)
        alpha = rho / _ip(p, q)
        x += alpha * p
        r -= alpha * q
        rn = np.linalg.norm(r)
        hist.append(rn)
        if rn <= tol * r0:
            break
        z = M(r)
        rho_new = _ip(r, z)
        p = z + (rho_new / rho) * p
        rho = rho_new
    return x, np.array(hist)


# ---------------------------------------------------------------- patches/adrt-gram-freq.patch
def gram_freq(a, omega):
    """A_omega^* A_omega row by row (patch: adrt_cdefs_gram.hpp gram_freq, lines 161-250): a (..., rows, N) complex,
    omega (rows,) real; the forward levels 1..n then the adjoint levels n..1, z = exp(i omega) per row. The
    restatement uses this oracle's butterflies (cpp/oblique.cpp:22-51, the same level arithmetic)."""
    a = np.asarray(a)
    rows, N = a.shape[-2], a.shape[-1]
    n = N.bit_length() - 1
    z = np.exp(1j * np.asarray(omega, dtype=float))
    X = a.reshape(-1, rows, N).astype(np.complex128)
    out = np.empty_like(X)
    for i in range(X.shape[0]):
        out[i] = bflyT_levels(n, z, bfly_levels(n, z, X[i], 1, n), 1, n)
    return out.reshape(a.shape)


def gram(a):
    """R^T R a (patch: core.py gram): quadrant strips of the zero-padded 2N x 2N image packed in pairs (0,1), (2,3)
    as real + i imag, an FFT along the offset, gram_freq at omega = 2 pi fftfreq(2N), the inverse FFT, the strips'
    adjoints summed and cropped."""
    a = np.asarray(a, dtype=float)
    N = a.shape[-1]
    n = N.bit_length() - 1
    L = 2 * N
    X = np.zeros((L, L))
    X[:N, :N] = a
    packed = [Tq(n, 0, X) + 1j * Tq(n, 1, X), Tq(n, 2, X) + 1j * Tq(n, 3, X)]
    om = 2 * np.pi * np.fft.fftfreq(L)
    out = np.zeros((L, L))
    for k, P in enumerate(packed):
        w = np.fft.ifft(gram_freq(np.fft.fft(P, axis=0), om), axis=0)
        out += TqT(n, 2 * k, w.real) + TqT(n, 2 * k + 1, w.imag)
    return out[:N, :N]


def lstsq_cheb(b, lam_min, lam_max, tol=1e-10, degree=None):
    """x_D = c_D(R^T R) R^T b (patch: core.py lstsq_cheb), with y = R^T b from the spatial transpose."""
    b = np.asarray(b, dtype=float)
    N = b.shape[-1]
    n = N.bit_length() - 1
    y = A.adrt_T(n, b)
    lo, hi = float(lam_min), float(lam_max)
    if degree is None:
        kap = hi / lo
        rho = (np.sqrt(kap) - 1) / (np.sqrt(kap) + 1)
        deg = max(1, int(np.ceil(np.log(tol / 2) / np.log(rho))))
    else:
        deg = int(degree)
    c, a = (hi - lo) / (hi + lo), 2.0 / (hi + lo)
    x_prev, x = np.zeros_like(y), a * y
    om = 1.0
    for k in range(1, deg):
        om = 1.0 / (1.0 - c * c / 2.0) if k == 1 else 1.0 / (1.0 - c * c * om / 4.0)
        r = y - gram(x)
        x_prev, x = x, x + om * (a * r) + (om - 1.0) * (x - x_prev)
    return x
