"""Oracle (test infrastructure only): NumPy FP64 restatement of the reference's explicit oblique inverses.

Restates, function by function, `fastspec.py`, `fasthybrid.py`, `fastops.py` and the Python side of `fastcpp.py`
of dsrim/adrt-pinv (file:line cited on each function). Only tests, `__graft_entry__.smoke()` and `bench.py`'s CPU
baseline use it, and only as the checker or as the timed CPU baseline; the product never imports it.
Pinned against the reference by `tests/golden/*.npz` (made by `tests/golden/make_golden.py`).

Plans can be injected (Lambda, degrees, outer interval and degree) so that a device result and this oracle
evaluate the same fixed polynomial operator; only the apply arithmetic is then compared.
"""

import numpy as np

PAIRS = ((0, 1), (2, 3))  # quadrant packing pairs (fastops.py:176)


# ---------------------------------------------------------------- frequencies
def offset_freqs(L):
    """omega_k = 2 pi fftfreq(L)_k (fastops.py:185, fastspec.py:97)."""
    return 2 * np.pi * np.fft.fftfreq(L)


def offset_z(L):
    """z_k = exp(i omega_k) (fastops.py:186)."""
    return np.exp(1j * offset_freqs(L))


# ---------------------------------------------------------------- butterflies
def bfly_levels(n, z, X, m_lo=1, m_hi=None):
    """Forward butterflies B_{m_hi} ... B_{m_lo}, one frequency z[k] per row (fasthybrid.py:23-37,
    fastspec.py:21-35 for the full range, fastops.py:71-83 for the operation order, cpp/oblique.cpp:22-33).

    Level m, w = 2^(m-1), strip l, t < w: with u = z^t f1[t]:
        out[l*2w + 2t] = f0[t] + u,   out[l*2w + 2t + 1] = f0[t] + z u.
    """
    m_hi = n if m_hi is None else m_hi
    g = np.array(X, dtype=complex)
    K, N = g.shape
    z = np.asarray(z, dtype=complex).reshape(K)
    for m in range(m_lo, m_hi + 1):
        w = 1 << (m - 1)
        ns = N // (2 * w)
        src = g.reshape(K, ns, 2, w)
        u = src[:, :, 1, :] * (z[:, None] ** np.arange(w)[None, :])[:, None, :]
        out = np.empty((K, ns, w, 2), dtype=complex)
        out[..., 0] = src[:, :, 0, :] + u
        out[..., 1] = src[:, :, 0, :] + u * z[:, None, None]
        g = out.reshape(K, N)
    return g


def bflyT_levels(n, z, G, m_lo=1, m_hi=None):
    """Adjoint butterflies B_{m_lo}^* ... B_{m_hi}^* (fasthybrid.py:40-54, fastspec.py:38-52,
    fastops.py:85-98 for the operation order, cpp/oblique.cpp:36-51).

    Level m: out0[t] = g[2t] + g[2t+1],  out1[t] = conj(z^t) (g[2t] + conj(z) g[2t+1]).
    """
    m_hi = n if m_hi is None else m_hi
    f = np.array(G, dtype=complex)
    K, N = f.shape
    z = np.asarray(z, dtype=complex).reshape(K)
    for m in range(m_hi, m_lo - 1, -1):
        w = 1 << (m - 1)
        ns = N // (2 * w)
        src = f.reshape(K, ns, w, 2)
        out = np.empty((K, ns, 2, w), dtype=complex)
        out[:, :, 0, :] = src[..., 0] + src[..., 1]
        twc = np.conj(z[:, None] ** np.arange(w)[None, :])
        out[:, :, 1, :] = (src[..., 0] + src[..., 1] * np.conj(z)[:, None, None]) * twc[:, None, :]
        f = out.reshape(K, N)
    return f


def bfly(n, z, X):
    """A_omega X over all levels (fastspec.py:21)."""
    return bfly_levels(n, z, X, 1, n)


def bflyT(n, z, G):
    """A_omega^* G over all levels (fastspec.py:38)."""
    return bflyT_levels(n, z, G, 1, n)


# ---------------------------------------------------------------- inner Chebyshev filter
def cheb_coeffs(lam_max, tau):
    """Semi-iteration constants on [tau, lam_max + tau]: c = (hi-lo)/(hi+lo), a = 2/(hi+lo) (fastspec.py:56-59)."""
    lo, hi = tau, np.asarray(lam_max, dtype=float) + tau
    return (hi - lo) / (hi + lo), 2.0 / (hi + lo)


def cheb_omegas(c, d):
    """omega_j, j = 1..d-1, of the semi-iteration for one row: omega_1 = 1/(1 - c^2/2),
    omega_j = 1/(1 - c^2 omega_{j-1}/4) (fastspec.py:78, cpp/oblique.cpp:88)."""
    om, out = 1.0, []
    for j in range(1, int(d)):
        om = 1.0 / (1.0 - c * c / 2.0) if j == 1 else 1.0 / (1.0 - c * c * om / 4.0)
        out.append(om)
    return out


def poly_apply_levels(n, z, Y, lam_max, tau, deg, m_lo=1, m_hi=None, count=None):
    """Z_k = p_k(M_k) Y_k with M_k = B^* B over levels m_lo..m_hi and p_k the degree-deg[k] Chebyshev
    semi-iteration polynomial for (M + tau)^{-1} on [0, lam_max[k]] (fasthybrid.py:57-77, fastspec.py:62-86,
    fastops.py:118-138, cpp/oblique.cpp:74-104). Rows are advanced only while deg[k] > j."""
    m_hi = n if m_hi is None else m_hi
    Y = np.asarray(Y, dtype=complex)
    K = Y.shape[0]
    deg = np.asarray(deg, dtype=int).reshape(K)
    c, a = cheb_coeffs(np.asarray(lam_max, dtype=float).reshape(K), tau)
    z = np.asarray(z, dtype=complex).reshape(K)
    Z = a[:, None] * Y
    Zprev = np.zeros_like(Y)
    om = np.ones(K)
    for j in range(1, int(deg.max()) if K else 0):
        act = np.nonzero(deg > j)[0]
        if act.size == 0:
            break
        omj = 1.0 / (1.0 - c[act] ** 2 / 2.0) if j == 1 else 1.0 / (1.0 - c[act] ** 2 * om[act] / 4.0)
        Za = Z[act]
        R = Y[act] - bflyT_levels(n, z[act], bfly_levels(n, z[act], Za, m_lo, m_hi), m_lo, m_hi) - tau * Za
        Znew = Za + omj[:, None] * (a[act][:, None] * R) + (omj - 1.0)[:, None] * (Za - Zprev[act])
        Zprev[act] = Za
        Z[act] = Znew
        om[act] = omj
        if count is not None:
            count[0] += act.size * 2 * (m_hi - m_lo + 1)
    return Z


# ---------------------------------------------------------------- level-1 stencils (hybrid)
def K_rows(x):
    """Tridiagonal (1, 2, 1) along axis 0 (fasthybrid.py:81-85)."""
    y = 2.0 * x
    y[1:] += x[:-1]
    y[:-1] += x[1:]
    return y


def J_cols(x):
    """Swap of column pairs (2j, 2j+1) (fasthybrid.py:88-92)."""
    y = np.empty_like(x)
    y[:, 0::2] = x[:, 1::2]
    y[:, 1::2] = x[:, 0::2]
    return y


def G1_apply(x):
    """G_1 x = 8x + J(K x) + (J(K x^T))^T (fasthybrid.py:95-98)."""
    return 8.0 * x + J_cols(K_rows(x)) + J_cols(K_rows(x.T)).T


def Pi_apply(x):
    """2x2-cell averaging projector (fasthybrid.py:101-105)."""
    N = x.shape[0]
    c = x.reshape(N // 2, 2, N // 2, 2).mean(axis=(1, 3))
    return np.repeat(np.repeat(c, 2, axis=0), 2, axis=1)


def lorr_inv(y):
    """(4I + 8 Pi)^{-1} y = (y - Pi y)/4 + Pi y / 12 (fasthybrid.py:108-111)."""
    p = Pi_apply(y)
    return (y - p) / 4.0 + p / 12.0


def lorr_fwd(y):
    """4 y + 8 Pi y, the inverse of lorr_inv (fasthybrid.py:235, fastops.py:318)."""
    return 4.0 * y + 8.0 * Pi_apply(y)


def cheb_solve(op, y, lo, hi, deg):
    """Fixed-degree Chebyshev semi-iteration for op^{-1} y with spec(op) in [lo, hi] (fasthybrid.py:114-126)."""
    c = (hi - lo) / (hi + lo)
    a = 2.0 / (hi + lo)
    x_prev = np.zeros_like(y)
    x = a * y
    om = 1.0
    for k in range(1, deg):
        om = 1.0 / (1.0 - c * c / 2.0) if k == 1 else 1.0 / (1.0 - c * c * om / 4.0)
        r = y - op(x)
        x_new = x + om * (a * r) + (om - 1.0) * (x - x_prev)
        x_prev, x = x, x_new
    return x


def g1_inv(y, deg=14):
    """P = degree-`deg` Chebyshev approximation of G_1^{-1} on [4, 16] (fasthybrid.py:129-130)."""
    return cheb_solve(G1_apply, y, 4.0, 16.0, deg)


# ---------------------------------------------------------------- spectral bounds
def cert_rowsum_levels(n, om, m_lo=2):
    """Certified bound on the max row sum of |M_omega| for levels m_lo..n (fasthybrid.py:134-150,
    cpp/oblique.cpp:106-130): r_m(a) = |1+z^a| r(2a) + max(|1+z^(a+1)| r(2a+1), |1+z^(a-1)| r(2a-1)),
    |a| <= 2^(n-m) - 1, with r = 1 below level m_lo; the bound is r_n(0)."""
    z = np.exp(1j * om)
    A = 1 << n
    r = np.ones(2 * A + 1)
    for m in range(m_lo, n + 1):
        amax = (1 << (n - m)) - 1
        a = np.arange(-amax, amax + 1)
        t0 = np.abs(1 + z**a) * r[2 * a + A]
        tp = np.abs(1 + z ** (a + 1)) * r[2 * a + 1 + A]
        tm = np.abs(1 + z ** (a - 1)) * r[2 * a - 1 + A]
        rn = np.zeros(2 * A + 1)
        rn[a + A] = t0 + np.maximum(tp, tm)
        r = rn
    return r[A]


def explicit_lam_max(n, oms):
    """Lambda_k = min(N^2, 2N(1+n)/|omega_k|), N^2 at omega = 0 (fastcpp.py:128-134, fastspec.py:100-104)."""
    N = 1 << n
    w = np.abs(np.asarray(oms, dtype=float))
    lam = np.full(len(w), float(N) ** 2)
    nz = w > 0
    lam[nz] = np.minimum(float(N) ** 2, 2.0 * N * (1 + n) / w[nz])
    return lam


def power_lam_max(n, z, m_lo, iters=40, safety=1.5, seeds=(0, 1)):
    """safety x Rayleigh quotient of M_k = B^* B (levels m_lo..n) after `iters` normalised power steps.

    seeds=(0, 1): start vectors as fastcpp.power_lam_max (fastcpp.py:102-118, real part from
    default_rng(0), imaginary part from default_rng(1)); seeds=(0,): both parts from one default_rng(0)
    stream as fastops.FastLp/FastHybrid (fastops.py:266-272, 309-316)."""
    N = 1 << n
    K = len(z)
    if len(seeds) == 2:
        V = np.random.default_rng(seeds[0]).standard_normal((K, N)) + 1j * np.random.default_rng(
            seeds[1]
        ).standard_normal((K, N))
    else:
        rng = np.random.default_rng(seeds[0])
        V = rng.standard_normal((K, N)) + 1j * rng.standard_normal((K, N))

    def M(V):
        return bflyT_levels(n, z, bfly_levels(n, z, V, m_lo, n), m_lo, n)

    for _ in range(iters):
        V = M(V)
        V /= np.linalg.norm(V, axis=1, keepdims=True)
    return safety * np.real(np.sum(np.conj(V) * M(V), axis=1))


def sym_lam(lam):
    """Lambda_k <- max(Lambda_k, Lambda_{-k}) so that p_{-k} = conj(p_k) (fastops.py:170-172)."""
    L = len(lam)
    return np.maximum(lam, lam[(-np.arange(L)) % L])


def inner_degrees(lam, tau, eps_in):
    """d_k = max(2, ceil(log(eps/2) / log((sqrt(kappa)-1)/(sqrt(kappa)+1)))), kappa = 1 + Lambda/tau
    (fastops.py:190-192, fastspec.py:115-117, fasthybrid.py:188-190)."""
    kap = 1.0 + lam / tau
    rate = (np.sqrt(kap) - 1) / (np.sqrt(kap) + 1)
    return np.maximum(2, np.ceil(np.log(eps_in / 2.0) / np.log(np.maximum(rate, 1e-12)))).astype(int)


def outer_degree(lo, hi, eps):
    """D = ceil(log(eps/2)/log((sqrt(k)-1)/(sqrt(k)+1))) + 2 with k = hi/lo (fastops.py:244-245)."""
    kap = hi / lo
    return int(np.ceil(np.log(eps / 2.0) / np.log((np.sqrt(kap) - 1) / (np.sqrt(kap) + 1)))) + 2


def dense_tikhonov(n, zk, tau, m_lo, m_hi):
    """Exact filter F = (M + tau)^{-1} = V diag(1/(lambda+tau)) V^* for one frequency (fastops.py:31-39)."""
    N = 1 << n
    A = bfly_levels(n, np.full(N, zk), np.eye(N, dtype=complex), m_lo, m_hi).T
    lam, V = np.linalg.eigh(A.conj().T @ A)
    lam = np.maximum(lam, 0)
    return (V / (lam + tau)) @ V.conj().T


# ---------------------------------------------------------------- quadrant strips
def Tq(n, q, X):
    """Torus quadrant strip of an L x L image: L x N (fastspec.py:142-152)."""
    N, L = 1 << n, 2 << n
    r = (N - 1 - np.arange(L)) % L
    if q == 2:
        return X[:, :N]
    if q == 1:
        return X[r][:, :N]
    if q == 0:
        return X.T[r][:, :N]
    if q == 3:
        return X[r][:, r].T[:, :N]
    raise ValueError(q)


def TqT(n, q, S):
    """Adjoint of Tq: L x N strip -> L x L image (fastspec.py:154-168)."""
    N, L = 1 << n, 2 << n
    r = (N - 1 - np.arange(L)) % L
    X = np.zeros((L, L), dtype=S.dtype)
    X[:, :N] = S
    if q == 2:
        return X
    if q == 1:
        return X[r]
    if q == 0:
        return X[r].T
    if q == 3:
        return X.T[:, r][r]
    raise ValueError(q)


def iota(n, bq):
    """Embed sinogram rows h in [-(N-1), N-1] at cyclic row h mod L (fastspec.py:170-174)."""
    N, L = 1 << n, 2 << n
    S = np.zeros((L, N))
    S[np.arange(-(N - 1), N) % L] = bq
    return S


# ---------------------------------------------------------------- row engine (FP64)
class RowEngineOracle:
    """Row-batched operator engine over R = copies * L frequency rows (fastops.py:20-167 semantics,
    single chunk). ops are ('B'|'BT'|'P', m_lo, m_hi) applied left to right; rows whose degree exceeds
    dense_cap use the dense Tikhonov filter in 'P' (fastops.py:28-40, 100-117)."""

    def __init__(self, n, z, deg, lam_max, tau, copies=2, dense_cap=None, p_levels=(1, None)):
        self.n, self.N, self.tau = n, 1 << n, tau
        self.L = len(z)
        self.copies = copies
        self.z = np.tile(np.asarray(z, dtype=complex), copies)
        self.deg = np.tile(np.asarray(deg, dtype=int), copies)
        self.lam = np.tile(np.asarray(lam_max, dtype=float), copies)
        lo, hi = p_levels[0], p_levels[1] or n
        self.dense = {}
        if dense_cap is not None:
            for k in np.nonzero(np.asarray(deg) > dense_cap)[0]:
                self.dense[int(k)] = dense_tikhonov(n, z[k], tau, lo, hi)
        self.n_dense = len(self.dense)
        self.count = [0]

    def _P(self, Y, lo, hi):
        Z = np.empty_like(Y)
        rows = np.arange(Y.shape[0])
        dmask = np.array([(int(r) % self.L) in self.dense for r in rows], dtype=bool)
        for r in rows[dmask]:
            Z[r] = self.dense[int(r) % self.L] @ Y[r]
        pr = rows[~dmask]
        if pr.size:
            Z[pr] = poly_apply_levels(self.n, self.z[pr], Y[pr], self.lam[pr], self.tau, self.deg[pr], lo, hi, self.count)
        self.count[0] += int(dmask.sum()) * self.N // max(1, self.n)
        return Z

    def run(self, Y, ops):
        X = np.array(Y, dtype=complex)
        K = X.shape[0]
        for op, lo, hi in ops:
            if op == "B":
                X = bfly_levels(self.n, self.z, X, lo, hi)
                self.count[0] += K * (hi - lo + 1)
            elif op == "BT":
                X = bflyT_levels(self.n, self.z, X, lo, hi)
                self.count[0] += K * (hi - lo + 1)
            elif op == "P":
                X = self._P(X, lo, hi)
            else:
                raise ValueError(op)
        return X


def packed(n, eng, strips_fn, ops):
    """Quadrant pairs as a + i b, FFT along axis 0, row ops, iFFT, Re -> qa, Im -> qb, sum, crop
    (fastops.py:209-220)."""
    N, L = 1 << n, 2 << n
    Y = np.empty((2 * L, N), dtype=complex)
    for i, (qa, qb) in enumerate(PAIRS):
        Y[i * L : (i + 1) * L] = np.fft.fft(strips_fn(qa) + 1j * strips_fn(qb), axis=0)
    Z = eng.run(Y, ops)
    out = np.zeros((L, L))
    for i, (qa, qb) in enumerate(PAIRS):
        W = np.fft.ifft(Z[i * L : (i + 1) * L], axis=0)
        out += TqT(n, qa, W.real) + TqT(n, qb, W.imag)
    return out[:N, :N]


def outer_cheb(y, Gop, lo, hi, D, P=lambda v: v):
    """Fixed-degree outer Chebyshev on P G (fastops.py:247-258)."""
    c = (hi - lo) / (hi + lo)
    a = 2.0 / (hi + lo)
    x_prev = np.zeros_like(y)
    x = a * P(y)
    om = 1.0
    for k in range(1, D):
        om = 1.0 / (1.0 - c * c / 2.0) if k == 1 else 1.0 / (1.0 - c * c * om / 4.0)
        r = P(y - Gop(x))
        x_new = x + om * (a * r) + (om - 1.0) * (x - x_prev)
        x_prev, x = x, x_new
    return x


def outer_interval(N, Gop, Pinv=None, P=None, eps=1e-10, maxiter=300, margins=(0.99, 1.01)):
    """[lo, hi] of P G by Lanczos (eigsh, tol 1e-3) + residual enclosure and 0.99/1.01 margins, and the outer
    degree (fastops.py:222-245; fastspec.py:119-138 uses maxiter 200 and no margins)."""
    import scipy.sparse.linalg as spla

    A = spla.LinearOperator((N * N, N * N), matvec=lambda v: Gop(v.reshape(N, N)).ravel(), dtype=float)
    if Pinv is None:
        lo, ulo = spla.eigsh(A, k=1, which="SA", tol=1e-3, maxiter=maxiter)
        hi, uhi = spla.eigsh(A, k=1, which="LA", tol=1e-3, maxiter=maxiter)

        def res(th, u):
            return np.linalg.norm(A.matvec(u[:, 0]) - th * u[:, 0])

    else:
        Mop = spla.LinearOperator((N * N, N * N), matvec=lambda v: Pinv(v.reshape(N, N)).ravel(), dtype=float)
        Minv = spla.LinearOperator((N * N, N * N), matvec=lambda v: P(v.reshape(N, N)).ravel(), dtype=float)
        lo, ulo = spla.eigsh(A, k=1, M=Mop, Minv=Minv, which="SA", tol=1e-3, maxiter=maxiter)
        hi, uhi = spla.eigsh(A, k=1, M=Mop, Minv=Minv, which="LA", tol=1e-3, maxiter=maxiter)

        def res(th, u):
            u = u[:, 0]
            r = A.matvec(u) - th * Mop.matvec(u)
            return np.sqrt(abs(r @ Minv.matvec(r))) / np.sqrt(abs(u @ Mop.matvec(u)))

    lo, hi = float(lo[0]), float(hi[0])
    lo_b, hi_b = (lo - res(lo, ulo)) * margins[0], (hi + res(hi, uhi)) * margins[1]
    return lo_b, hi_b, outer_degree(lo_b, hi_b, eps)


# ---------------------------------------------------------------- the two packed inverses (fastops)
class _PackedBase:
    """Shared setup of FastLp / FastHybrid (fastops.py:175-258) with plan injection:
    lam_max (Lambda before symmetrisation), deg (overrides the computed degrees), deg_cap (d_k <- min(p, d_k)),
    outer=(lo, hi, D) (skips the Lanczos setup)."""

    p_levels = (1, None)

    def _setup(self, n, tau_fac, eps_in, eps, lam_max, deg, deg_cap, dense_cap, outer):
        self.n = n
        self.N = N = 1 << n
        self.L = 2 * N
        self.tau = tau_fac * N
        self.oms = offset_freqs(self.L)
        self.z = offset_z(self.L)
        self.lam_max = np.maximum(sym_lam(np.asarray(lam_max, dtype=float)), 1.0)
        d = inner_degrees(self.lam_max, self.tau, eps_in) if deg is None else np.asarray(deg, dtype=int)
        if deg_cap is not None:
            d = np.minimum(d, int(deg_cap))
        self.deg = d
        self.eng = RowEngineOracle(n, self.z, self.deg, self.lam_max, self.tau, 2, dense_cap, self.p_levels)
        self.eps = eps
        self._outer_plan = outer

    def _finish(self, Pinv=None, P=None):
        if self._outer_plan is None:
            self.lo, self.hi, self.outer_deg = outer_interval(self.N, self._G, Pinv, P, self.eps)
        else:
            self.lo, self.hi, self.outer_deg = float(self._outer_plan[0]), float(self._outer_plan[1]), int(self._outer_plan[2])
        self.eng.count = [0]

    def _embed(self, x):
        X = np.zeros((self.L, self.L))
        X[: self.N, : self.N] = x
        return X


class LpOracle(_PackedBase):
    """fastops.FastLp (fastops.py:261-288)."""

    p_levels = (1, None)

    def __init__(self, n, tau_fac=0.2, eps_in=0.1, eps=1e-10, lam_max=None, deg=None, deg_cap=None,
                 dense_cap=None, outer=None, power_iters=40, safety=1.5):
        if lam_max is None:
            lam_max = power_lam_max(n, offset_z(2 << n), 1, power_iters, safety, seeds=(0,))
        self._setup(n, tau_fac, eps_in, eps, lam_max, deg, deg_cap, dense_cap, outer)
        self._G = self.frame_window
        self._finish()

    def frame_window(self, x):
        n = self.n
        X = self._embed(x)
        return packed(n, self.eng, lambda q: Tq(n, q, X), [("P", 1, n), ("B", 1, n), ("BT", 1, n)])

    def backproject(self, b):
        n = self.n
        return packed(n, self.eng, lambda q: iota(n, b[q]), [("BT", 1, n), ("P", 1, n)])

    def apply(self, b):
        return outer_cheb(self.backproject(b), self.frame_window, self.lo, self.hi, self.outer_deg)


class HybridOracle(_PackedBase):
    """fastops.FastHybrid (fastops.py:291-338)."""

    p_levels = (2, None)

    def __init__(self, n, tau_fac=0.2, eps_in=0.1, eps=1e-10, lam_max=None, deg=None, deg_cap=None,
                 dense_cap=None, outer=None, g1_deg=14, precond="g1", power_iters=40, safety=1.5):
        if lam_max is None:
            lam_max = power_lam_max(n, offset_z(2 << n), 2, power_iters, safety, seeds=(0,))
        self.g1_deg = g1_deg
        self.precond = precond
        self._setup(n, tau_fac, eps_in, eps, lam_max, deg, deg_cap, dense_cap, outer)
        self._G = self.Gh
        Pinv = G1_apply if precond == "g1" else lorr_fwd
        self._finish(Pinv, self.P)

    def P(self, y):
        return g1_inv(y, self.g1_deg) if self.precond == "g1" else lorr_inv(y)

    def Gh(self, x):
        n = self.n
        X = self._embed(x)
        ops = [("B", 1, 1), ("P", 2, n), ("B", 2, n), ("BT", 2, n), ("BT", 1, 1)]
        return packed(n, self.eng, lambda q: Tq(n, q, X), ops)

    def backproject(self, b):
        n = self.n
        return packed(n, self.eng, lambda q: iota(n, b[q]), [("BT", 2, n), ("P", 2, n), ("BT", 1, 1)])

    def apply(self, b):
        return outer_cheb(self.backproject(b), self.Gh, self.lo, self.hi, self.outer_deg, self.P)


# ---------------------------------------------------------------- unpacked NumPy references (fastspec / fasthybrid)
class SpectralOracle:
    """fastspec.FastSpectralInverse (fastspec.py:90-215): four quadrant passes, unsymmetrised Lambda, inner
    degrees from the same eps as the outer iteration. Plan injection as in _PackedBase."""

    def __init__(self, n, tau_fac=0.2, eps=1e-10, lam_max=None, deg=None, outer=None, power_iters=40, safety=1.5):
        self.n = n
        N = self.N = 1 << n
        self.L = 2 * N
        self.tau = tau_fac * N
        self.oms = offset_freqs(self.L)
        self.z = np.exp(1j * self.oms)
        if lam_max is None:
            lam_max = np.maximum(power_lam_max(n, self.z, 1, power_iters, safety, seeds=(0,)), 1.0)
        self.lam_max = np.asarray(lam_max, dtype=float)
        self.deg = inner_degrees(self.lam_max, self.tau, eps) if deg is None else np.asarray(deg, dtype=int)
        self.count = [0]
        if outer is None:
            outer = outer_interval(N, self.frame_window, None, None, eps, maxiter=200, margins=(1.0, 1.0))
        self.lo, self.hi, self.outer_deg = float(outer[0]), float(outer[1]), int(outer[2])
        self.count = [0]

    def frame_window(self, x):
        n, N, L = self.n, self.N, self.L
        X = np.zeros((L, L))
        X[:N, :N] = x
        out = np.zeros((L, L))
        for q in range(4):
            Sf = np.fft.fft(Tq(n, q, X), axis=0)
            Pf = poly_apply_levels(n, self.z, Sf, self.lam_max, self.tau, self.deg, 1, n, self.count)
            Mf = bflyT(n, self.z, bfly(n, self.z, Pf))
            self.count[0] += L
            out += TqT(n, q, np.real(np.fft.ifft(Mf, axis=0)))
        return out[:N, :N]

    def backproject(self, b):
        n, N, L = self.n, self.N, self.L
        out = np.zeros((L, L))
        for q in range(4):
            Yf = bflyT(n, self.z, np.fft.fft(iota(n, b[q]), axis=0))
            self.count[0] += L
            Pf = poly_apply_levels(n, self.z, Yf, self.lam_max, self.tau, self.deg, 1, n, self.count)
            out += TqT(n, q, np.real(np.fft.ifft(Pf, axis=0)))
        return out[:N, :N]

    def apply(self, b):
        return outer_cheb(self.backproject(b), self.frame_window, self.lo, self.hi, self.outer_deg)


class HybridSpectralOracle:
    """fasthybrid.FastHybridInverse (fasthybrid.py:153-309): four quadrant passes, unsymmetrised Lambda,
    inner degrees from eps. Plan injection: lam_max, deg, outer=(lo, hi, D)."""

    def __init__(self, n, tau_fac=0.2, eps=1e-10, lam_max=None, deg=None, outer=None, precond="g1", g1_deg=14):
        self.n = n
        N = self.N = 1 << n
        self.L = 2 * N
        self.tau = tau_fac * N
        self.precond = precond
        self.g1_deg = g1_deg
        self.oms = offset_freqs(self.L)
        self.z = np.exp(1j * self.oms)
        if lam_max is None:
            lam_max = power_lam_max(n, self.z, 2, 40, 1.5, seeds=(0,))
        self.lam_max = np.maximum(np.asarray(lam_max, dtype=float), 1.0)
        self.deg = inner_degrees(self.lam_max, self.tau, eps) if deg is None else np.asarray(deg, dtype=int)
        self.count = [0]
        if outer is None:
            Pinv = {"g1": G1_apply, "lorr": lorr_fwd}.get(precond)
            outer = outer_interval(N, self.Gh, Pinv, self.P if Pinv else None, eps, maxiter=300)
        self.lo, self.hi, self.outer_deg = float(outer[0]), float(outer[1]), int(outer[2])
        self.count = [0]

    def P(self, y):
        if self.precond == "g1":
            return g1_inv(y, self.g1_deg)
        if self.precond == "lorr":
            return lorr_inv(y)
        return y

    def Gh(self, x):
        n, N, L, z, c = self.n, self.N, self.L, self.z, self.count
        X = np.zeros((L, L))
        X[:N, :N] = x
        out = np.zeros((L, L))
        for q in range(4):
            Sf = bfly_levels(n, z, np.fft.fft(Tq(n, q, X), axis=0), 1, 1)
            c[0] += L
            Pf = poly_apply_levels(n, z, Sf, self.lam_max, self.tau, self.deg, 2, n, c)
            Mf = bflyT_levels(n, z, bfly_levels(n, z, Pf, 2, n), 2, n)
            c[0] += 2 * L * (n - 1)
            out += TqT(n, q, np.real(np.fft.ifft(bflyT_levels(n, z, Mf, 1, 1), axis=0)))
            c[0] += L
        return out[:N, :N]

    def backproject(self, b):
        n, N, L, z, c = self.n, self.N, self.L, self.z, self.count
        out = np.zeros((L, L))
        for q in range(4):
            Yf = bflyT_levels(n, z, np.fft.fft(iota(n, b[q]), axis=0), 2, n)
            c[0] += L * (n - 1)
            Pf = poly_apply_levels(n, z, Yf, self.lam_max, self.tau, self.deg, 2, n, c)
            out += TqT(n, q, np.real(np.fft.ifft(bflyT_levels(n, z, Pf, 1, 1), axis=0)))
            c[0] += L
        return out[:N, :N]

    def apply(self, b):
        return outer_cheb(self.backproject(b), self.Gh, self.lo, self.hi, self.outer_deg, self.P)
