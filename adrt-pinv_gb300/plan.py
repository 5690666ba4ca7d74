"""Plan of an explicit oblique inverse: everything that is fixed before any data arrives (FP64, host).

Mirrors the setup of the reference's packed inverses (fastops.py:179-203): offset frequencies, symmetrised
spectral bounds Lambda_k, inner degrees d_k, Chebyshev constants, the dense low-frequency rows, and the outer
interval [lo, hi] with its degree D. Two additions, both optional:
  * deg_cap (the "p" of a degree-p filter): d_k <- min(p, d_k). The cap keeps k <-> -k symmetry, so quadrant
    packing stays valid; p >= max d_k reproduces the reference's degrees.
  * plan caching: `save(path)` / `Plan.load(path)` round-trip every array through an .npz file.
The device tables derived here (roots of unity, per-frequency coefficient rows, row order) are built in FP64 and
rounded once to the compute precision.
"""

import numpy as np

METHODS = ("lp", "hybrid")


def offset_freqs(L):
    """omega_k = 2 pi fftfreq(L)_k (fastops.py:185)."""
    return 2 * np.pi * np.fft.fftfreq(L)


def roots_of_unity(L):
    """exp(2 pi i j / L), j < L, to FP64 accuracy; z_k = root[k] and z_k^t = root[(k t) mod L]."""
    j = np.arange(L)
    return np.cos(2 * np.pi * j / L) + 1j * np.sin(2 * np.pi * j / L)


def sym_lam(lam):
    """max(Lambda_k, Lambda_{-k}) (fastops.py:170-172)."""
    L = len(lam)
    return np.maximum(lam, lam[(-np.arange(L)) % L])


def inner_degrees(lam, tau, eps_in):
    """d_k = max(2, ceil(log(eps/2)/log((sqrt k - 1)/(sqrt k + 1)))), k = 1 + Lambda/tau (fastops.py:190-192)."""
    kap = 1.0 + lam / tau
    rate = (np.sqrt(kap) - 1) / (np.sqrt(kap) + 1)
    return np.maximum(2, np.ceil(np.log(eps_in / 2.0) / np.log(np.maximum(rate, 1e-12)))).astype(int)


def cheb_coeffs(lam, tau):
    """c = Lambda/(Lambda + 2 tau), a = 2/(Lambda + 2 tau) (fastspec.py:56-59)."""
    lo, hi = tau, np.asarray(lam, dtype=float) + tau
    return (hi - lo) / (hi + lo), 2.0 / (hi + lo)


def coef_table(lam, tau, deg):
    """Per frequency: a_k, then (omega_j, omega_j a_k, omega_j - 1) for j = 1..d_k-1, with the semi-iteration
    recurrence omega_1 = 1/(1 - c^2/2), omega_j = 1/(1 - c^2 omega_{j-1}/4) (fastspec.py:78, cpp/oblique.cpp:88)."""
    c, a = cheb_coeffs(lam, tau)
    dmax = max(int(np.max(deg)), 1)
    stride = 1 + 3 * (dmax - 1)
    tab = np.zeros((len(lam), stride))
    tab[:, 0] = a
    om = np.ones(len(lam))
    for j in range(1, dmax):
        om = np.where(j == 1, 1.0 / (1.0 - c * c / 2.0), 1.0 / (1.0 - c * c * om / 4.0))
        tab[:, 3 * j - 2] = om
        tab[:, 3 * j - 1] = om * a
        tab[:, 3 * j] = om - 1.0
    return tab, stride


def outer_degree(lo, hi, eps):
    """D = ceil(log(eps/2)/log((sqrt k - 1)/(sqrt k + 1))) + 2, k = hi/lo (fastops.py:244-245)."""
    kap = hi / lo
    return int(np.ceil(np.log(eps / 2.0) / np.log((np.sqrt(kap) - 1) / (np.sqrt(kap) + 1)))) + 2


def outer_coeffs(lo, hi, D):
    """(a, c, [(omega_k a, omega_k - 1) for k = 1..D-1]) of the outer semi-iteration (fastops.py:247-258)."""
    c = (hi - lo) / (hi + lo)
    a = 2.0 / (hi + lo)
    steps, om = [], 1.0
    for k in range(1, D):
        om = 1.0 / (1.0 - c * c / 2.0) if k == 1 else 1.0 / (1.0 - c * c * om / 4.0)
        steps.append((om * a, om - 1.0))
    return a, c, steps


class Plan:
    """Data-independent plan of an L_p ('lp') or hybrid ('hybrid') inverse at N = 2^n.

    lam_max: Lambda_k before symmetrisation (length L = 2N); deg overrides the computed degrees; deg_cap caps them;
    dense_cap: rows with d_k > dense_cap use the exact Tikhonov filter (fastops.py:28-40); outer = (lo, hi, D)."""

    def __init__(self, method, n, lam_max, tau_fac=0.2, eps_in=0.1, eps=1e-10, deg=None, deg_cap=None, dense_cap=None,
                 precond="g1", g1_deg=14, outer=None, raw_lam=False, high_rows="dense"):
        if method not in METHODS:
            raise ValueError(f"method must be one of {METHODS}")
        if not (1 <= n <= 11):
            raise ValueError(f"n={n} out of range 1..11")
        if precond not in ("g1", "lorr", "none"):
            raise ValueError(f"precond {precond!r}")
        self.method, self.n = method, n
        self.N = N = 1 << n
        self.L = L = 2 * N
        self.tau_fac, self.eps_in, self.eps = tau_fac, eps_in, eps
        self.tau = tau_fac * N
        self.precond, self.g1_deg = precond, int(g1_deg)
        self.p_levels = (1, n) if method == "lp" else (2, n)
        lam_max = np.asarray(lam_max, dtype=float)
        if lam_max.shape != (L,):
            raise ValueError(f"lam_max must have length L = {L}")
        # raw_lam: use Lambda as given (fastops.RowEngine receives it already symmetrised, fastops.py:189, 193)
        self.lam_max = lam_max.copy() if raw_lam else np.maximum(sym_lam(lam_max), 1.0)
        d = inner_degrees(self.lam_max, self.tau, eps_in) if deg is None else np.asarray(deg, dtype=int).copy()
        if deg_cap is not None:
            d = np.minimum(d, int(deg_cap))
        if d.shape != (L,) or d.min() < 1:
            raise ValueError("deg must be L positive integers")
        self.deg = d
        self.deg_cap, self.dense_cap = deg_cap, dense_cap
        self.dense_freqs = np.nonzero(d > dense_cap)[0].astype(np.int64) if dense_cap is not None else np.zeros(0, np.int64)
        # the rows with d_k > dense_cap: "dense" applies the reference's exact dense filter (fastops.py:28-40, the
        # operators held on the device), "ff" keeps the polynomial filter and runs those rows' op lists in
        # float-float arithmetic (compensated rows: no operator memory, more arithmetic)
        if high_rows not in ("dense", "ff"):
            raise ValueError("high_rows must be 'dense' or 'ff'")
        self.high_rows = high_rows
        self.dense_tables = None
        self.coef, self.coef_stride = coef_table(self.lam_max, self.tau, self.deg)
        self.set_outer(outer)

    # ---------------------------------------------------------------- outer interval
    def set_outer(self, outer):
        if outer is None:
            self.lo = self.hi = None
            self.outer_deg = None
        else:
            self.lo, self.hi = float(outer[0]), float(outer[1])
            self.outer_deg = int(outer[2]) if len(outer) > 2 and outer[2] is not None else outer_degree(self.lo, self.hi, self.eps)

    # ---------------------------------------------------------------- row order and cost
    def packed_rows(self, dense=False):
        """Packed rows (copies stacked, R = 2L) sorted by descending degree (stable, fastops.py:42); with dense=False
        the dense-table rows are left out, with dense=True only they are returned."""
        dd = np.tile(self.deg, 2)
        order = np.argsort(-dd, kind="stable")
        isd = np.isin(order % self.L, self.dense_freqs)
        return order[isd] if dense else order[~isd]

    def level_rows(self, ops, dense_rows=None):
        """Level-row count of one packed op list, as the reference counts it (fastops.py:144-153, 117)."""
        R, n = 2 * self.L, self.n
        poly_high = getattr(self, "high_rows", "dense") == "ff"  # compensated rows keep the polynomial filter
        nd = 0 if poly_high else 2 * len(self.dense_freqs)
        tot = 0
        for op, lo, hi in ops:
            if op in ("B", "BT"):
                tot += R * (hi - lo + 1)
            elif op == "P":
                d = np.tile(self.deg, 2)
                keep = np.ones(R, bool) if poly_high else ~np.isin(np.arange(R) % self.L, self.dense_freqs)
                tot += int(np.sum(np.maximum(d[keep] - 1, 0))) * 2 * (hi - lo + 1)
                tot += nd * self.N // max(1, n)
        return tot

    # ---------------------------------------------------------------- dense low-frequency tables
    def build_dense_tables(self):
        """F_k = V diag(1/(lambda+tau)) V^* of M_k for each dense frequency (fastops.py:31-39), FP64, (Kd, N, N)."""
        if self.dense_tables is not None or not len(self.dense_freqs):
            return self.dense_tables
        n, N = self.n, self.N
        lo, hi = self.p_levels
        z = roots_of_unity(self.L)
        out = np.empty((len(self.dense_freqs), N, N), dtype=complex)
        self._dense_eig = []
        for i, k in enumerate(self.dense_freqs):
            A = _butterfly_matrix(n, z[k], lo, hi)
            lam, V = np.linalg.eigh(A.conj().T @ A)
            lam = np.maximum(lam, 0)
            out[i] = (V / (lam + self.tau)) @ V.conj().T
            self._dense_eig.append((A, lam, V))
        self.dense_tables = out
        return out

    def dense_row_operator(self, fold_pre_adjoint, fold_post_gram, pre_b1, post_b1t):
        """dense_operator with the level-1 butterfly of the hybrid folded in as well: right-multiplied by B_1 when the
        op list applies B(1,1) before the filter, left-multiplied by B_1^* when it applies BT(1,1) after it
        (fastops.py:330, 335), so that each dense row of an op list is one matrix. (Kd, N, N) complex, FP64."""
        T = self.dense_operator(fold_pre_adjoint, fold_post_gram)
        if T is None or not (pre_b1 or post_b1t):
            return T
        z = roots_of_unity(self.L)[self.dense_freqs]
        out = T.copy()
        for i, zk in enumerate(z):
            B1 = _butterfly_matrix(self.n, zk, 1, 1)
            if pre_b1:
                out[i] = out[i] @ B1
            if post_b1t:
                out[i] = B1.conj().T @ out[i]
        return out

    def dense_operator(self, fold_pre_adjoint, fold_post_gram):
        """Per dense frequency, the exact operator that replaces the filter op of an op list together with the
        butterflies around it: F_k, F_k A_k^* (filter after the adjoint levels, as in the back-projections) or
        M_k F_k = V diag(lambda/(lambda+tau)) V^* (filter then M, as in G_h and the frame operator). In exact
        arithmetic these equal the reference's dense-row path (fastops.py:100-117) followed / preceded by the
        butterflies; evaluated once in FP64 they keep the ill-conditioned low-frequency rows accurate when the
        rest of the pipeline runs in FP32. (Kd, N, N) complex, FP64."""
        self.build_dense_tables()
        key = (bool(fold_pre_adjoint), bool(fold_post_gram))
        cache = self.__dict__.setdefault("_dense_ops", {})
        if key in cache:
            return cache[key]
        mats = []
        for (A, lam, V), F in zip(self._dense_eig, self.dense_tables):
            if key == (False, True):
                T = (V * (lam / (lam + self.tau))) @ V.conj().T
            elif key == (True, False):
                T = F @ A.conj().T
            elif key == (True, True):
                T = (V * (lam / (lam + self.tau))) @ V.conj().T @ A.conj().T
            else:
                T = F
            mats.append(T)
        cache[key] = np.array(mats) if mats else None
        return cache[key]

    def dense_row_operator_torch(self, fold_pre_adjoint, fold_post_gram, pre_b1, post_b1t, device, chunk=None):
        """dense_row_operator computed with torch on `device` (batched over chunks of dense frequencies), FP64,
        returned as a (Kd, N, N) complex128 tensor on that device. Instead of an eigendecomposition it uses the
        identities F = (M + tau I)^-1 (one Cholesky factorisation and inverse per frequency) and
        M F = I - tau F, exact in exact arithmetic and about five times cheaper; used for large N, where the host
        eigendecompositions dominate the setup."""
        import torch

        Kd = len(self.dense_freqs)
        if not Kd:
            return None
        out = torch.empty((Kd, self.N, self.N), dtype=torch.complex128, device=torch.device(device))
        for c0, T in self.dense_row_operator_chunks(fold_pre_adjoint, fold_post_gram, pre_b1, post_b1t, device, chunk):
            out[c0:c0 + T.shape[0]] = T
        return out

    def dense_row_operator_chunks(self, fold_pre_adjoint, fold_post_gram, pre_b1, post_b1t, device, chunk=None):
        """The chunks (first dense-frequency index, (k, N, N) complex128 tensor) of dense_row_operator_torch."""
        import torch

        n, N, Kd = self.n, self.N, len(self.dense_freqs)
        lo, hi = self.p_levels
        dev = torch.device(device)
        z = torch.from_numpy(roots_of_unity(self.L)[self.dense_freqs]).to(dev)
        if chunk is None:
            chunk = max(1, min(Kd, (1 << 30) // (N * N * 16)))  # about 1 GB per N x N batch
        eye = torch.eye(N, dtype=torch.complex128, device=dev)
        for c0 in range(0, Kd, chunk):
            zc = z[c0:c0 + chunk]
            A = _butterfly_matrix_torch(n, zc, lo, hi)
            F = A.mH @ A
            F.diagonal(dim1=-2, dim2=-1).add_(self.tau)
            F = torch.cholesky_inverse(torch.linalg.cholesky(F))
            T = eye - self.tau * F if fold_post_gram else F
            if fold_pre_adjoint:
                T = T @ A.mH
            del A, F
            if pre_b1 or post_b1t:
                B1 = _butterfly_matrix_torch(n, zc, 1, 1)
                if pre_b1:
                    T = T @ B1
                if post_b1t:
                    T = B1.mH @ T
            yield c0, T

    # ---------------------------------------------------------------- cache
    def save(self, path):
        np.savez(path, method=self.method, n=self.n, lam_max=self.lam_max, tau_fac=self.tau_fac, eps_in=self.eps_in,
                 eps=self.eps, deg=self.deg, deg_cap=-1 if self.deg_cap is None else self.deg_cap,
                 dense_cap=-1 if self.dense_cap is None else self.dense_cap, precond=self.precond, g1_deg=self.g1_deg,
                 outer=np.array([np.nan, np.nan, -1] if self.lo is None else [self.lo, self.hi, self.outer_deg]))

    @classmethod
    def load(cls, path):
        f = np.load(path, allow_pickle=False)
        outer = f["outer"]
        cap, dcap = int(f["deg_cap"]), int(f["dense_cap"])
        return cls(str(f["method"]), int(f["n"]), f["lam_max"], float(f["tau_fac"]), float(f["eps_in"]), float(f["eps"]),
                   deg=f["deg"], deg_cap=None if cap < 0 else cap, dense_cap=None if dcap < 0 else dcap,
                   precond=str(f["precond"]), g1_deg=int(f["g1_deg"]),
                   outer=None if np.isnan(outer[0]) else (outer[0], outer[1], int(outer[2])))


def _butterfly_matrix(n, zk, lo, hi):
    """Dense matrix of B_hi ... B_lo at one frequency (columns = images of the unit vectors), FP64 host."""
    N = 1 << n
    X = np.eye(N, dtype=complex)
    for m in range(lo, hi + 1):
        w = 1 << (m - 1)
        src = X.reshape(N, N // (2 * w), 2, w)
        u = src[:, :, 1, :] * (zk ** np.arange(w))[None, None, :]
        out = np.empty((N, N // (2 * w), w, 2), dtype=complex)
        out[..., 0] = src[:, :, 0, :] + u
        out[..., 1] = src[:, :, 0, :] + u * zk
        X = out.reshape(N, N)
    return X.T


def _butterfly_matrix_torch(n, zk, lo, hi):
    """_butterfly_matrix for a batch of frequencies zk (k,) with torch: (k, N, N) complex128 on zk's device."""
    import torch

    N = 1 << n
    k = zk.shape[0]
    X = torch.eye(N, dtype=torch.complex128, device=zk.device).expand(k, N, N).contiguous()
    for m in range(lo, hi + 1):
        w = 1 << (m - 1)
        src = X.reshape(k, N, N // (2 * w), 2, w)
        tw = zk[:, None] ** torch.arange(w, device=zk.device, dtype=torch.float64)[None, :]
        u = src[:, :, :, 1, :] * tw[:, None, None, :]
        out = torch.empty((k, N, N // (2 * w), w, 2), dtype=torch.complex128, device=zk.device)
        out[..., 0] = src[:, :, :, 0, :] + u
        out[..., 1] = src[:, :, :, 0, :] + u * zk[:, None, None, None]
        X = out.reshape(k, N, N)
    return X.transpose(-1, -2)
