"""Oracle (test infrastructure only): NumPy restatement of the reference's spatial ADRT.

Follows `adrtcore.py` of dsrim/adrt-pinv function by function (file:line cited on each). Nothing in the
product imports this module; only tests, `__graft_entry__.smoke()` and `bench.py`'s CPU baseline do, and only
as the checker. Parity of this restatement with the reference itself is pinned by `tests/golden/*.npz`
(generated by `tests/golden/make_golden.py`, which imports the reference).

Layout conventions (reference `adrtcore.py:9-20`): single-quadrant level-m data lives on
E^n_m = {(h, s): -(s mod 2^m) <= h < N} and is stored dense as an array of shape (N + 2^m - 1, N) whose row
index is h + 2^m - 1. The full sinogram is (4, 2N - 1, N): quadrant q, row h + N - 1, slope column s.
"""

import numpy as np


def T_apply(q, f):
    """Quadrant permutation T_q of an N x N image (adrtcore.py:29-39).

    q=0: (T f)(i,j) = f(j, N-1-i); q=1: f(N-1-i, j); q=2: identity; q=3: f(N-1-j, N-1-i).
    """
    f = np.asarray(f)
    if q == 0:
        # (i, j) -> f(j, N-1-i): reverse the columns, then transpose
        out = np.swapaxes(f[:, ::-1], 0, 1)
    elif q == 1:
        out = f[::-1, :]
    elif q == 2:
        out = f
    elif q == 3:
        out = np.swapaxes(f[::-1, ::-1], 0, 1)
    else:
        raise ValueError(q)
    return np.ascontiguousarray(out)


def T_apply_T(q, g):
    """Inverse (= transpose) of T_q (adrtcore.py:42-52)."""
    g = np.asarray(g)
    if q == 0:
        out = np.swapaxes(g, 0, 1)[:, ::-1]
    elif q == 1:
        out = g[::-1, :]
    elif q == 2:
        out = g
    elif q == 3:
        out = np.swapaxes(g, 0, 1)[::-1, ::-1]
    else:
        raise ValueError(q)
    return np.ascontiguousarray(out)


def level_shape(n, m):
    """Stored shape of level-m single-quadrant data (adrtcore.py:58-60)."""
    N = 1 << n
    return (N + (1 << m) - 1, N)


def _level_geometry(n, m):
    N = 1 << n
    w = 1 << (m - 1)
    return N, w, N + w - 1, N + 2 * w - 1, N // (2 * w)


def S_apply(n, m, f):
    """Level S_m: E^n_{m-1} -> E^n_m (adrtcore.py:63-83).

    For strip l (width 2w, w = 2^(m-1)), half c, position t < w and output parity b:
        g(h, l*2w + 2t + b) = f(h, l*2w + t) + f(h + t + b, l*2w + w + t),
    where each term is taken only where its input row lies inside E^n_{m-1} (h >= -t on that column).
    Row r of an array at level m stores offset h = r - (2^m - 1).
    """
    N, w, Hin, Hout, ns = _level_geometry(n, m)
    f = np.asarray(f)
    if f.shape != (Hin, N):
        raise ValueError(f"level {m} input must have shape {(Hin, N)}, got {f.shape}")
    src = f.reshape(Hin, ns, 2, w)
    dst = np.zeros((Hout, ns, w, 2), dtype=f.dtype)
    in0, out0 = w - 1, 2 * w - 1  # row of offset h = 0 at the input / output level
    for t in range(w):
        for b in (0, 1):
            # first term: input rows h in [-t, N) of the left half
            h_lo, h_hi = -t, N
            dst[out0 + h_lo : out0 + h_hi, :, t, b] += src[in0 + h_lo : in0 + h_hi, :, 0, t]
            # second term: input row h' = h + t + b must lie in [-t, N)
            h_lo, h_hi = -t - (t + b), N - (t + b)
            dst[out0 + h_lo : out0 + h_hi, :, t, b] += src[in0 + h_lo + t + b : in0 + h_hi + t + b, :, 1, t]
    return dst.reshape(Hout, N)


def S_apply_T(n, m, g):
    """Adjoint of S_m: scatter-add back to level m-1 (adrtcore.py:86-101)."""
    N, w, Hin, Hout, ns = _level_geometry(n, m)
    g = np.asarray(g)
    if g.shape != (Hout, N):
        raise ValueError(f"level {m} adjoint input must have shape {(Hout, N)}, got {g.shape}")
    src = g.reshape(Hout, ns, w, 2)
    dst = np.zeros((Hin, ns, 2, w), dtype=g.dtype)
    in0, out0 = w - 1, 2 * w - 1
    for t in range(w):
        for b in (0, 1):
            h_lo, h_hi = -t, N
            dst[in0 + h_lo : in0 + h_hi, :, 0, t] += src[out0 + h_lo : out0 + h_hi, :, t, b]
            h_lo, h_hi = -t - (t + b), N - (t + b)
            dst[in0 + h_lo + t + b : in0 + h_hi + t + b, :, 1, t] += src[out0 + h_lo : out0 + h_hi, :, t, b]
    return dst.reshape(Hin, N)


def sq_adrt(n, x, dtype=float):
    """Single-quadrant ADRT: levels 1..n on the image (adrtcore.py:104-109). dtype=float as in the reference;
    an integer dtype gives the exact integer transform (the levels only add)."""
    g = np.asarray(x, dtype=dtype)
    for m in range(1, n + 1):
        g = S_apply(n, m, g)
    return g


def sq_adrt_T(n, g, dtype=float):
    """Adjoint single-quadrant ADRT: levels n..1 (adrtcore.py:112-116)."""
    f = np.asarray(g, dtype=dtype)
    for m in range(n, 0, -1):
        f = S_apply_T(n, m, f)
    return f


def adrt(n, x, dtype=float):
    """Full ADRT R: N x N image -> (4, 2N-1, N) sinogram (adrtcore.py:122-128)."""
    N = 1 << n
    x = np.asarray(x, dtype=dtype).reshape(N, N)
    out = np.empty((4, 2 * N - 1, N), dtype=dtype)
    for q in range(4):
        out[q] = sq_adrt(n, T_apply(q, x), dtype)
    return out


def adrt_T(n, b, dtype=float):
    """Transpose R^T: (4, 2N-1, N) -> N x N, summing the four quadrant back-projections (adrtcore.py:131-137)."""
    N = 1 << n
    b = np.asarray(b, dtype=dtype).reshape(4, 2 * N - 1, N)
    x = np.zeros((N, N), dtype=dtype)
    for q in range(4):
        x += T_apply_T(q, sq_adrt_T(n, b[q], dtype))
    return x


def mask_full(n):
    """Structurally non-zero entries of the sinogram: row h + N - 1 with h >= -s in column s (adrtcore.py:140-146)."""
    N = 1 << n
    h = np.arange(2 * N - 1)[:, None] - (N - 1)
    s = np.arange(N)[None, :]
    return np.broadcast_to(h >= -s, (4, 2 * N - 1, N)).copy()


def delta_s(n, s, t):
    """Digital-line offset delta_s(t) = sum_k bit_{n-1-k}(s) * floor((t + 2^k) / 2^{k+1}) (adrtcore.py:179-185)."""
    return sum(((t + (1 << k)) >> (k + 1)) for k in range(n) if (s >> (n - 1 - k)) & 1)


def digital_line(n, h, s):
    """Pixels (row, column) of the digital line through offset h with slope index s (adrtcore.py:188-190)."""
    return [(h + delta_s(n, s, t), t) for t in range(1 << n)]


def dense_from_op(op, in_shape, out_shape):
    """Dense matrix of a linear operator by columns (adrtcore.py:152-161)."""
    nin = int(np.prod(in_shape))
    nout = int(np.prod(out_shape))
    A = np.zeros((nout, nin))
    for k in range(nin):
        e = np.zeros(nin)
        e[k] = 1.0
        A[:, k] = np.asarray(op(e.reshape(in_shape))).ravel()
    return A
