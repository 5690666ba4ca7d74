"""The ADRT's normal operator row by row in the offset-frequency domain, on the GPU: the competitor path of the
reference's patch to the `adrt` package (patches/adrt-gram-freq.patch):

  gram_freq(a, omega)   the C++ kernel gram_freq (patch lines 161-250): out[b, k] = A_k^* A_k a[b, k] for complex
                        rows a (..., rows, N), A_k = B_n ... B_1 the butterfly product at offset frequency omega[k]
  gram(a)               adrt.core.gram (patch, core.py): R^T R a for real images (..., N, N), the quadrant pairs
                        packed as complex rows, an FFT along the offset, gram_freq on every row, the inverse FFT
  lstsq_cheb(b, ...)    adrt.core.lstsq_cheb (patch, core.py): the fixed-degree Chebyshev least-squares inverse
                        x_D = c_D(R^T R) R^T b on a spectral interval [lam_min, lam_max]

All three run on the library's kernels: gram_freq is the row engine's Gram op ('M', 1, n) with a per-row twiddle
table built on the device from omega; gram and lstsq_cheb are the device pipeline of the packed passes
(pack + FFT kernel, row engine, inverse FFT + unpack) with that op, and lstsq_cheb's iteration is the pipeline's
outer Chebyshev step (FP64 iterates). Images and sinograms are in this repository's (the reference's) layout;
R^T R does not depend on the layout. The patch's mapping between the `adrt` package's sinogram layout and this one
(skimage_adrt_pkg.py:17-52) needs the `adrt` package itself and is not provided.

float32 input runs the rows in FP32 (complex64), float64 in FP64; NumPy in -> NumPy out, torch in -> torch out.
"""

import ctypes

import numpy as np
import torch

from . import _lib as C
from .device import OPCODE, Pipeline
from .plan import Plan

_REAL = {torch.complex64: torch.float32, torch.complex128: torch.float64}


def gram_freq(a, omega):
    """A_omega^* A_omega applied to every row of a (..., rows, N) complex (N = 2^n), omega (rows,) real offset
    frequencies of the same precision (complex64 with float32, complex128 with float64), as the patch's C++
    gram_freq; returns a new array of a's shape and dtype."""
    is_torch = isinstance(a, torch.Tensor)
    at = a if is_torch else torch.from_numpy(np.ascontiguousarray(a))
    om = omega if isinstance(omega, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(omega))
    if at.dim() < 2:
        raise ValueError("array must have shape (..., rows, N) with N a power of two")
    rows, N = at.shape[-2], at.shape[-1]
    if N < 2 or N & (N - 1) or rows < 1 or at.numel() == 0:
        raise ValueError("array must have shape (..., rows, N) with N a power of two")
    if at.dtype not in _REAL:
        raise TypeError(f"unsupported array dtype {at.dtype}")
    if om.dim() != 1 or om.shape[0] != rows:
        raise ValueError("omega must have one entry per row")
    if om.dtype != _REAL[at.dtype]:
        raise TypeError(f"omega must be {_REAL[at.dtype]} for {at.dtype} rows")
    n = N.bit_length() - 1
    if n > 11:
        raise ValueError("N above 2048 is not supported")
    dev = at.device if at.is_cuda else torch.device("cuda")
    X = at.to(dev).reshape(-1, rows, N).contiguous().clone()
    z = torch.polar(torch.ones(rows, dtype=torch.float64, device=dev), om.to(dev, torch.float64))
    code = C.dtype_code(_REAL[at.dtype])
    st = C.stream_handle()
    tab = torch.empty((rows, N // 2 + 1), dtype=at.dtype, device=dev)
    C.call("adrt_twiddle_table", code, n, rows, C.ptr(z), C.ptr(tab), st)
    counter = torch.zeros(4, dtype=torch.int32, device=dev)
    j = C.RowJob()
    j.dtype, j.n, j.nimg, j.nsel, j.img_stride = code, n, X.shape[0], rows, rows * N
    j.X, j.rows, j.freq_mod, j.roots, j.twtab = X.data_ptr(), None, rows, None, tab.data_ptr()
    j.deg, j.coef, j.coef_stride, j.tau = None, None, 0, 0.0
    j.nops = 1
    j.op[0], j.lo[0], j.hi[0] = OPCODE["M"], 1, n
    j.counter, j.grid = counter.data_ptr(), 0
    C.call("adrt_rows_run", ctypes.byref(j), st)
    out = X.reshape(at.shape)
    return out if is_torch and at.is_cuda else (out.cpu() if is_torch else out.cpu().numpy())


class NormalOperator:
    """R^T R (and the fixed-degree Chebyshev least squares on it) for a batch of B images of size N = 2^n in one
    precision: a device pipeline whose op lists are the Gram rows ('B', 1, n), ('BT', 1, n) and, for R^T b, the
    adjoint rows ('BT', 1, n)."""

    def __init__(self, n, batch=1, precision="fp64", device="cuda"):
        N = 1 << n
        self.n, self.N, self.B = n, N, int(batch)
        self.plan = Plan("lp", n, np.full(2 * N, 4.0), outer=(1.0, 2.0, 2))
        self.pipe = Pipeline(self.plan, self.B, precision, device)
        self.pipe.ops = {"G": [("B", 1, n), ("BT", 1, n)], "BP": [("BT", 1, n)]}
        self.out = torch.empty((self.B, N, N), dtype=torch.float64, device=self.pipe.device)

    def gram(self, x):
        """R^T R x for x (B, N, N) real on the device; returns an FP64 buffer (valid until the next call)."""
        self.pipe.G(x)
        return self.pipe.sum_parts(self.out)

    def lstsq_cheb(self, b, lo, hi, deg):
        """x_deg = c_deg(R^T R) R^T b for sinograms b (B, 4, 2N-1, N) FP64 on the device (FP64 result buffer)."""
        self.plan.set_outer((lo, hi, int(deg)))
        return self.pipe.apply(b)


_ops = {}


def _operator(n, batch, precision, device):
    key = (n, int(batch), precision, str(device))
    if key not in _ops:
        _ops[key] = NormalOperator(n, batch, precision, device)
    return _ops[key]


def _images(a):
    is_torch = isinstance(a, torch.Tensor)
    at = a if is_torch else torch.from_numpy(np.ascontiguousarray(np.asarray(a)))
    if at.dim() < 2 or at.shape[-1] != at.shape[-2]:
        raise ValueError(f"array must be square, but had shape {tuple(at.shape)}")
    N = at.shape[-1]
    if N < 1 or N & (N - 1):
        raise ValueError(f"array size must be a power of two, but was {N}")
    if at.dtype not in (torch.float32, torch.float64):
        raise TypeError(f"unsupported array dtype {at.dtype}")
    return is_torch, at


def _back(x, like, is_torch, dtype):
    x = x.reshape(like).to(dtype)
    if is_torch:
        return x
    return x.cpu().numpy()


def gram(a, device="cuda"):
    """R^T R a for square images a (..., N, N) float32 / float64 (adrt.core.gram of the patch), same shape and
    dtype; N = 1 is the identity."""
    is_torch, at = _images(a)
    N = at.shape[-1]
    if N == 1:
        return at.clone() if is_torch else at.numpy().copy()
    n = N.bit_length() - 1
    x = at.reshape(-1, N, N).to(device).contiguous()
    op = _operator(n, x.shape[0], "fp32" if at.dtype == torch.float32 else "fp64", device)
    out = op.gram(x)
    res = _back(out, at.shape, is_torch, at.dtype)
    return res.to(at.device) if is_torch else res


def lstsq_cheb(b, *, lam_min, lam_max=None, tol=1e-10, degree=None, device="cuda"):
    """Least-squares inverse of the ADRT by a fixed-degree Chebyshev polynomial (adrt.core.lstsq_cheb of the
    patch): x_D = c_D(R^T R) R^T b on [lam_min, lam_max], D = max(1, ceil(log(tol/2) / log(rho))) unless given,
    rho = (sqrt k - 1)/(sqrt k + 1), k = lam_max/lam_min. lam_max, when omitted, comes from 50 normalised power
    steps of R^T R from the patch's seeded start vector, enlarged by the residual norm. b: (..., 4, 2N-1, N)."""
    is_torch = isinstance(b, torch.Tensor)
    bt = b if is_torch else torch.from_numpy(np.ascontiguousarray(np.asarray(b)))
    if bt.dim() < 3 or bt.shape[-3] != 4 or bt.shape[-2] != 2 * bt.shape[-1] - 1:
        raise ValueError(f"array must have the shape of an ADRT output, but had shape {tuple(bt.shape)}")
    N = bt.shape[-1]
    if N < 2 or N & (N - 1):
        raise ValueError(f"array size must be a power of two, but was {N}")
    n = N.bit_length() - 1
    dtype = bt.dtype if bt.dtype in (torch.float32, torch.float64) else torch.float64
    prec = "fp32" if dtype == torch.float32 else "fp64"
    if lam_max is None:
        op1 = _operator(n, 1, prec, device)
        v = torch.from_numpy(np.random.default_rng(0).standard_normal((N, N)).astype(
            np.float32 if dtype == torch.float32 else np.float64)).to(device, torch.float64)
        v = v / v.norm()
        for _ in range(50):
            w = op1.gram(v[None])[0]
            v = w / w.norm()
        w = op1.gram(v[None])[0]
        theta = float((v * w).sum())
        lam_max = theta + float((w - theta * v).norm())
    lo, hi = float(lam_min), float(lam_max)
    if not 0 < lo < hi:
        raise ValueError("need 0 < lam_min < lam_max")
    if degree is None:
        kap = hi / lo
        rho = (np.sqrt(kap) - 1) / (np.sqrt(kap) + 1)
        deg = max(1, int(np.ceil(np.log(tol / 2) / np.log(rho))))
    else:
        deg = int(degree)
    batch_shape = bt.shape[:-3]
    x = bt.reshape(-1, 4, 2 * N - 1, N).to(device=device, dtype=torch.float64).contiguous()
    op = _operator(n, x.shape[0], prec, device)
    out = op.lstsq_cheb(x, lo, hi, deg)
    res = out.reshape(tuple(batch_shape) + (N, N)).to(dtype)
    return res.clone() if is_torch else res.cpu().numpy()


__all__ = ["gram_freq", "gram", "lstsq_cheb", "NormalOperator"]
