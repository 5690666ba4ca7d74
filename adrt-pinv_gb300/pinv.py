"""Moore-Penrose pseudoinverse of the full ADRT on the GPU: drop-in for the reference's pinv.py (pinv.py:1-90).

    R^+ b = (R^T R)^{-1} R^T b

  cgls(n, b, tol, maxit, x0, callback)             CGLS on min ||R x - b|| (pinv.py:23-48)
  pcg_normal(n, b, M, tol, maxit, x0, callback, rhs)  PCG on R^T R x = R^T b (pinv.py:51-82)
  pinv_dense(n)                                     dense pseudoinverse, small N (pinv.py:85-88)

Every iteration costs one spatial ADRT and one back-projection (the library's FP64 level kernels) plus FP64 inner
products and vector updates (csrc/cgls.cu). b may be one sinogram (4, 2N-1, N) or a batch (B, 4, 2N-1, N), NumPy
or torch; a batch is solved at once, each sinogram with its own scalars and its own stopping test, and each ends
with the iterate the reference's loop would return for it alone. NumPy in -> NumPy out; torch in -> torch (CUDA)
out. Histories: one array per sinogram (the reference's `hist`), a list of them for a batch.

Without a callback the iterations run in blocks recorded once as a CUDA graph and replayed; the host reads the
per-image active flags between blocks only. With a callback (single sinogram only, as in the reference) each
iteration is followed by callback(it, x, norm) with x on the host.

A starting residual of exactly zero (R^T (b - R x0) = 0) ends at iteration 0 with x = x0, a least-squares
solution; the reference's loop divides by zero there.
"""

import ctypes

import numpy as np
import torch

from . import _lib as C
from .device import graph_capture


def _nblk(nimg, length, sms):
    """CTAs per image of the inner products: enough to cover the SMs a few times, at least 2048 elements each."""
    return int(max(1, min(-(-8 * sms // nimg), length // 2048 + 1, 1024)))


def _as_batch(b, N, what):
    is_torch = isinstance(b, torch.Tensor)
    bt = b if is_torch else torch.from_numpy(np.ascontiguousarray(np.asarray(b, dtype=np.float64)))
    single = bt.dim() == 3 if what == "sino" else bt.dim() == 2
    shape = (4, 2 * N - 1, N) if what == "sino" else (N, N)
    bt = bt.reshape((-1,) + shape)
    return is_torch, single, bt


class _Solver:
    def __init__(self, n, nimg, maxit, tol, device, block):
        if n < 1 or n > 12:
            raise ValueError("n must be in [1, 12]")
        C.load()
        self.n, self.N, self.nimg = n, 1 << n, int(nimg)
        self.maxit, self.tol = int(maxit), float(tol)
        self.device = torch.device(device)
        self.block = max(1, int(block))
        N, dev = self.N, self.device
        f64 = dict(dtype=torch.float64, device=dev)
        self.img = lambda: torch.zeros((self.nimg, N, N), **f64)
        self.sino = lambda: torch.zeros((self.nimg, 4, 2 * N - 1, N), **f64)
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        self.nblk = _nblk(self.nimg, N * N, sms)
        self.scratch = torch.empty(2 * self.nimg * 4 * (2 * N - 1) * N, **f64)
        self.partial = torch.zeros(self.nimg * self.nblk, **f64)
        self.scal = torch.zeros(self.nimg * 4, **f64)
        self.it = torch.zeros(self.nimg, dtype=torch.int32, device=dev)
        self.active = torch.zeros(self.nimg, dtype=torch.int32, device=dev)
        self.hist = torch.zeros((self.nimg, self.maxit + 1), **f64)
        self.graph = None

    def _fill(self, st, names):
        st.n, st.nimg, st.maxit, st.nblk, st.tol = self.n, self.nimg, self.maxit, self.nblk, self.tol
        for f in names:
            setattr(st, f, getattr(self, f).data_ptr())
        return st

    def results(self):
        its = self.it.cpu().numpy()
        hist = self.hist.cpu().numpy()
        return [hist[i, : its[i] + 1].copy() for i in range(self.nimg)]

    def _run_blocks(self, step_block):
        """Replay blocks of iterations until no image is active (graph recorded on the first block)."""
        while bool(self.active.any()):
            if self.graph is None:
                side = torch.cuda.Stream(device=self.device)
                side.wait_stream(torch.cuda.current_stream(self.device))
                with torch.cuda.stream(side):
                    g = torch.cuda.CUDAGraph()
                    with graph_capture(g, side):
                        step_block()
                torch.cuda.current_stream(self.device).wait_stream(side)
                self.graph = g
            self.graph.replay()


class CglsSolver(_Solver):
    """Device state of CGLS for `nimg` sinograms of size N = 2^n (pinv.py:23-48)."""

    def __init__(self, n, nimg=1, maxit=10000, tol=1e-12, device="cuda", block=16):
        super().__init__(n, nimg, maxit, tol, device, block)
        self.x, self.p, self.s = self.img(), self.img(), self.img()
        self.r, self.q = self.sino(), self.sino()
        self.state = self._fill(C.CglsState(), ("x", "p", "s", "r", "q", "scratch", "partial", "scal", "it",
                                                "active", "hist"))

    def start(self, b, x0=None):
        """b: (nimg, 4, 2N-1, N) FP64 on the device; x0 None (zeros) or (nimg, N, N)."""
        if x0 is None:
            self.x.zero_()
        else:
            self.x.copy_(x0)
        C.call("adrt_cgls_start", ctypes.byref(self.state), C.ptr(b), C.stream_handle())

    def iterate(self, k):
        C.call("adrt_cgls_iterate", ctypes.byref(self.state), int(k), C.stream_handle())

    def solve(self, b, x0=None, callback=None):
        """Run to convergence (or maxit) for every sinogram; returns (x (nimg, N, N) device tensor, histories)."""
        self.start(b, x0)
        if callback is None:
            self._run_blocks(lambda: self.iterate(self.block))
        else:
            while bool(self.active.any()):
                self.iterate(1)
                k = int(self.it[0])
                callback(k - 1, self.x[0].cpu().numpy(), float(self.hist[0, k]))
        return self.x, self.results()


class PcgSolver(_Solver):
    """Device state of PCG on R^T R x = R^T b for `nimg` images (pinv.py:51-82). M: None (identity, the whole
    iteration on the device, replayed from a CUDA graph) or a callable taking the residuals as a device tensor
    (nimg, N, N) FP64 and returning M r of the same shape (called once per iteration, for all images)."""

    def __init__(self, n, nimg=1, M=None, maxit=10000, tol=1e-12, device="cuda", block=16):
        super().__init__(n, nimg, maxit, tol, device, block)
        self.M = M
        self.x, self.r, self.p, self.q = self.img(), self.img(), self.img(), self.img()
        self.z = self.r if M is None else self.img()
        self.t = self.sino()
        self.state = self._fill(C.PcgState(), ("x", "r", "z", "p", "q", "t", "scratch", "partial", "scal", "it",
                                               "active", "hist"))

    def _precondition(self):
        if self.M is not None:
            self.z.copy_(self.M(self.r))

    def _one(self):
        st = C.stream_handle()
        C.call("adrt_pcg_step", ctypes.byref(self.state), st)
        self._precondition()
        C.call("adrt_pcg_direction", ctypes.byref(self.state), st)

    def solve(self, rhs, x0=None, callback=None):
        """rhs = R^T b (nimg, N, N) on the device; returns (x, histories)."""
        if x0 is None:
            self.x.zero_()
        else:
            self.x.copy_(x0)
        st = C.stream_handle()
        C.call("adrt_pcg_start", ctypes.byref(self.state), C.ptr(rhs), st)
        self._precondition()
        C.call("adrt_pcg_rho", ctypes.byref(self.state), st)
        if callback is None and self.M is None:
            self._run_blocks(lambda: [self._one() for _ in range(self.block)])
        else:
            while bool(self.active.any()):
                self._one()
                if callback is not None:
                    k = int(self.it[0])
                    callback(k - 1, self.x[0].cpu().numpy(), float(self.hist[0, k]))
        return self.x, self.results()


def _finish(x, hists, is_torch, single):
    out = x[0] if single else x
    out = out.clone() if is_torch else out.cpu().numpy()
    return out, (hists[0] if single else hists)


def cgls(n, b, tol=1e-12, maxit=10000, x0=None, callback=None, device="cuda"):
    """CGLS for min ||R x - b||_2 (pinv.py:23-48); returns (x, hist)."""
    N = 1 << n
    is_torch, single, bt = _as_batch(b, N, "sino")
    if callback is not None and bt.shape[0] != 1:
        raise ValueError("a callback is supported for a single sinogram only")
    bt = bt.to(device=device, dtype=torch.float64).contiguous()
    S = CglsSolver(n, bt.shape[0], maxit, tol, device)
    x0t = None if x0 is None else _as_batch(x0, N, "img")[2].to(device=device, dtype=torch.float64)
    x, hists = S.solve(bt, x0t, callback)
    return _finish(x, hists, is_torch, single)


def pcg_normal(n, b, M=None, tol=1e-12, maxit=10000, x0=None, callback=None, rhs=None, device="cuda"):
    """PCG for R^T R x = R^T b with SPD preconditioner M (pinv.py:51-82); returns (x, hist of ||r||_2).
    M: None for the identity, else a callable on device tensors (nimg, N, N) -> (nimg, N, N); rhs (optional)
    replaces R^T b."""
    from . import adrtcore

    N = 1 << n
    if rhs is None:
        is_torch, single, bt = _as_batch(b, N, "sino")
        rt = adrtcore.adrt_T(n, bt.to(device=device, dtype=torch.float64).contiguous())
    else:
        is_torch, single, rt = _as_batch(rhs, N, "img")
        rt = rt.to(device=device, dtype=torch.float64).contiguous()
    if callback is not None and rt.shape[0] != 1:
        raise ValueError("a callback is supported for a single right-hand side only")
    S = PcgSolver(n, rt.shape[0], M, maxit, tol, device)
    x0t = None if x0 is None else _as_batch(x0, N, "img")[2].to(device=device, dtype=torch.float64)
    x, hists = S.solve(rt, x0t, callback)
    return _finish(x, hists, is_torch, single)


def adrt_dense(n, device="cuda"):
    """The ADRT as a dense (4 (2N-1) N) x N^2 FP64 matrix (adrtcore.adrt_dense): the GPU transform of every unit
    image, as a NumPy array."""
    from . import adrtcore

    N = 1 << n
    E = torch.eye(N * N, dtype=torch.float64, device=device).reshape(N * N, N, N)
    return adrtcore.adrt(n, E).reshape(N * N, -1).T.cpu().numpy()


def pinv_dense(n, device="cuda"):
    """Dense Moore-Penrose pseudoinverse of the ADRT, N^2 x (4 (2N-1) N), small N only (pinv.py:85-88): the dense
    matrix from the GPU transform, its pseudoinverse by torch.linalg.pinv in FP64 on the GPU."""
    A = torch.from_numpy(adrt_dense(n, device)).to(device)
    return torch.linalg.pinv(A).cpu().numpy()
