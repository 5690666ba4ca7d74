"""GPU explicit oblique inverses with the reference's Python surface.

`FastLpGpu` / `FastHybridGpu` take the constructor arguments of fastops.FastLp / FastHybrid (fastops.py:262-320) and
fastcpp.FastLpCpp / FastHybridCpp (`lam_bound`, fastcpp.py:137-169), keep their attributes (n, N, L, tau, oms, z,
lam_max, deg, lo, hi, outer_deg, eng.count, eng.n_dense) and methods (frame_window / Gh, backproject, apply), and
run everything on one GPU:
  * setup: power iteration for Lambda_k (row kernels, FP64), degrees and tables (host FP64), outer interval by
    Lanczos (scipy eigsh, as the reference) whose matvecs are the device operator in FP64;
  * apply: the device pipeline (pack+FFT, fused row engine, iFFT+unpack, G_1 stencil, outer update).
Extra keywords: deg_cap (degree-p filter: d_k <- min(p, d_k)), precision ('fp32' | 'fp64'), outer=(lo, hi, D) to
inject a precomputed outer interval, device, high_rows ('dense': the rows with d_k > dense_cap take the exact dense
filter, as the reference; 'ff': they keep the polynomial filter in float-float arithmetic, compensated rows without
operator memory), stencil_precision (hybrid: 'fp32' | 'ff' | 'fp64' for the cross-quadrant preconditioner).

`apply` accepts one sinogram (4, 2N-1, N) or a batch (B, 4, 2N-1, N), as NumPy (host) or torch (CUDA) arrays, and
returns the same kind: NumPy FP64 for NumPy input, a torch FP64 CUDA tensor for CUDA input.
"""

import numpy as np
import torch

from . import _lib as C
from . import stencils
from .device import Pipeline
from .plan import Plan, offset_freqs, roots_of_unity


class EngineInfo:
    """The parts of fastops.RowEngine callers read: the level-row counter and the number of dense rows."""

    def __init__(self, n_dense):
        self.count = [0]
        self.n_dense = n_dense


def power_lam_max(n, m_lo, iters=40, safety=1.5, device="cuda", seeds=(0, 1)):
    """Lambda_k = safety x Rayleigh quotient after `iters` normalised power steps of M_k = B^* B over levels m_lo..n,
    for all L = 2N frequencies, computed by the row kernels in FP64 (fastcpp.py:102-118, same start vectors)."""
    N, L = 1 << n, 2 << n
    if len(seeds) == 2:
        V = np.random.default_rng(seeds[0]).standard_normal((L, N)) + 1j * np.random.default_rng(seeds[1]).standard_normal((L, N))
    else:
        rng = np.random.default_rng(seeds[0])
        V = rng.standard_normal((L, N)) + 1j * rng.standard_normal((L, N))
    dev = torch.device(device)
    Vd = torch.from_numpy(V).to(dev)
    z = torch.from_numpy(roots_of_unity(L)).to(dev)
    tab = torch.empty((L, N // 2 + 1), dtype=torch.complex128, device=dev)
    out = torch.empty(L, dtype=torch.float64, device=dev)
    cnt = torch.zeros(4, dtype=torch.int32, device=dev)
    st = C.stream_handle()
    C.call("adrt_twiddle_table", C.F64, n, L, C.ptr(z), C.ptr(tab), st)
    C.call("adrt_power_rows", C.F64, n, L, C.ptr(Vd), C.ptr(tab), m_lo, iters, safety, C.ptr(out), C.ptr(cnt), st)
    return out.cpu().numpy()


def cert_lam_max(n, oms, m_lo=1, threads=1, device="cuda"):
    """Certified bounds (fastcpp.py:121-125) by the device row-sum recursion."""
    del threads
    om = torch.as_tensor(np.ascontiguousarray(oms, dtype=float), device=device)
    out = torch.empty(len(oms), dtype=torch.float64, device=device)
    C.call("adrt_cert_rowsum_dev", n, len(oms), C.ptr(om), m_lo, C.ptr(out), C.stream_handle())
    return out.cpu().numpy()


def explicit_lam_max(n, oms):
    """Lambda_k = min(N^2, 2N(1+n)/|omega_k|) (fastcpp.py:128-134)."""
    N = 1 << n
    w = np.abs(np.asarray(oms, dtype=float))
    lam = np.full(len(w), float(N) ** 2)
    nz = w > 0
    lam[nz] = np.minimum(float(N) ** 2, 2.0 * N * (1 + n) / w[nz])
    return lam


class _GpuInverse:
    method = None
    m_lo = 1

    def _setup(self, n, tau_fac, eps_in, eps, threads, lam_max, power_iters, safety, dense_cap, deg_cap, precision,
               outer, device, lam_bound, precond="none", g1_deg=14, stencil_precision=None, high_rows="dense"):
        if not torch.cuda.is_available():
            raise RuntimeError("a CUDA device is required (no CPU fallback)")
        C.load()
        self.n = n
        self.N = N = 1 << n
        self.L = L = 2 * N
        self.tau = tau_fac * N
        self.threads = threads
        self.oms = offset_freqs(L)
        self.z = np.exp(1j * self.oms)
        self.device = torch.device(device)
        self.precision = precision
        self.stencil_precision = stencil_precision
        self.graphs = True  # apply() replays a CUDA graph per batch size from its second call on
        if lam_max is None:
            if lam_bound == "power":
                lam_max = power_lam_max(n, self.m_lo, power_iters, safety, device)
            elif lam_bound == "cert":
                lam_max = cert_lam_max(n, self.oms, self.m_lo, device=device)
            elif lam_bound == "explicit" and self.method == "lp":
                lam_max = explicit_lam_max(n, self.oms)
            else:
                raise ValueError(f"lam_bound {lam_bound!r}")
        if high_rows == "ff" and precision != "fp32":
            high_rows = "dense"  # in FP64 the polynomial rows are exact enough; the compensated kernel is FP32-only
        self.plan = Plan(self.method, n, lam_max, tau_fac, eps_in, eps, deg_cap=deg_cap, dense_cap=dense_cap,
                         precond=precond, g1_deg=g1_deg, high_rows=high_rows)
        self.lam_max, self.deg = self.plan.lam_max, self.plan.deg
        self.eng = EngineInfo(len(self.plan.dense_freqs))
        self._pipes = {}
        if outer is None:
            outer = self._outer_interval(eps)
        self.plan.set_outer(outer)
        self.lo, self.hi, self.outer_deg = self.plan.lo, self.plan.hi, self.plan.outer_deg
        self.eng.count = [0]

    # ---------------------------------------------------------------- device pipelines
    def pipeline(self, batch=1, precision=None):
        key = (int(batch), precision or self.precision)
        if key not in self._pipes:
            self._pipes[key] = Pipeline(self.plan, batch, key[1], self.device, self.stencil_precision)
        return self._pipes[key]

    def _count(self, pipe, before):
        self.eng.count[0] += pipe.tables.count - before

    # ---------------------------------------------------------------- setup: outer interval (fastops.py:222-245)
    def _outer_interval(self, eps):
        import scipy.sparse.linalg as spla

        N = self.N
        # the interval is estimated to a relative accuracy of about 1e-3 and widened by 1% on both sides: the FP64
        # operator is used up to N = 512, the FP32 one (relative error ~1e-6) above, where FP64 matvecs dominate setup
        pipe = self.pipeline(1, "fp64" if N <= 512 else "fp32")

        def G(v):
            return self._image_op(pipe, lambda x: pipe.G(x), v.reshape(N, N)).ravel()

        A = spla.LinearOperator((N * N, N * N), matvec=G, dtype=float)
        # a seeded Lanczos start vector (ARPACK's default is random), so that a plan is the same on every build
        v0 = np.random.default_rng(0).uniform(-1.0, 1.0, N * N)
        if self.method == "lp" or self.plan.precond == "none":
            lo, ulo = spla.eigsh(A, k=1, which="SA", tol=1e-3, maxiter=300, v0=v0)
            hi, uhi = spla.eigsh(A, k=1, which="LA", tol=1e-3, maxiter=300, v0=v0)

            def res(th, u):
                return np.linalg.norm(A.matvec(u[:, 0]) - th * u[:, 0])
        else:
            Pinv = stencils.G1_apply if self.plan.precond == "g1" else stencils.lorr_fwd
            Mop = spla.LinearOperator((N * N, N * N), matvec=lambda v: Pinv(v.reshape(N, N)).ravel(), dtype=float)

            def Pv(v):
                x = torch.from_numpy(np.ascontiguousarray(v.reshape(1, N, N))).to(self.device)
                pipe.s.copy_(x.to(pipe.s.dtype))
                return pipe.precond(pipe.s).double().cpu().numpy().ravel()

            Minv = spla.LinearOperator((N * N, N * N), matvec=Pv, dtype=float)
            lo, ulo = spla.eigsh(A, k=1, M=Mop, Minv=Minv, which="SA", tol=1e-3, maxiter=300, v0=v0)
            hi, uhi = spla.eigsh(A, k=1, M=Mop, Minv=Minv, which="LA", tol=1e-3, maxiter=300, v0=v0)

            def res(th, u):
                u = u[:, 0]
                r = A.matvec(u) - th * Mop.matvec(u)
                return np.sqrt(abs(r @ Minv.matvec(r))) / np.sqrt(abs(u @ Mop.matvec(u)))

        lo, hi = float(lo[0]), float(hi[0])
        lo_b, hi_b = (lo - res(lo, ulo)) * 0.99, (hi + res(hi, uhi)) * 1.01
        from .plan import outer_degree

        return lo_b, hi_b, outer_degree(lo_b, hi_b, eps)

    def _image_op(self, pipe, fn, x):
        xd = torch.from_numpy(np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(1, self.N, self.N)))
        xd = xd.to(self.device)
        before = pipe.tables.count
        fn(xd)
        out = torch.empty((1, self.N, self.N), dtype=torch.float64, device=self.device)
        pipe.sum_parts(out)
        self._count(pipe, before)
        return out[0].cpu().numpy()

    # ---------------------------------------------------------------- the reference's methods
    def _G(self, x):
        pipe = self.pipeline(1)
        return self._image_op(pipe, lambda xd: pipe.G(xd), x)

    def backproject(self, b):
        """E^T sum_q ... (fastops.py:283-285 / 333-335) of one sinogram (4, 2N-1, N) -> N x N (FP64)."""
        pipe = self.pipeline(1)
        bd = torch.from_numpy(np.ascontiguousarray(np.asarray(b, dtype=np.float64).reshape(1, 4, 2 * self.N - 1, self.N)))
        bd = bd.to(self.device)
        out = torch.empty((1, self.N, self.N), dtype=torch.float64, device=self.device)
        before = pipe.tables.count
        pipe.backproject_into(bd, out)
        self._count(pipe, before)
        return out[0].cpu().numpy()

    def apply(self, b, out=None):
        """x = L b (fastops.py:287-288 / 337-338) for one sinogram or a batch; see the module docstring.
        out: optional result buffer (torch, host or device) written with a stream-ordered copy and returned."""
        is_torch = isinstance(b, torch.Tensor)
        bt = b if is_torch else torch.from_numpy(np.ascontiguousarray(np.asarray(b, dtype=np.float64)))
        single = bt.dim() == 3
        if single:
            bt = bt.unsqueeze(0)
        if tuple(bt.shape[1:]) != (4, 2 * self.N - 1, self.N):
            raise ValueError(f"sinograms must have shape (4, {2 * self.N - 1}, {self.N})")
        if bt.dtype not in (torch.float32, torch.float64):
            bt = bt.double()
        host_in = not bt.is_cuda
        pipe = self.pipeline(bt.shape[0])
        before = pipe.tables.count
        if self.graphs and getattr(pipe, "graph", None) is None and getattr(pipe, "_applied", False):
            pipe.capture()  # the second call of this batch size records the whole apply as a CUDA graph
            before = pipe.tables.count
        if self.graphs and getattr(pipe, "graph", None) is not None:
            if out is not None and host_in and not out.is_cuda and bt.dtype == torch.float64 and bt.is_pinned():
                # host in, host out: pipelined across calls (the copy of this batch overlaps the previous graph);
                # the dense kernel's error flag of a call is checked at the next call or by check()
                pipe.replay_host(bt.contiguous(), out[None] if single else out)
                self._count(pipe, before)
                self._last_pipe = pipe
                return out
            x = pipe.replay(bt.contiguous())
        else:
            x = pipe.apply(bt.to(self.device, non_blocking=True).contiguous())
            pipe._applied = True
        self._count(pipe, before)
        x = x[0] if single else x
        if out is not None:
            out.copy_(x, non_blocking=True)
            if not out.is_cuda:
                pipe.tables.raise_if_error()
            return out
        if not is_torch:
            res = x.cpu().numpy()
            pipe.tables.raise_if_error()
            return res
        if host_in:
            res = x.to("cpu")
            pipe.tables.raise_if_error()
            return res
        return x.clone()


def _check(self):
    """Wait for the last pipelined host call (apply with pinned host input and a host `out`) and raise if its dense
    rows failed."""
    pipe = getattr(self, "_last_pipe", None)
    if pipe is not None:
        pipe.check_host()


_GpuInverse.check = _check


class FastLpGpu(_GpuInverse):
    """L_p inverse on the GPU: fastops.FastLp / fastcpp.FastLpCpp surface (fastops.py:261-288, fastcpp.py:137-153)."""

    method = "lp"
    m_lo = 1

    def __init__(self, n, tau_fac=0.2, eps_in=0.1, eps=1e-10, threads=8, lam_max=None, power_iters=40, safety=1.5,
                 dense_cap=None, lam_bound="power", deg_cap=None, precision="fp32", outer=None, device="cuda",
                 high_rows="dense"):
        self._setup(n, tau_fac, eps_in, eps, threads, lam_max, power_iters, safety, dense_cap, deg_cap, precision, outer,
                    device, lam_bound, high_rows=high_rows)

    def frame_window(self, x):
        """E^T sum_q T_q^T [M p(M)] T_q E x (fastops.py:277-281), FP64 N x N in and out."""
        return self._G(x)


class FastHybridGpu(_GpuInverse):
    """Hybrid inverse on the GPU: fastops.FastHybrid / fastcpp.FastHybridCpp surface (fastops.py:291-338,
    fastcpp.py:156-169). stencil_precision sets the precision of the explicit cross-quadrant preconditioner
    (default: the pipeline precision)."""

    method = "hybrid"
    m_lo = 2

    def __init__(self, n, tau_fac=0.2, eps_in=0.1, eps=1e-10, threads=8, lam_max=None, g1_deg=14, power_iters=40,
                 safety=1.5, dense_cap=None, precond="g1", lam_bound="power", deg_cap=None, precision="fp32", outer=None,
                 device="cuda", stencil_precision=None, high_rows="dense"):
        if n < 2:
            raise ValueError("the hybrid inverse needs n >= 2")
        self.g1_deg, self.precond = g1_deg, precond
        self._setup(n, tau_fac, eps_in, eps, threads, lam_max, power_iters, safety, dense_cap, deg_cap, precision, outer,
                    device, lam_bound, precond, g1_deg, stencil_precision, high_rows)

    def Gh(self, x):
        """G_h x (fastops.py:325-331), FP64 N x N in and out."""
        return self._G(x)

    def P(self, y):
        """The preconditioner (fastops.py:322-323) on one N x N image."""
        pipe = self.pipeline(1)
        yd = torch.from_numpy(np.ascontiguousarray(np.asarray(y, dtype=np.float64).reshape(1, self.N, self.N)))
        pipe.s.copy_(yd.to(self.device).to(pipe.s.dtype))
        return pipe.precond(pipe.s)[0].double().cpu().numpy()
