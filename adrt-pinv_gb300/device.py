"""Device pipeline of the explicit oblique inverses (one GPU, stream-ordered, no host round trips).

For a plan, a batch size B and a precision, `Pipeline` owns every device buffer and evaluates, for B images at once:
  packed_image / packed_sino : fastops._packed (fastops.py:209-220) = pack+FFT kernel -> row engine -> iFFT+unpack
  precond                    : the hybrid's P = g1_inv / lorr_inv (fasthybrid.py:108-130)
  apply                      : backproject + fixed-degree outer Chebyshev (fastops.py:247-258, 283-288, 333-338)
Layouts in HBM (per batch): Y (B, 2L, N) complex rows (pair (0,1) then (2,3), each L offset-frequency rows);
three real image-space partial sums (3, B, N, N); outer state x, x_prev, x_new as float-float planes (B, 2, N, N)
FP32 with y FP32 where the register-resident fused outer step runs (FP32 rows and stencil, 64 <= N <= 512), else
(B, N, N) FP64; the FP64 result (B, N, N) converted once per apply."""

import contextlib
import ctypes
import gc
import weakref

import numpy as np
import torch

from . import _lib as C
from .plan import Plan, outer_coeffs, roots_of_unity

OPCODE = {"B": C.OP_B, "BT": C.OP_BT, "M": C.OP_M, "P": C.OP_P}
PRECISIONS = {"fp32": torch.float32, "fp64": torch.float64}
# the cross-quadrant preconditioner's precision: "ff" is float-float (pairs of FP32, about 48 significant bits) in the
# fused outer step, with FP64 buffers for the separate stencil kernels where the fused step does not apply
STENCIL_PRECISIONS = {"fp32": torch.float32, "fp64": torch.float64, "ff": torch.float64}
STENCIL_CODES = {"fp32": C.F32, "fp64": C.F64, "ff": C.F32X2}


def fuse_ops(ops):
    """Merge ('B', lo, hi) immediately followed by ('BT', lo, hi) into ('M', lo, hi) (one Gram application)."""
    out = []
    for op in ops:
        op = (op[0], int(op[1]), int(op[2]))
        if out and op[0] == "BT" and out[-1][0] == "B" and out[-1][1:] == op[1:]:
            out[-1] = ("M", op[1], op[2])
        else:
            out.append(op)
    return out


def _cdtype(real):
    return torch.complex64 if real == torch.float32 else torch.complex128


@contextlib.contextmanager
def graph_capture(graph, stream):
    """torch.cuda.graph with Python's cyclic garbage collector paused for the capture: a collection inside it could
    destroy CUDA objects (graphs, events, streams) of unreachable pipelines, which invalidates a global-mode
    capture ("operation failed due to a previous error during capture")."""
    enabled = gc.isenabled()
    gc.collect()
    gc.disable()
    try:
        with torch.cuda.graph(graph, stream=stream):
            yield
    finally:
        if enabled:
            gc.enable()


class RowTables:
    """Device copies of a plan's per-frequency tables in one precision, plus the work counter."""

    def __init__(self, plan: Plan, real, device):
        self.plan, self.real, self.device = plan, real, device
        self.code = C.dtype_code(real)
        self.roots = torch.from_numpy(roots_of_unity(plan.L)).to(device=device, dtype=_cdtype(real))
        self.deg = torch.from_numpy(plan.deg.astype(np.int32)).to(device)
        self.coef = torch.from_numpy(np.ascontiguousarray(plan.coef.ravel())).to(device=device, dtype=real)
        self.rows_main = torch.from_numpy(plan.packed_rows(dense=False).astype(np.int32)).to(device)
        self.rows_dense = torch.from_numpy(plan.packed_rows(dense=True).astype(np.int32)).to(device)
        self.counter = torch.zeros(4, dtype=torch.int32, device=device)
        # dense rows: row r of the dense selection uses frequency table index dense_idx[r]
        idx = {int(k): i for i, k in enumerate(plan.dense_freqs)}
        self.dense_sel = np.array([idx[int(r) % plan.L] for r in plan.packed_rows(dense=True)], dtype=np.int64)
        self._dense_dev = {}
        self.count = 0  # level-rows applied, counted as the reference does
        self.timer = None  # list: when set, (start, end) CUDA events of every polynomial-row launch are appended
        self.use_tc = real == torch.float32  # dense rows on tensor cores in FP32
        self.split_dense = True  # the tensor-core rows on pre-split operators where the kernel exists (dense_mode)
        # small batches (<= 16 images, FP32): the streaming CUDA-core kernel, with the operators stored transposed;
        # set by the owning pipeline before the first dense table is built
        self.stream_dense = False
        self.row_grid = 0  # CTAs of the row programs (0: one per SM); set by the autotuner
        self.dense_tile = 0  # images per CTA of the tensor-core dense rows (0: from the batch); set by the autotuner
        self.err = torch.zeros(1, dtype=torch.int32, device=device)
        self._zd = None
        # compensated high rows: float-float kernel in an FP32 pipeline; an FP64 pipeline runs them as ordinary
        # polynomial rows (FP64 is accurate enough there)
        self.high_poly = getattr(plan, "high_rows", "dense") == "ff" and len(plan.dense_freqs) > 0
        self.high_ff = self.high_poly and real == torch.float32
        if self.high_ff:
            # the compensated rows read the roots of unity and the filter constants in FP64
            self.roots64 = torch.from_numpy(roots_of_unity(plan.L)).to(device=device, dtype=torch.complex128)
            self.coef64 = torch.from_numpy(np.ascontiguousarray(plan.coef.ravel())).to(device=device,
                                                                                      dtype=torch.float64)

    def job(self, Y, ops, rows):
        p = self.plan
        B, R, N = Y.shape
        j = C.RowJob()
        j.dtype, j.n, j.nimg, j.nsel = self.code, p.n, B, int(rows.numel())
        j.img_stride = R * N
        j.X = Y.data_ptr()
        j.rows = rows.data_ptr()
        j.freq_mod = p.L
        j.roots = self.roots.data_ptr()
        j.twtab = None
        j.deg = self.deg.data_ptr()
        j.coef = self.coef.data_ptr()
        j.coef_stride = p.coef_stride
        j.tau = p.tau
        if len(ops) > C.MAX_OPS:
            raise ValueError("too many ops")
        j.nops = len(ops)
        for i, (op, lo, hi) in enumerate(ops):
            j.op[i], j.lo[i], j.hi[i] = OPCODE[op], lo, hi
        j.counter = self.counter.data_ptr()
        j.grid = self.row_grid
        return j

    def _timed_main(self, Y, ops, st):
        if self.timer is None:
            C.call("adrt_rows_run", ctypes.byref(self.job(Y, ops, self.rows_main)), st)
            return
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        C.call("adrt_rows_run", ctypes.byref(self.job(Y, ops, self.rows_main)), st)
        e1.record()
        self.timer.append((e0, e1, ops))

    def main_level_rows(self, ops):
        """Level-rows processed by the polynomial-row launch of one op list (the dense rows excluded)."""
        p = self.plan
        n_main = int(self.rows_main.numel())
        d = np.tile(p.deg, 2)[p.packed_rows(dense=False)]
        tot = 0
        for op, lo, hi in ops_unfused(fuse_ops(ops)):
            if op in ("B", "BT"):
                tot += n_main * (hi - lo + 1)
            elif op == "P":
                tot += int(np.sum(np.maximum(d - 1, 0))) * 2 * (hi - lo + 1)
        return tot

    def dense_table(self, fold_pre, fold_post, pre_b1=False, post_b1t=False):
        """The folded dense-row operators of one op list, one per dense packed row, in the row precision. Built on
        the host in FP64 up to n = 8 and on the device (FP64 torch, Cholesky form) for larger n."""
        key = (fold_pre, fold_post, pre_b1, post_b1t, self.stream_dense)
        # pipelines of one plan share their tables (same device, precision and layout) while any of them holds one
        shared = self.plan.__dict__.setdefault("_dense_shared", weakref.WeakValueDictionary())
        skey = (str(self.device), str(self.real), key)
        if key not in self._dense_dev and skey in shared:
            self._dense_dev[key] = shared[skey]
        if key not in self._dense_dev:
            if self.plan.n >= 9 and self.device.type == "cuda":
                N = self.plan.N
                out = torch.empty((len(self.dense_sel), N, N), dtype=_cdtype(self.real), device=self.device)
                sel = torch.from_numpy(self.dense_sel).to(self.device)
                for c0, T in dense_row_operator_device(self.plan, fold_pre, fold_post, pre_b1, post_b1t, self.device):
                    hit = ((sel >= c0) & (sel < c0 + T.shape[0])).nonzero().flatten()
                    Th = T[sel[hit] - c0]
                    out[hit] = (Th.transpose(-1, -2) if self.stream_dense else Th).to(out.dtype)
                self._dense_dev[key] = out
            else:
                T = self.plan.dense_row_operator(fold_pre, fold_post, pre_b1, post_b1t)[self.dense_sel]
                if self.stream_dense:
                    T = T.transpose(0, 2, 1)
                self._dense_dev[key] = torch.from_numpy(np.ascontiguousarray(T)).to(
                    device=self.device, dtype=_cdtype(self.real))
            shared[skey] = self._dense_dev[key]
        return self._dense_dev[key]

    def raise_if_error(self):
        """Raise if a tensor-core dense-row launch gave up on a bounded wait since the last check (reads one int: a
        device synchronisation, so callers make it where they synchronise anyway); clears the flag."""
        code = int(self.err.item())
        if code:
            self.err.zero_()
            more = ("" if code == 1 else "; the drain of its MMAs ran out as well, so later results on this stream "
                    "cannot be trusted")
            raise RuntimeError("dense_tc_kernel: an mbarrier wait ran out; the dense-row results of that launch "
                               "were not written" + more)

    def split_table(self, T):
        """The pre-split form of a dense table T for the complex-blocked tensor-core kernel (adrt_dense_split),
        built once per table and shared like the table itself."""
        Ws = getattr(T, "_adrt_split", None)  # held by the table itself: it lives exactly as long as T
        if Ws is None:
            N = self.plan.N
            Ws = torch.empty((T.shape[0], 4 * N * N), dtype=torch.float32, device=self.device)
            C.call("adrt_dense_split", self.plan.n, T.shape[0], C.ptr(T), C.ptr(Ws), C.stream_handle())
            T._adrt_split = Ws
        return Ws

    def dense_mode(self):
        """Kernel of the dense rows: 3 complex-blocked tensor cores on pre-split operators (FP32, 7 <= n <= 10),
        1 the real-form tensor-core kernel, 2 the streaming CUDA-core kernel (small FP32 batches), 0 CUDA cores."""
        if self.stream_dense:
            return 2
        if not self.use_tc:
            return 0
        return 3 if self.split_dense and 7 <= self.plan.n <= 10 else 1

    def dense_apply(self, Y, T):
        """Y[b, r] <- T_r Y[b, r] for the dense rows (FP32: tensor cores, or the streaming CUDA-core kernel for small
        batches; FP64: CUDA cores)."""
        B, R, N = Y.shape
        nd = int(self.rows_dense.numel())
        mode = self.dense_mode()
        if mode != 3 and (self._zd is None or self._zd.shape[1] != B):  # mode 3 writes in place
            self._zd = torch.empty((nd, B, N), dtype=Y.dtype, device=self.device)
        W = self.split_table(T) if mode == 3 else T
        C.call("adrt_dense_rows", self.code, self.plan.n, B, nd, C.ptr(self.rows_dense), C.ptr(W), C.ptr(Y), R * N,
               None if mode == 3 else C.ptr(self._zd), C.ptr(self.err), mode,
               self.dense_tile if mode in (1, 3) else 0, C.stream_handle())

    def run_ff(self, Y, ops):
        """The op list on the high-condition rows in float-float arithmetic (adrt_rows_ff_run)."""
        j = self.job(Y, ops, self.rows_dense)
        j.roots = self.roots64.data_ptr()
        j.coef = self.coef64.data_ptr()
        C.call("adrt_rows_ff_run", ctypes.byref(j), C.stream_handle())

    def main_job(self, Y, ops):
        """The row job of the polynomial rows of one op list (what run() launches first), for a caller that launches
        it itself (one persistent launch over several pipelines' rows)."""
        return self.job(Y, fuse_ops(ops), self.rows_main)

    def run(self, Y, ops, skip_main=False):
        """RowEngine.run (fastops.py:156-167) on device rows Y (B, 2L, N), in place. Dense rows take the exact
        filter (fastops.py:100-117), fused with the butterflies around it (adjoint levels before, Gram levels and
        the level-1 butterflies of the hybrid around it) into one precomputed operator per row; with compensated
        high rows (plan.high_rows == "ff") they keep the polynomial filter in float-float arithmetic instead.
        skip_main: the polynomial rows (main_job) were run by the caller; only the rest is done here."""
        ops = fuse_ops(ops)
        B = Y.shape[0]
        if not ops:
            return
        st = C.stream_handle()
        pidx = [i for i, o in enumerate(ops) if o[0] == "P"]
        if len(pidx) > 1:
            raise ValueError("at most one filter op per list")
        dense = len(self.plan.dense_freqs) > 0
        if skip_main and (not dense or not pidx):
            if dense:  # no filter: the dense rows take the op list like the others
                C.call("adrt_rows_run", ctypes.byref(self.job(Y, ops, self.rows_dense)), st)
            self.count += B * self.plan.level_rows(ops_unfused(ops))
            return
        if dense and self.high_poly:
            if self.high_ff:
                if not skip_main:
                    self._timed_main(Y, ops, st)
                self.run_ff(Y, ops)
            else:
                rows = self.rows_dense if skip_main else torch.cat([self.rows_main, self.rows_dense])
                C.call("adrt_rows_run", ctypes.byref(self.job(Y, ops, rows)), st)
            self.count += B * self.plan.level_rows(ops_unfused(ops))
            return
        if not dense or not pidx:
            if dense:
                rows = torch.cat([self.rows_main, self.rows_dense])
                C.call("adrt_rows_run", ctypes.byref(self.job(Y, ops, rows)), st)
            else:
                self._timed_main(Y, ops, st)
        else:
            i = pidx[0]
            _, plo, phi = ops[i]
            pre, post = list(ops[:i]), list(ops[i + 1 :])
            fold_pre = bool(pre) and pre[-1] == ("BT", plo, phi)
            if fold_pre:
                pre = pre[:-1]
            fold_post = bool(post) and post[0] == ("M", plo, phi)
            if fold_post:
                post = post[1:]
            pre_b1 = pre == [("B", 1, 1)]
            post_b1t = post == [("BT", 1, 1)]
            if pre_b1:
                pre = []
            if post_b1t:
                post = []
            if not skip_main:
                self._timed_main(Y, ops, st)
            if pre:
                C.call("adrt_rows_run", ctypes.byref(self.job(Y, pre, self.rows_dense)), st)
            self.dense_apply(Y, self.dense_table(fold_pre, fold_post, pre_b1, post_b1t))
            if post:
                C.call("adrt_rows_run", ctypes.byref(self.job(Y, post, self.rows_dense)), st)
        self.count += B * self.plan.level_rows(ops_unfused(ops))


def _rows_apply_f64(X, z_rows, ops, n, counter):
    """The row ops on the K rows of X (K, N) complex128 in place (natural order in and out), row i at frequency
    z_rows[i] (complex128 on the device), through the library's FP64 row kernels with a per-row twiddle table."""
    K, N = X.shape
    st = C.stream_handle()
    tab = torch.empty((K, N // 2 + 1), dtype=torch.complex128, device=X.device)
    C.call("adrt_twiddle_table", C.dtype_code(torch.float64), n, K, C.ptr(z_rows), C.ptr(tab), st)
    j = C.RowJob()
    j.dtype, j.n, j.nimg, j.nsel, j.img_stride = C.dtype_code(torch.float64), n, 1, K, K * N
    j.X, j.rows, j.freq_mod, j.roots, j.twtab = X.data_ptr(), None, K, None, tab.data_ptr()
    j.deg, j.coef, j.coef_stride, j.tau = None, None, 0, 0.0
    j.nops = len(ops)
    for i, (op, lo, hi) in enumerate(ops):
        j.op[i], j.lo[i], j.hi[i] = OPCODE[op], lo, hi
    j.counter, j.grid = counter.data_ptr(), 0
    C.call("adrt_rows_run", ctypes.byref(j), st)


def _load_torch_linalg():
    """torch opens its CUDA linear-algebra library lazily by file name; where a profiler's library injection changes
    the search path that lookup fails, so the library is loaded once by its full path first."""
    import os

    p = os.path.join(os.path.dirname(torch.__file__), "lib", "libtorch_cuda_linalg.so")
    if os.path.exists(p):
        ctypes.CDLL(p, mode=ctypes.RTLD_GLOBAL)


def dense_row_operator_device(plan: Plan, fold_pre, fold_post, pre_b1, post_b1t, device, chunk=None):
    """Plan.dense_row_operator built on the device in FP64, in chunks of dense frequencies: yields (first index,
    (k, N, N) complex128). The Gram matrices M_k and every butterfly fold come from the library's own FP64 row
    kernels applied to unit vectors (O(n N^2) per frequency instead of a dense O(N^3) product):
        rows of M e_j          -> M^T = conj(M)                    (M Hermitian)
        T A^H,  row t          -> conj(A conj(t))                  (A = B_hi ... B_lo)
        T B_1,  row t          -> conj(B_1^* conj(t))
        B_1^* T                -> B_1^* applied to the columns of T
    and the filter itself from one Cholesky factorisation and inverse per frequency (torch, FP64):
        F = (M + tau I)^-1,   M F = I - tau F."""
    n, N, Kd, tau = plan.n, plan.N, len(plan.dense_freqs), plan.tau
    lo, hi = plan.p_levels
    dev = torch.device(device)
    if dev.type == "cuda":
        _load_torch_linalg()
    z = torch.from_numpy(roots_of_unity(plan.L)[plan.dense_freqs]).to(dev)
    if chunk is None:
        chunk = max(1, min(Kd, (1 << 29) // (N * N * 16)))  # about 512 MB per (k, N, N) block
    eye = torch.eye(N, dtype=torch.complex128, device=dev)
    counter = torch.zeros(4, dtype=torch.int32, device=dev)
    for c0 in range(0, Kd, chunk):
        zc = z[c0:c0 + chunk]
        k = zc.shape[0]
        zr = zc.repeat_interleave(N)
        # the kernels read raw memory: every conjugate handed to them is materialised (conj_physical, not the
        # lazy conjugate view)
        X = eye.expand(k, N, N).reshape(k * N, N).clone()
        _rows_apply_f64(X, zr, [("M", lo, hi)], n, counter)
        Mk = torch.conj_physical(X.view(k, N, N))
        Mk.diagonal(dim1=-2, dim2=-1).add_(tau)
        F = torch.cholesky_inverse(torch.linalg.cholesky(Mk))
        del Mk, X
        T = eye - tau * F if fold_post else F
        if fold_pre:
            X = torch.conj_physical(T).reshape(k * N, N).contiguous()
            _rows_apply_f64(X, zr, [("B", lo, hi)], n, counter)
            T = torch.conj_physical(X.view(k, N, N))
        if pre_b1:
            X = torch.conj_physical(T).reshape(k * N, N).contiguous()
            _rows_apply_f64(X, zr, [("BT", 1, 1)], n, counter)
            T = torch.conj_physical(X.view(k, N, N))
        if post_b1t:
            X = T.transpose(-1, -2).reshape(k * N, N).contiguous()
            _rows_apply_f64(X, zr, [("BT", 1, 1)], n, counter)
            T = X.view(k, N, N).transpose(-1, -2)
        yield c0, T


def ops_unfused(ops):
    out = []
    for op, lo, hi in ops:
        if op == "M":
            out += [("B", lo, hi), ("BT", lo, hi)]
        else:
            out.append((op, lo, hi))
    return out


class Pipeline:
    """Every device buffer for one (plan, batch size, precision)."""

    def __init__(self, plan: Plan, batch, precision="fp32", device="cuda", stencil_precision=None, state="auto"):
        if precision not in PRECISIONS:
            raise ValueError(f"precision must be one of {tuple(PRECISIONS)}")
        C.load()
        self.plan, self.B, self.precision = plan, int(batch), precision
        self.device = torch.device(device)
        self.real = PRECISIONS[precision]
        self.outer_real = torch.float64
        self.stencil_precision = stencil_precision or precision
        if self.stencil_precision not in STENCIL_PRECISIONS:
            raise ValueError(f"stencil_precision must be one of {tuple(STENCIL_PRECISIONS)}")
        self.stencil_real = STENCIL_PRECISIONS[self.stencil_precision]
        self.stencil_code = STENCIL_CODES[self.stencil_precision]
        self.tables = RowTables(plan, self.real, self.device)
        self.tables.stream_dense = self.real == torch.float32 and self.B <= 16
        N, L, B = plan.N, plan.L, self.B
        dev = self.device
        self.Y = torch.empty((B, 2 * L, N), dtype=_cdtype(self.real), device=dev)
        self.parts = torch.empty((3, B, N, N), dtype=self.real, device=dev)
        # the outer state: FP64 images, or (where the register-resident fused outer step runs: FP32 rows and
        # stencil, 64 <= N <= 512) float-float planes (B, 2, N, N), hi then lo per image, with y in FP32 (it is an
        # FP32 sum of the partial images either way) and the FP64 result converted once at the end of an apply
        if state not in ("auto", "fp64"):
            raise ValueError("state must be 'auto' (float-float where the register-resident outer step runs) or 'fp64'")
        self.ff_state = state == "auto" and Pipeline.ff_state_for(plan, precision, self.stencil_precision)
        if self.ff_state:
            self.xs = [torch.empty((B, 2, N, N), dtype=torch.float32, device=dev) for _ in range(3)]
            self.y = torch.empty((B, N, N), dtype=torch.float32, device=dev)
            self.x64 = torch.empty((B, N, N), dtype=torch.float64, device=dev)
        else:
            self.xs = [torch.empty((B, N, N), dtype=self.outer_real, device=dev) for _ in range(3)]
            self.y = torch.empty((B, N, N), dtype=self.outer_real, device=dev)
            self.x64 = None
        self.s = torch.empty((B, N, N), dtype=self.stencil_real, device=dev)
        self.st = [torch.empty((B, N, N), dtype=self.stencil_real, device=dev) for _ in range(3)]
        self.ops = _op_lists(plan)
        self.launches = 0
        self.timer = None  # list: when set, ("pack_image" | "pack_sino" | "unpack", start, end) CUDA events per launch
        self.band = 0  # rows per CTA of the fused outer step (0: from the batch); set by the autotuner
        self.fft_cols = 0  # strip columns per CTA of the offset FFTs (0: the default); set by the autotuner

    def prefix(self, b):
        """A pipeline over the first b images of this one's buffers (views of the same memory; same plan, precision
        and kernel choices, its own row-table state and dense-row staging): steps over a prefix of the batch cost in
        proportion to b."""
        b = int(b)
        if not 1 <= b <= self.B:
            raise ValueError("prefix size out of range")
        q = object.__new__(Pipeline)
        q.__dict__.update(self.__dict__)
        q.B = b
        t = RowTables(self.plan, self.real, self.device)
        for k in ("stream_dense", "use_tc", "split_dense", "row_grid", "dense_tile"):
            setattr(t, k, getattr(self.tables, k))
        q.tables = t
        q.Y = self.Y[:b]
        q.parts = self.parts[:, :b]
        q.xs = [x[:b] for x in self.xs]
        q.y = self.y[:b]
        q.x64 = None if self.x64 is None else self.x64[:b]
        q.s = self.s[:b]
        q.st = [x[:b] for x in self.st]
        q.timer = None
        return q

    # ---------------------------------------------------------------- packed passes
    def _codes(self):
        return C.dtype_code(self.real)

    def _timed(self, name, fn):
        if self.timer is None:
            fn()
            return
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        self.timer.append((name, e0, e1))

    def packed_image(self, x, ops):
        """fastops._packed with strips Tq(q, E x): x (B, N, N) real, or float-float planes (B, 2, N, N), on device
        -> self.parts."""
        st = C.stream_handle()
        self._timed("pack_image", lambda: self.pack(x, sino=False))
        self.tables.run(self.Y, ops)
        self._unpack(st)
        return self.parts

    def packed_sino(self, b, ops):
        """fastops._packed with strips iota(b_q): b (B, 4, 2N-1, N) real on device -> self.parts."""
        self.pack(b, sino=True)
        self.tables.run(self.Y, ops)
        self._unpack(C.stream_handle())
        return self.parts

    def _unpack(self, st):
        self._timed("unpack", lambda: C.call("adrt_ifft_unpack", self._codes(), self.plan.n, self.B, C.ptr(self.Y),
                                             C.ptr(self.parts[0]), C.ptr(self.parts[1]), C.ptr(self.parts[2]),
                                             C.ptr(self.tables.roots), self.fft_cols, st))

    def sum_parts(self, out):
        C.call("adrt_sum3", self._codes(), self.plan.n, self.B, C.ptr(self.parts[0]), C.ptr(self.parts[1]),
               C.ptr(self.parts[2]), C.ptr(out), C.dtype_code(out.dtype), C.stream_handle())
        return out

    # ---------------------------------------------------------------- image-space steps
    def resid(self, y, with_parts=True):
        """s = y - (sum of the partial images) in the stencil precision (parts omitted: a cast of y)."""
        p0, p1, p2 = (self.parts[0], self.parts[1], self.parts[2]) if with_parts else (None, None, None)
        C.call("adrt_resid", C.dtype_code(self.s.dtype), self.plan.n, self.B, C.dtype_code(y.dtype), C.ptr(y),
               C.ptr(p0), C.ptr(p1), C.ptr(p2), C.ptr(self.s), C.stream_handle())
        return self.s

    def precond(self, s):
        """Hybrid preconditioner P applied to s (fasthybrid.py:224-229): g1_inv (Chebyshev on [4, 16] of the G_1
        stencil), lorr_inv, or the identity."""
        p, st = self.plan, C.stream_handle()
        code = C.dtype_code(s.dtype)
        if p.precond == "none":
            return s
        if p.precond == "lorr":
            out = self.st[0]
            C.call("adrt_lorr", code, p.n, self.B, C.ptr(s), C.ptr(out), st)
            return out
        a, c, steps = outer_coeffs(4.0, 16.0, p.g1_deg)
        bufs = self.st
        C.call("adrt_g1_step", code, p.n, self.B, C.ptr(s), None, None, C.ptr(bufs[0]), 0.0, 0.0, a, st)
        cur, prev = 0, None
        for om_a, om_1 in steps:
            nxt = 1 if cur != 1 and prev != 1 else (2 if cur != 2 and prev != 2 else 0)
            C.call("adrt_g1_step", code, p.n, self.B, C.ptr(s), C.ptr(bufs[cur]),
                   None if prev is None else C.ptr(bufs[prev]), C.ptr(bufs[nxt]), om_a, om_1, 0.0, st)
            prev, cur = cur, nxt
        return bufs[cur]

    def fused_outer_ok(self):
        """The fused outer step exists for this size and pairing (FP32 rows with any stencil precision, FP64 rows
        with the FP64 stencil)."""
        pair = self.real == torch.float32 or self.stencil_precision == "fp64"
        return pair and self.plan.n <= C.load().adrt_outer_step_max_n(self.stencil_code)

    def fused_outer_step(self, y, with_parts, x, x_prev, x_new, om_a, om_1, a0, om_img=None):
        """Residual + preconditioner + outer update in one clustered kernel (adrt_outer_step, or adrt_outer_step_ff
        when x_new is a float-float state (B, 2, N, N)); om_img (device (B, 2) FP64, optional): per-image
        (om_a, om_1)."""
        p = self.plan
        pc = {"none": 0, "g1": 1, "lorr": 2}[p.precond] if p.method == "hybrid" else 0
        if pc == 1:
            ga, _, gsteps = outer_coeffs(4.0, 16.0, p.g1_deg)
            coef = np.array([ga] + [v for st in gsteps for v in st], dtype=np.float64)
        else:
            coef = np.zeros(1)
        parts = (self.parts[0], self.parts[1], self.parts[2]) if with_parts else (None, None, None)
        if x_new.dim() == 4:
            C.call("adrt_outer_step_ff", p.n, self.B, C.ptr(y), C.ptr(parts[0]), C.ptr(parts[1]), C.ptr(parts[2]),
                   C.ptr(x), C.ptr(x_prev), C.ptr(x_new), om_a, om_1, a0, pc, p.g1_deg if pc == 1 else 0,
                   coef.ctypes.data_as(ctypes.c_void_p), C.ptr(om_img), self.band & 0xFF, C.stream_handle())
            return
        C.call("adrt_outer_step", self.stencil_code, self._codes(), p.n, self.B, C.ptr(y), C.ptr(parts[0]),
               C.ptr(parts[1]), C.ptr(parts[2]), C.ptr(x), C.ptr(x_prev), C.ptr(x_new), om_a, om_1, a0, pc,
               p.g1_deg if pc == 1 else 0, coef.ctypes.data_as(ctypes.c_void_p), C.ptr(om_img), self.band,
               C.stream_handle())

    def outer_step(self, x, x_prev, r, x_new, om_a, om_1, a0, om_img=None):
        """x_new = x + om_a r + om_1 (x - x_prev) (x None: a0 r); om_img (device (B, 2) FP64, optional): per-image
        (om_a, om_1)."""
        C.call("adrt_outer_update", C.dtype_code(x_new.dtype), self.plan.n, self.B, C.ptr(x), C.ptr(x_prev), C.ptr(r),
               C.dtype_code(r.dtype), C.ptr(x_new), om_a, om_1, a0, C.ptr(om_img), C.stream_handle())

    def step_all(self, y, x, x_prev, x_new, om_img):
        """One outer step of every image with per-image coefficients (x_new = x + om_a P(y - G x) + om_1 (x - x_prev)
        with G x already in the partial images): the fused kernel where it exists, else the separate kernels."""
        if self.fused_outer_ok():
            self.fused_outer_step(y, True, x, x_prev, x_new, 0.0, 0.0, 0.0, om_img=om_img)
            return
        s = self.resid(y)
        r = self.precond(s) if self.plan.method == "hybrid" else s
        self.outer_step(x, x_prev, r, x_new, 0.0, 0.0, 0.0, om_img=om_img)

    # ---------------------------------------------------------------- operators
    def G(self, x):
        """The frame operator (L_p: frame_window, fastops.py:277-281) or G_h (hybrid, fastops.py:325-331) of x."""
        return self.packed_image(x, self.ops["G"])

    def backproject_into(self, b, y):
        self.packed_sino(b, self.ops["BP"])
        return self.sum_parts(y)

    # ---------------------------------------------------------------- CUDA graph of a whole apply
    def device_bytes(self):
        """Device memory held by this pipeline (buffers and tables)."""
        t = self.tables
        bufs = [self.Y, self.parts, self.y, self.s, *self.xs, *self.st, t.roots, t.deg, t.coef, t.rows_main,
                t.rows_dense, *t._dense_dev.values()]
        if self.x64 is not None:
            bufs.append(self.x64)
        bufs += [T._adrt_split for T in t._dense_dev.values() if getattr(T, "_adrt_split", None) is not None]
        if t.high_ff:
            bufs += [t.roots64, t.coef64]
        if t._zd is not None:
            bufs.append(t._zd)
        for name in ("b_in", "b_in2"):
            if getattr(self, name, None) is not None:
                bufs.append(getattr(self, name))
        return sum(x.numel() * x.element_size() for x in bufs)

    @staticmethod
    def ff_state_for(plan: Plan, precision="fp32", stencil_precision=None):
        """Whether a pipeline keeps its outer state as float-float planes: where the register-resident fused outer
        step runs (FP32 rows and stencil, 64 <= N <= 512)."""
        return precision == "fp32" and (stencil_precision or precision) == "fp32" and 6 <= plan.n <= 9

    @staticmethod
    def estimate_bytes(plan: Plan, batch, precision="fp32", stencil_precision=None, captured=True):
        """Device bytes a pipeline for (plan, batch, precision) holds once it has run apply (and capture, which adds
        the two input buffers): the buffers of __init__, the two folded dense-row tables (filter of G and of the
        backprojection) and the dense-row staging, computed without allocating anything."""
        N, L, B = plan.N, plan.L, int(batch)
        rs = PRECISIONS[precision].itemsize
        ss = STENCIL_PRECISIONS[stencil_precision or precision].itemsize
        nd = 2 * len(plan.dense_freqs)
        ff = getattr(plan, "high_rows", "dense") == "ff" and nd > 0
        img = B * N * N
        # y and three outer states: FP64, or FP32 y, float-float states and the FP64 result buffer
        state = 36 * img if Pipeline.ff_state_for(plan, precision, stencil_precision) else 32 * img
        total = B * 2 * L * N * 2 * rs + 3 * img * rs + state + 4 * img * ss
        if ff:  # FP64 roots and coefficients of the compensated rows instead of dense operators
            total += L * 16 + plan.coef.size * 8
        else:
            total += 2 * nd * N * N * 2 * rs + nd * B * N * 2 * rs
            if precision == "fp32" and B > 16 and 7 <= plan.n <= 10:  # their pre-split tensor-core form (in place)
                total += 2 * nd * N * N * 16 - nd * B * N * 2 * rs
        total += L * 2 * rs + 3 * L * 4 + plan.coef.size * rs  # roots; deg and the row lists; coefficients
        if captured:  # the two input buffers of the captured graphs
            total += 2 * B * 4 * (2 * N - 1) * N * 8
        return int(total)

    def capture(self):
        """Record apply() on a private input buffer into a CUDA graph (after one eager warm-up run, so that every
        lazily built table and kernel attribute exists). replay(b) then copies b in and replays the graph."""
        N = self.plan.N
        self.b_in = torch.zeros((self.B, 4, 2 * N - 1, N), dtype=torch.float64, device=self.device)
        side = torch.cuda.Stream(device=self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(side):
            self.apply(self.b_in)
            side.synchronize()
            self.graph = torch.cuda.CUDAGraph()
            before = self.tables.count
            with graph_capture(self.graph, side):
                self.x_out = self.apply(self.b_in)
            self.graph_count = self.tables.count - before  # level-rows of one replay
            # a second graph on a second input buffer: host batches alternate between the two, so that the copy of
            # the next batch (on its own stream) overlaps the graph of the current one
            self.b_in2 = torch.zeros_like(self.b_in)
            self.graph2 = torch.cuda.CUDAGraph()
            with graph_capture(self.graph2, side):
                x2 = self.apply(self.b_in2)
            self.tables.count -= self.graph_count
            assert x2.data_ptr() == self.x_out.data_ptr()
        torch.cuda.current_stream(self.device).wait_stream(side)
        self.copy_stream = torch.cuda.Stream(device=self.device)
        self._flip = 0
        self._free = [None, None]  # per input buffer: the event after the graph that last read it
        self._err_host = torch.zeros(1, dtype=torch.int32, pin_memory=True)
        self._err_event = None  # the previous host-side replay's error-flag copy
        return self

    def replay(self, b=None):
        """Run the captured apply on the current stream (b copied into the graph's input buffer first; a host tensor
        is copied straight from host memory)."""
        if b is not None:
            self.b_in.copy_(b, non_blocking=True)
        self.graph.replay()
        self.tables.count += self.graph_count
        return self.x_out

    def replay_host(self, b, out):
        """Host batch in, host result out, pipelined across calls: b is copied into one of the two input buffers on
        the copy stream (waiting only for the graph that last read that buffer), the matching graph replays on the
        current stream once the copy is done, and the result and the dense kernel's error flag are copied back
        without a host synchronisation. The error flag of the PREVIOUS host replay is checked here, after the
        copy is queued (so that copy still overlaps the previous graph); check_host() checks the last one."""
        i = self._flip
        self._flip ^= 1
        buf, graph = (self.b_in, self.graph) if i == 0 else (self.b_in2, self.graph2)
        cur = torch.cuda.current_stream(self.device)
        cs = self.copy_stream
        if self._free[i] is not None:
            cs.wait_event(self._free[i])
        with torch.cuda.stream(cs):
            buf.copy_(b, non_blocking=True)
        copied = torch.cuda.Event()
        copied.record(cs)
        self.check_host()
        cur.wait_event(copied)
        graph.replay()
        self.tables.count += self.graph_count
        free = torch.cuda.Event()
        free.record(cur)
        self._free[i] = free
        out.copy_(self.x_out, non_blocking=True)
        self._err_host.copy_(self.tables.err, non_blocking=True)
        self.tables.err.zero_()
        self._err_event = torch.cuda.Event()
        self._err_event.record(cur)
        return out

    def check_host(self):
        """Raise if the last replay_host's dense-row launch gave up on a bounded wait (waits for that replay)."""
        ev, self._err_event = getattr(self, "_err_event", None), None
        if ev is None:
            return
        ev.synchronize()
        code = int(self._err_host.item())
        if code:
            raise RuntimeError("dense_tc_kernel: an mbarrier wait ran out; the dense-row results of the previous "
                               "batch were not written" + ("" if code == 1 else " (and the MMA drain ran out)"))

    def first_step(self, y, x_out, a):
        """x_1 = a P(y) (P = identity for L_p): the outer iteration's first step (fastops.py:250)."""
        if self.fused_outer_ok():
            self.fused_outer_step(y, False, None, None, x_out, 0.0, 0.0, a)
        elif self.plan.method == "hybrid":
            r = self.precond(self.resid(y, with_parts=False))
            self.outer_step(None, None, r, x_out, 0.0, 0.0, a)
        else:
            self.outer_step(None, None, y, x_out, 0.0, 0.0, a)

    def next_step(self, y, x, x_prev, x_new, om_a, om_1):
        """x_new = x + om_a P(y - G x) + om_1 (x - x_prev), with G x already in the partial images
        (fastops.py:252-257)."""
        if self.fused_outer_ok():
            self.fused_outer_step(y, True, x, x_prev, x_new, om_a, om_1, 0.0)
        else:
            s = self.resid(y)
            r = self.precond(s) if self.plan.method == "hybrid" else s
            self.outer_step(x, x_prev, r, x_new, om_a, om_1, 0.0)

    def apply(self, b):
        """x = L b for B sinograms b (B, 4, 2N-1, N) on device; returns the FP64 (B, N, N) result buffer (a view
        of internal storage, valid until the next call)."""
        p = self.plan
        if p.lo is None:
            raise RuntimeError("plan has no outer interval")
        a, c, steps = outer_coeffs(p.lo, p.hi, p.outer_deg)
        y = self.backproject_into(b, self.y)
        x, xp = self.xs[0], None
        self.first_step(y, x, a)
        free = [self.xs[1], self.xs[2]]
        for om_a, om_1 in steps:
            self.G(x)
            xn = free.pop(0)
            self.next_step(y, x, xp, xn, om_a, om_1)
            if xp is not None:
                free.append(xp)
            xp, x = x, xn
        return self.result(x)

    def result(self, x, out=None):
        """The FP64 images of an outer state: x itself (FP64 state), or hi + lo of float-float planes converted into
        out (default: this pipeline's result buffer, rows matching x's)."""
        if x.dim() == 3:
            return x
        if out is None:
            out = self.x64[:x.shape[0]]
        C.call("adrt_ff_to_f64", self.plan.n, x.shape[0], C.ptr(x), C.ptr(out), C.stream_handle())
        return out

    # ---------------------------------------------------------------- the stages around the row engine
    def pack(self, src, sino):
        """The pack + FFT kernel of one packed pass: sinograms (B, 4, 2N-1, N), images (B, N, N) or float-float
        images (B, 2, N, N) -> Y. Of a float-float image only the hi plane is read: the FFT runs in FP32, and the
        FP32 rounding of hi + lo is hi."""
        p, st = self.plan, C.stream_handle()
        stride = 0
        if not sino and src.dim() == 4:
            if src.shape[1] != 2 or src.dtype != torch.float32 or not src.is_contiguous():
                raise ValueError("float-float images are contiguous (B, 2, N, N) FP32")
            stride = 2 * p.N * p.N
        C.call("adrt_pack_fft", self._codes(), p.n, self.B, 1 if sino else 0, C.dtype_code(src.dtype), C.ptr(src),
               stride, C.ptr(self.Y), C.ptr(self.tables.roots), self.fft_cols, st)

    def finish_pass(self, ops):
        """Everything of a packed pass after the polynomial-row launch: the dense (or compensated) rows, the inverse
        FFT and the unpack into the partial images."""
        self.tables.run(self.Y, ops, skip_main=True)
        self._unpack(C.stream_handle())


def _op_lists(plan):
    n = plan.n
    if plan.method == "lp":  # fastops.py:277-285
        return {"G": [("P", 1, n), ("B", 1, n), ("BT", 1, n)], "BP": [("BT", 1, n), ("P", 1, n)]}
    return {  # fastops.py:325-335
        "G": [("B", 1, 1), ("P", 2, n), ("B", 2, n), ("BT", 2, n), ("BT", 1, 1)],
        "BP": [("BT", 2, n), ("P", 2, n), ("BT", 1, 1)],
    }
