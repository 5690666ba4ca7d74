"""Oracle (timed CPU baseline and checker only): the reference's C++ engine path on the host cores.

Restates `fastcpp.CppEngine` (fastcpp.py:49-99) over the C row kernels: `_ref/liboblique.so` (the reference's own
cpp/oblique.cpp compiled by `oracle/Makefile`, kind "reference") when it exists, else `_build/liboblique_port.so`
(this directory's C restatement, kind "port"). FFTs, quadrant packing, the dense table, the G_1 stencil and the
outer iteration stay in NumPy exactly as in the reference (fastcpp.py:1-4). Plans are injected as for the
NumPy oracle, so the CPU baseline evaluates the same operator as the device.
"""

import ctypes
import os
import subprocess

import numpy as np

from . import oblique_np as O

HERE = os.path.dirname(os.path.abspath(__file__))
REF_LIB = os.path.join(HERE, "_ref", "liboblique.so")
PORT_LIB = os.path.join(HERE, "_build", "liboblique_port.so")

_libs = {}


def build():
    """Compile the port (and the reference library when its source is present)."""
    subprocess.check_call(["make", "-s", "-C", HERE, "all"])


def load(kind=None):
    """(ctypes library, kind). kind None picks "reference" when available, else "port"."""
    if kind is None:
        kind = "reference" if os.path.exists(REF_LIB) else "port"
    if kind in _libs:
        return _libs[kind], kind
    path = REF_LIB if kind == "reference" else PORT_LIB
    if not os.path.exists(path):
        build()
    lib = ctypes.CDLL(path)
    P, I = ctypes.c_void_p, ctypes.c_int
    lib.bfly_rows.argtypes = [I, I, P, P, I, I, I, I]
    lib.bfly_rows.restype = None
    lib.cheb_rows.argtypes = [I, I, P, P, P, P, ctypes.c_double, P, P, I, I, I, P]
    lib.cheb_rows.restype = None
    lib.cert_rowsum.argtypes = [I, I, P, I, P, I]
    lib.cert_rowsum.restype = None
    lib.omp_max_threads.restype = I
    _libs[kind] = lib
    return lib, kind


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class CRowEngine(O.RowEngineOracle):
    """RowEngineOracle with the row kernels in C (fastcpp.py:49-99): rows processed in descending-degree order
    (fastops.py:41-42), dense rows by matmul, the rest by cheb_rows; B / BT by bfly_rows in place."""

    def __init__(self, n, z, deg, lam_max, tau, copies=2, dense_cap=None, p_levels=(1, None), threads=1, kind=None,
                 dense=None):
        super().__init__(n, z, deg, lam_max, tau, copies, dense_cap, p_levels)
        if dense:
            self.dense = dict(dense)
            self.n_dense = len(self.dense)
        self.lib, self.kind = load(kind)
        self.threads = max(1, int(threads))
        self.order = np.argsort(-self.deg, kind="stable")
        zc = self.z[self.order]
        self.zc = np.ascontiguousarray(zc)
        self.dc = np.ascontiguousarray(self.deg[self.order], dtype=np.int32)
        c, a = O.cheb_coeffs(self.lam[self.order], tau)
        self.ac, self.cc = np.ascontiguousarray(a), np.ascontiguousarray(c)
        isd = np.array([(int(r) % self.L) in self.dense for r in self.order], dtype=bool)
        self.Kd = int(isd.sum())  # dense rows have the largest degrees, so they lead the order
        assert isd[: self.Kd].all()
        self.Fd = np.array([self.dense[int(r) % self.L] for r in self.order[: self.Kd]]) if self.Kd else None

    def run(self, Y, ops):
        X = np.ascontiguousarray(np.asarray(Y, dtype=complex)[self.order])
        K = X.shape[0]
        for op, lo, hi in ops:
            if op in ("B", "BT"):
                self.lib.bfly_rows(self.n, K, _p(self.zc), _p(X), lo, hi, 1 if op == "BT" else 0, self.threads)
                self.count[0] += K * (hi - lo + 1)
            elif op == "P":
                Z = np.empty_like(X)
                if self.Kd:
                    Z[: self.Kd] = np.matmul(self.Fd, X[: self.Kd, :, None])[:, :, 0]
                steps = ctypes.c_longlong(0)
                Kr = K - self.Kd
                if Kr:
                    Zr = np.empty((Kr, self.N), dtype=complex)
                    s = slice(self.Kd, K)
                    self.lib.cheb_rows(self.n, Kr, _p(self.zc[s].copy()), _p(self.dc[s].copy()), _p(self.ac[s].copy()),
                                       _p(self.cc[s].copy()), self.tau, _p(np.ascontiguousarray(X[s])), _p(Zr), lo, hi,
                                       self.threads, ctypes.byref(steps))
                    Z[s] = Zr
                X = Z
                self.count[0] += steps.value + self.Kd * self.N // max(1, self.n)
            else:
                raise ValueError(op)
        out = np.empty_like(X)
        out[self.order] = X
        return out


def _with_c_engine(obj, threads, kind):
    """Swap the NumPy row engine of an oracle inverse for the C one, reusing its dense tables."""
    obj.eng = CRowEngine(obj.n, obj.z, obj.deg, obj.lam_max, obj.tau, 2, None, obj.p_levels, threads, kind,
                         dense=obj.eng.dense)
    return obj


def hybrid_cpu(n, plan_kw, threads=1, kind=None):
    """HybridOracle (fastops.FastHybrid semantics) with the C row kernels: the FastHybridCpp path."""
    P = O.HybridOracle(n, **plan_kw)
    return _with_c_engine(P, threads, kind)


def lp_cpu(n, plan_kw, threads=1, kind=None):
    """LpOracle with the C row kernels: the FastLpCpp path."""
    P = O.LpOracle(n, **plan_kw)
    return _with_c_engine(P, threads, kind)
