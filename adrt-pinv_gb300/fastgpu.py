"""Drop-in for the reference's `fastcpp` module (fastcpp.py) on the GPU.

* `lib()` returns the ctypes library whose `bfly_rows`, `cheb_rows`, `cert_rowsum`, `omp_max_threads` have the
  signatures of cpp/oblique.cpp (host pointers; the library copies to the GPU and back), bound exactly as
  fastcpp.py:22-32 binds the reference's library; `_ptr` as fastcpp.py:45-46.
* `GpuEngine` (alias `CppEngine`) is a RowEngine for the `engine_cls` seam of fastops._Base (fastops.py:177): the
  reference's own FastLp / FastHybrid run unchanged with their row ops on the GPU.
* `FastLpCpp` / `FastHybridCpp` are the full-device inverses (inverse.FastLpGpu / FastHybridGpu).
* `power_lam_max`, `cert_lam_max`, `explicit_lam_max` as fastcpp.py:102-134.
"""

import ctypes

import numpy as np
import torch

from . import _lib as C
from .device import RowTables
from .inverse import FastHybridGpu, FastLpGpu, cert_lam_max, explicit_lam_max
from .inverse import power_lam_max as _power
from .plan import Plan, roots_of_unity


def lib():
    """The C ABI library (fastcpp.lib, fastcpp.py:38-42)."""
    return C.load()


def _ptr(x):
    return x.ctypes.data_as(ctypes.c_void_p)


def power_lam_max(n, z, m_lo, iters=40, safety=1.5, threads=1):
    """fastcpp.power_lam_max (fastcpp.py:102-118) for the standard frequencies z = exp(2 pi i fftfreq(2N))."""
    del threads
    L = 2 << n
    if len(z) != L or not np.allclose(np.asarray(z), roots_of_unity(L), atol=1e-12):
        raise ValueError("power_lam_max: z must be the 2N offset frequencies exp(2 pi i fftfreq(2N))")
    return _power(n, m_lo, iters, safety)


class GpuEngine:
    """fastops.RowEngine interface (fastops.py:20-167) on the GPU: run(Y, ops) with Y (2L, N) complex NumPy rows
    (copies stacked) returns the transformed rows; `count` accumulates level-rows as the reference counts them."""

    def __init__(self, n, z, deg, lam_max, tau, threads=1, copies=2, dense_cap=None, p_levels=(1, None)):
        del threads
        if copies != 2:
            raise ValueError("GpuEngine supports the packed layout (copies=2)")
        L = len(z)
        if L != 2 << n or not np.allclose(np.asarray(z), roots_of_unity(L), atol=1e-12):
            raise ValueError("GpuEngine: z must be the 2N offset frequencies")
        method = "lp" if (p_levels[0] or 1) == 1 else "hybrid"
        self.n, self.N, self.R, self.tau = n, 1 << n, 2 * L, tau
        self.plan = Plan(method, n, np.asarray(lam_max, dtype=float), tau_fac=tau / (1 << n), deg=np.asarray(deg),
                         dense_cap=dense_cap, raw_lam=True)
        self.tables = RowTables(self.plan, torch.float64, torch.device("cuda"))
        self.n_dense = len(self.plan.dense_freqs)
        self.count = [0]

    def run(self, Y, ops):
        Yd = torch.from_numpy(np.ascontiguousarray(np.asarray(Y, dtype=complex))).to("cuda").unsqueeze(0)
        before = self.tables.count
        self.tables.run(Yd, list(ops))
        self.count[0] += self.tables.count - before
        return Yd[0].cpu().numpy()


CppEngine = GpuEngine
FastLpCpp = FastLpGpu
FastHybridCpp = FastHybridGpu

__all__ = ["lib", "_ptr", "power_lam_max", "cert_lam_max", "explicit_lam_max", "GpuEngine", "CppEngine",
           "FastLpCpp", "FastHybridCpp", "FastLpGpu", "FastHybridGpu"]
