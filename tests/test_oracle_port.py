"""The C restatement of the row kernels (oracle/oblique_port.c) against the NumPy oracle and, when it could be
built from the reference sources here, against the reference's own library (oracle/_ref/liboblique.so)."""

import ctypes
import os

import numpy as np
import pytest

from conftest import max_rel
from oracle import cpu_engine as C
from oracle import oblique_np as O


def _kinds():
    C.build()
    kinds = ["port"]
    if os.path.exists(C.REF_LIB):
        kinds.append("reference")
    return kinds


KINDS = _kinds()


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("n", [3, 6])
def test_bfly_rows(golden, kind, n):
    lib, _ = C.load(kind)
    N, L = 1 << n, 2 << n
    rng = np.random.default_rng(n)
    z = np.ascontiguousarray(O.offset_z(L))
    V = rng.standard_normal((L, N)) + 1j * rng.standard_normal((L, N))
    for lo, hi in ((1, n), (2, n), (1, 1), (3, n)):
        if lo > hi:
            continue
        for tr in (0, 1):
            X = V.copy()
            lib.bfly_rows(n, L, C._p(z), C._p(X), lo, hi, tr, 2)
            ref = O.bflyT_levels(n, z, V, lo, hi) if tr else O.bfly_levels(n, z, V, lo, hi)
            assert max_rel(X, ref) < 1e-13


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("lo", [1, 2])
def test_cheb_rows(golden, kind, lo):
    lib, _ = C.load(kind)
    n = 6
    N = 1 << n
    rows = golden[f"bf_rows_{n}"]
    z = np.ascontiguousarray(golden[f"bf_z_{n}"])
    Y = np.ascontiguousarray(golden[f"cheb_Y_{n}_{lo}"])
    K = len(rows)
    deg = np.ascontiguousarray(golden[f"cheb_deg_{n}_{lo}"], dtype=np.int32)
    c, a = O.cheb_coeffs(golden[f"cheb_lam_{n}_{lo}"], 0.2 * N)
    Z = np.empty_like(Y)
    steps = ctypes.c_longlong(5)
    lib.cheb_rows(n, K, C._p(z), C._p(deg), C._p(np.ascontiguousarray(a)), C._p(np.ascontiguousarray(c)), 0.2 * N,
                  C._p(Y), C._p(Z), lo, n, 3, ctypes.byref(steps))
    assert max_rel(Z, golden[f"cheb_Z_{n}_{lo}"]) < 1e-13
    assert steps.value == 5 + int(golden[f"cheb_steps_{n}_{lo}"])


@pytest.mark.parametrize("kind", KINDS)
def test_cert_rowsum(golden, kind):
    lib, _ = C.load(kind)
    for n in (4, 8):
        oms = np.ascontiguousarray(O.offset_freqs(2 << n))
        for lo in (1, 2):
            out = np.empty(len(oms))
            lib.cert_rowsum(n, len(oms), C._p(oms), lo, C._p(out), 2)
            assert max_rel(out, golden[f"cert_cpp_{n}_{lo}"]) < 1e-14
    assert lib.omp_max_threads() >= 1


@pytest.mark.parametrize("kind", KINDS)
def test_cpu_engine_inverses(golden, kind):
    n = 6
    x, b = golden[f"inv_x_{n}"], golden[f"inv_b_{n}"]
    for name, kw in (("hybd8", {"dense_cap": 8}), ("lp", {})):
        k = f"{name}_{n}"
        plan = dict(lam_max=golden[f"inv_lam_{k}"], outer=tuple(golden[f"inv_outer_{k}"]), **kw)
        P = (C.hybrid_cpu if name.startswith("hyb") else C.lp_cpu)(n, plan, threads=2, kind=kind)
        P.eng.count = [0]
        xr = P.apply(b)
        assert max_rel(xr, golden[f"inv_apply_{k}"]) < 1e-11
        assert P.eng.count[0] == int(golden[f"inv_count_{k}"])
        assert np.linalg.norm(xr - x) / np.linalg.norm(x) < 1e-9
