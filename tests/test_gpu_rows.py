"""GPU row kernels through the C ABI against the reference's own outputs (golden vectors from cpp/oblique.cpp and
fastspec / fasthybrid) and against the CPU oracle. FP64: <= 1e-12 relative (max-norm); FP32: <= 2e-6."""

import ctypes

import numpy as np
import pytest

from conftest import max_rel
from oracle import oblique_np as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib(pkg):
    import __graft_entry__ as ge

    ge.build()
    return pkg._lib.load()


def p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


@pytest.mark.parametrize("n", [4, 6])
def test_bfly_rows_dropin_matches_reference(lib, golden, n):
    V = golden[f"bf_V_{n}"]
    z = np.ascontiguousarray(golden[f"bf_z_{n}"])
    K = V.shape[0]
    for lo, hi in ((1, n), (2, n), (1, 1), (2, n - 1), (3, n)):
        for tr in (0, 1):
            X = V.copy()
            assert lib.bfly_rows(n, K, p(z), p(X), lo, hi, tr, 8) == 0, lib.adrt_last_error()
            assert max_rel(X, golden[f"cpp_bfly_{n}_{lo}_{hi}_{tr}"]) < 1e-12, (lo, hi, tr)


@pytest.mark.parametrize("n", [4, 6])
@pytest.mark.parametrize("lo", [1, 2])
def test_cheb_rows_dropin_matches_reference(lib, golden, n, lo):
    N = 1 << n
    z = np.ascontiguousarray(golden[f"bf_z_{n}"])
    Y = np.ascontiguousarray(golden[f"cheb_Y_{n}_{lo}"])
    K = Y.shape[0]
    deg = np.ascontiguousarray(golden[f"cheb_deg_{n}_{lo}"], dtype=np.int32)
    c, a = O.cheb_coeffs(golden[f"cheb_lam_{n}_{lo}"], 0.2 * N)
    a, c = np.ascontiguousarray(a), np.ascontiguousarray(c)
    Z = np.empty_like(Y)
    steps = ctypes.c_longlong(7)
    rc = lib.cheb_rows(n, K, p(z), p(deg), p(a), p(c), 0.2 * N, p(Y), p(Z), lo, n, 8, ctypes.byref(steps))
    assert rc == 0, lib.adrt_last_error()
    assert max_rel(Z, golden[f"cheb_Z_{n}_{lo}"]) < 1e-12
    assert steps.value == 7 + int(golden[f"cheb_steps_{n}_{lo}"])


def test_cert_rowsum_dropin_matches_reference(lib, golden):
    for n in (4, 6, 8):
        oms = np.ascontiguousarray(O.offset_freqs(2 << n))
        for lo in (1, 2):
            out = np.empty(len(oms))
            assert lib.cert_rowsum(n, len(oms), p(oms), lo, p(out), 1) == 0
            assert max_rel(out, golden[f"cert_cpp_{n}_{lo}"]) < 1e-12
    assert lib.omp_max_threads() > 0


@pytest.mark.parametrize("n", [7, 8, 9])
def test_bfly_rows_fp64_larger_n(lib, n):
    N, L = 1 << n, 2 << n
    rng = np.random.default_rng(n)
    z = np.ascontiguousarray(O.offset_z(L))
    V = rng.standard_normal((L, N)) + 1j * rng.standard_normal((L, N))
    for lo, hi, tr in ((1, n, 0), (2, n, 1), (1, n, 1), (2, n - 2, 0)):
        X = V.copy()
        assert lib.bfly_rows(n, L, p(z), p(X), lo, hi, tr, 1) == 0
        ref = O.bflyT_levels(n, z, V, lo, hi) if tr else O.bfly_levels(n, z, V, lo, hi)
        assert max_rel(X, ref) < 1e-12


PACKED = {
    "lp": lambda n: ([("P", 1, n), ("B", 1, n), ("BT", 1, n)], [("BT", 1, n), ("P", 1, n)]),
    "hyb": lambda n: ([("B", 1, 1), ("P", 2, n), ("B", 2, n), ("BT", 2, n), ("BT", 1, 1)],
                      [("BT", 2, n), ("P", 2, n), ("BT", 1, 1)]),
}


@pytest.mark.parametrize("name,dense_cap", [("lp", None), ("hyb", None), ("hyb", 8), ("lp", 8)])
def test_gpu_engine_seam_fp64(pkg, golden, name, dense_cap):
    """GpuEngine (the engine_cls seam, fastops.py:177) against the oracle RowEngine on the packed op lists."""
    n = 6
    N, L = 1 << n, 2 << n
    k = f"{name}_{n}"
    plan = pkg.Plan("lp" if name == "lp" else "hybrid", n, golden[f"inv_lam_{k}"])
    p_levels = (1, None) if name == "lp" else (2, None)
    eng = pkg.fastgpu.GpuEngine(n, O.offset_z(L), plan.deg, plan.lam_max, plan.tau, 8, 2, dense_cap, p_levels)
    ref = O.RowEngineOracle(n, O.offset_z(L), plan.deg, plan.lam_max, plan.tau, 2, dense_cap, p_levels)
    assert eng.n_dense == ref.n_dense
    rng = np.random.default_rng(11)
    Y = rng.standard_normal((2 * L, N)) + 1j * rng.standard_normal((2 * L, N))
    for ops in PACKED[name](n):
        out = eng.run(Y, ops)
        exp = ref.run(Y, ops)
        assert max_rel(out, exp) < 1e-12, ops
    assert eng.count[0] == ref.count[0]


@pytest.mark.parametrize("n,tol", [(5, 2e-6), (8, 1e-5)])
def test_device_rows_fp32(pkg, n, tol):
    """FP32 device rows (FP64-rounded tables) against the FP64 oracle on the hybrid G_h op list. The FP32 error
    grows with the condition (Lambda + tau)/tau of the low-frequency rows: a complex64 NumPy evaluation of the
    same op list gives 4e-6 at n=8."""
    import torch

    N, L = 1 << n, 2 << n
    lam = O.power_lam_max(n, O.offset_z(L), 2, iters=10)
    plan = pkg.Plan("hybrid", n, lam, deg_cap=32)
    tabs = pkg.device.RowTables(plan, torch.float32, torch.device("cuda"))
    rng = np.random.default_rng(5)
    Y = rng.standard_normal((2 * L, N)) + 1j * rng.standard_normal((2 * L, N))
    ops = PACKED["hyb"](n)[0]
    Yd = torch.from_numpy(Y).to("cuda", torch.complex64).unsqueeze(0).contiguous()
    tabs.run(Yd, ops)
    out = Yd[0].cpu().numpy()
    ref = O.RowEngineOracle(n, O.offset_z(L), plan.deg, plan.lam_max, plan.tau, 2, None, (2, None)).run(Y, ops)
    assert max_rel(out, ref) < tol


@pytest.mark.parametrize("n", [9, 10, 11])
@pytest.mark.parametrize("name", ["lp", "hyb"])
def test_device_programs_fp32_large_n(pkg, name, n):
    """The compile-time row programs at n = 9..11 (16 values per lane, rows over 1, 2, 4 warps, index bits 4..n-5 as
    warp-shuffle levels, named barriers per row group) on all four packed op lists against the FP64 oracle. Degrees
    capped at 6 keep the polynomial's FP32 error amplification small, so the tolerance checks the index arithmetic
    rather than the conditioning."""
    import torch

    N, L = 1 << n, 2 << n
    nimg = 2 if n < 11 else 1
    lo = 1 if name == "lp" else 2
    lam = O.power_lam_max(n, O.offset_z(L), lo, iters=10)
    plan = pkg.Plan("lp" if name == "lp" else "hybrid", n, lam, deg_cap=6)
    tabs = pkg.device.RowTables(plan, torch.float32, torch.device("cuda"))
    ref_eng = O.RowEngineOracle(n, O.offset_z(L), plan.deg, plan.lam_max, plan.tau, 2, None, (lo, None))
    rng = np.random.default_rng(9)
    Y = rng.standard_normal((nimg, 2 * L, N)) + 1j * rng.standard_normal((nimg, 2 * L, N))
    for ops in PACKED[name](n):
        Yd = torch.from_numpy(Y).to("cuda", torch.complex64).contiguous()
        tabs.run(Yd, ops)
        out = Yd.cpu().numpy()
        for i in range(nimg):
            assert max_rel(out[i], ref_eng.run(Y[i], ops)) < 5e-6, (ops, i)
