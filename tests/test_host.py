"""Host-side logic and the C ABI's CPU-checkable surface (no GPU needed)."""

import ctypes
import os
import re

import numpy as np
import pytest

from conftest import REPO, max_rel
from oracle import oblique_np as O

HEADER = os.path.join(REPO, "include", "adrt_pinv_gb300.h")


def _declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"typedef struct.*?\}\s*\w+;", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(\w+)\s*\(", src, flags=re.M)))


@pytest.fixture(scope="module")
def lib(pkg):
    import __graft_entry__ as ge

    ge.build()
    return pkg._lib.load()


def test_library_exports_every_declared_symbol(lib):
    names = _declared_functions()
    assert "bfly_rows" in names and "cheb_rows" in names and "cert_rowsum" in names and "omp_max_threads" in names
    for name in names:
        assert hasattr(lib, name), name


def test_reference_signatures_match_ctypes_binding(pkg):
    # the reference binds its library with these argtypes (fastcpp.py:25-32); ours must accept the same calls
    P = pkg._lib.PROTOTYPES
    I, D, V = ctypes.c_int, ctypes.c_double, ctypes.c_void_p
    assert P["bfly_rows"] == [I, I, V, V, I, I, I, I]
    assert P["cheb_rows"] == [I, I, V, V, V, V, D, V, V, I, I, I, V]
    assert P["cert_rowsum"] == [I, I, V, I, V, I]


def test_rowjob_layout_matches_header(pkg):
    # field order of adrt_row_job in the header equals the ctypes mirror
    src = open(HEADER).read()
    body = src[src.index("typedef struct adrt_row_job {") + len("typedef struct adrt_row_job {") : src.index("} adrt_row_job;")]
    decl = []
    for line in body.splitlines():
        line = line.split("/*")[0].strip().rstrip(";")
        for part in filter(None, (q.strip() for q in line.split(","))):
            decl.append(re.findall(r"(\w+)\s*(?:\[[^\]]*\])?\s*$", part)[0])
    mirror = [f[0] for f in pkg._lib.RowJob._fields_]
    assert decl == mirror


def test_argument_validation_without_gpu(lib):
    # these fail validation before any CUDA call
    X = np.zeros((4, 8), dtype=complex)
    z = np.ones(4, dtype=complex)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    assert lib.bfly_rows(0, 4, p(z), p(X), 1, 1, 0, 1) == 1
    assert lib.bfly_rows(3, 4, p(z), p(X), 2, 1, 0, 1) == 1
    assert b"levels" in lib.adrt_last_error()
    assert lib.bfly_rows(3, 4, p(z), p(X), 1, 4, 0, 1) == 1
    assert lib.bfly_rows(3, 0, p(z), p(X), 1, 3, 0, 1) == 0  # nothing to do
    deg = np.full(4, 3, dtype=np.int32)
    a = np.ones(4)
    assert lib.cheb_rows(12, 4, p(z), p(deg), p(a), p(a), 1.0, p(X), p(X), 1, 3, 1, None) == 1
    assert lib.cert_rowsum(0, 4, p(a), 1, p(a), 1) == 1
    assert lib.adrt_rows_run(None, None) == 1
    assert lib.adrt_pack_fft(0, 12, 1, 0, 0, None, 0, None, None, 0, None) == 1
    assert lib.adrt_ifft_unpack(0, 3, 1, None, None, None, None, None, 0, None) == 1
    assert lib.adrt_forward(0, 0, 1, None, None, None, None) == 1
    assert lib.adrt_outer_update(0, 3, 1, None, None, None, 1, None, 0.0, 0.0, 0.0, None, None) == 1  # f64 r, f32 x
    assert lib.adrt_rows_ff_run(None, None) == 1
    assert lib.adrt_cgls_start(None, None, None) == 1 and lib.adrt_pcg_step(None, None) == 1


def test_float_float_and_presplit_entries_validate_without_gpu(lib):
    """The entry points of the float-float outer state, the hi-plane pack and the pre-split dense rows reject bad
    arguments before any CUDA call (host buffers stand in for device pointers; they are never dereferenced)."""
    buf = np.zeros(1 << 16)
    q = buf.ctypes.data_as(ctypes.c_void_p)
    coef = np.ones(4)
    cq = coef.ctypes.data_as(ctypes.c_void_p)
    # pack: an image stride below N^2, not a multiple of 4, or given for sinograms
    assert lib.adrt_pack_fft(0, 4, 1, 0, 0, q, 8, q, q, 0, None) == 1 and b"src_stride" in lib.adrt_last_error()
    assert lib.adrt_pack_fft(0, 4, 1, 0, 0, q, 258, q, q, 0, None) == 1
    assert lib.adrt_pack_fft(0, 4, 1, 1, 1, q, 512, q, q, 0, None) == 1
    # float-float outer step: only 64 <= N <= 512, bands 16 / 32, a G_1 degree with its coefficients
    args = lambda n, pc, deg, band: (n, 2, q, q, q, q, q, q, q, 0.5, 0.25, 0.0, pc, deg, cq, None, band, None)
    assert lib.adrt_outer_step_ff(*args(5, 1, 3, 0)) == 1 and b"6..9" in lib.adrt_last_error()
    assert lib.adrt_outer_step_ff(*args(10, 1, 3, 0)) == 1
    assert lib.adrt_outer_step_ff(*args(8, 1, 3, 48)) == 1
    assert lib.adrt_outer_step_ff(*args(8, 1, 0, 0)) == 1
    assert lib.adrt_outer_step_ff(*args(8, 3, 3, 0)) == 1
    assert lib.adrt_ff_to_f64(12, 1, q, q, None) == 1
    # pre-split dense rows: the split for 7 <= n <= 10 only; use_tc = 3 takes FP32, 7 <= n <= 10 and an error flag
    assert lib.adrt_dense_split(6, 1, q, q, None) == 1 and lib.adrt_dense_split(11, 1, q, q, None) == 1
    rows = np.zeros(1, dtype=np.int32)
    rq = rows.ctypes.data_as(ctypes.c_void_p)
    assert lib.adrt_dense_rows(1, 8, 4, 1, rq, q, q, 256, None, q, 3, 0, None) == 1  # FP64
    assert lib.adrt_dense_rows(0, 6, 4, 1, rq, q, q, 64, None, q, 3, 0, None) == 1  # n < 7
    assert lib.adrt_dense_rows(0, 8, 4, 1, rq, q, q, 256, None, None, 3, 0, None) == 1  # no error flag
    assert lib.adrt_dense_rows(0, 8, 4, 1, rq, q, q, 256, None, q, 1, 0, None) == 1  # staging needed for use_tc 1
    assert lib.adrt_dense_rows(0, 8, 4, 1, rq, q, q, 256, None, q, 3, 48, None) == 1  # tile


def test_outer_state_format_choice(pkg):
    """Float-float outer state where the register-resident outer step runs (FP32 rows and stencil, 64 <= N <= 512);
    FP64 state otherwise."""
    from adrt_pinv_gb300.device import Pipeline

    def plan(n):
        return pkg.Plan("hybrid", n, np.full(2 << n, 4.0), outer=(1.0, 2.0, 3))

    assert all(Pipeline.ff_state_for(plan(n), "fp32") for n in (6, 7, 8, 9))
    assert not any(Pipeline.ff_state_for(plan(n), "fp32") for n in (4, 5, 10, 11))
    assert not Pipeline.ff_state_for(plan(8), "fp64")
    assert not Pipeline.ff_state_for(plan(8), "fp32", "ff") and not Pipeline.ff_state_for(plan(8), "fp32", "fp64")


@pytest.mark.parametrize("method,n", [("lp", 4), ("hybrid", 6), ("hybrid", 4), ("lp", 6)])
def test_plan_matches_oracle(pkg, golden, method, n):
    name = {"lp": "lp", "hybrid": "hyb"}[method]
    k = f"{name}_{n}"
    lam = golden[f"inv_lam_{k}"]
    plan = pkg.Plan(method, n, lam, outer=tuple(golden[f"inv_outer_{k}"]))
    assert np.array_equal(plan.deg, golden[f"inv_deg_{k}"])
    c, a = O.cheb_coeffs(plan.lam_max, plan.tau)
    for f in range(0, plan.L, 7):
        oms = O.cheb_omegas(c[f], plan.deg[f])
        row = plan.coef[f]
        assert row[0] == a[f]
        for j, om in enumerate(oms, start=1):
            assert row[3 * j - 2] == om
            assert row[3 * j - 1] == om * a[f]
            assert row[3 * j] == om - 1.0
    # level-row counts per apply equal the reference's counter
    ops = {"lp": ([("P", 1, n), ("B", 1, n), ("BT", 1, n)], [("BT", 1, n), ("P", 1, n)]),
           "hybrid": ([("B", 1, 1), ("P", 2, n), ("B", 2, n), ("BT", 2, n), ("BT", 1, 1)],
                      [("BT", 2, n), ("P", 2, n), ("BT", 1, 1)])}[method]
    total = plan.level_rows(ops[1]) + (plan.outer_deg - 1) * plan.level_rows(ops[0])
    assert total == int(golden[f"inv_count_{k}"])


def test_plan_dense_rows_and_order(pkg, golden):
    n = 6
    plan = pkg.Plan("hybrid", n, golden["inv_lam_hybd8_6"], dense_cap=8, outer=tuple(golden["inv_outer_hybd8_6"]))
    assert len(plan.dense_freqs) == int(golden["inv_ndense_hybd8_6"])
    main, dense = plan.packed_rows(False), plan.packed_rows(True)
    assert len(main) + len(dense) == 2 * plan.L
    assert np.all(np.diff(np.tile(plan.deg, 2)[main]) <= 0)
    assert set(dense % plan.L) == set(plan.dense_freqs)
    ops = [("B", 1, 1), ("P", 2, n), ("B", 2, n), ("BT", 2, n), ("BT", 1, 1)]
    bp = [("BT", 2, n), ("P", 2, n), ("BT", 1, 1)]
    assert plan.level_rows(bp) + (plan.outer_deg - 1) * plan.level_rows(ops) == int(golden["inv_count_hybd8_6"])
    F = plan.build_dense_tables()
    ref = O.dense_tikhonov(n, O.offset_z(plan.L)[plan.dense_freqs[0]], plan.tau, 2, n)
    assert max_rel(F[0], ref) < 1e-12


def test_plan_cap_and_cache(pkg, golden, tmp_path):
    plan = pkg.Plan("lp", 6, golden["c0_lam"], deg_cap=16, outer=tuple(golden["c0_outer"]))
    assert np.array_equal(plan.deg, golden["c0_deg"])
    path = os.path.join(tmp_path, "plan.npz")
    plan.save(path)
    back = pkg.Plan.load(path)
    assert np.array_equal(back.deg, plan.deg) and np.array_equal(back.lam_max, plan.lam_max)
    assert (back.lo, back.hi, back.outer_deg) == (plan.lo, plan.hi, plan.outer_deg)
    assert back.deg_cap == 16 and back.dense_cap is None


def test_fuse_ops(pkg):
    from adrt_pinv_gb300.device import fuse_ops, ops_unfused

    ops = [("B", 1, 1), ("P", 2, 8), ("B", 2, 8), ("BT", 2, 8), ("BT", 1, 1)]
    fused = fuse_ops(ops)
    assert fused == [("B", 1, 1), ("P", 2, 8), ("M", 2, 8), ("BT", 1, 1)]
    assert ops_unfused(fused) == ops


def test_outer_coeffs_match_reference_recurrence(pkg):
    a, c, steps = pkg.plan.outer_coeffs(0.3, 1.7, 12)
    om = 1.0
    for k, (om_a, om_1) in enumerate(steps, start=1):
        om = 1.0 / (1.0 - c * c / 2.0) if k == 1 else 1.0 / (1.0 - c * c * om / 4.0)
        assert om_a == om * a and om_1 == om - 1.0


def test_phantoms_deterministic(pkg):
    ph = pkg.phantoms
    a = ph.ellipse_phantom(64, 5)
    assert np.array_equal(a, ph.ellipse_phantom(64, 5))
    assert not np.array_equal(a, ph.ellipse_phantom(64, 6))
    t = ph.ellipse_phantom(32, 1, ellipses=40, texture=0.1)
    assert t.shape == (32, 32) and np.isfinite(t).all()
    im = ph.int_image(16, 2)
    assert im.dtype == np.int32 and im.min() >= 0 and im.max() <= 255


@pytest.mark.parametrize("method", ["hybrid", "lp"])
def test_dense_operator_torch_matches_host(pkg, method):
    """The device (torch, Cholesky form) dense-row operators used for n >= 9 equal the host eigendecomposition
    form for every folding, here with torch on the CPU."""
    from adrt_pinv_gb300.plan import Plan

    n, N = 5, 32
    plan = Plan(method, n, np.full(2 * N, 50.0 * N), 0.2, 0.1, 1e-10, dense_cap=8)
    assert len(plan.dense_freqs) > 0
    for key in [(a, b, c, d) for a in (0, 1) for b in (0, 1) for c in (0, 1) for d in (0, 1)]:
        ref = plan.dense_row_operator(*map(bool, key))
        got = plan.dense_row_operator_torch(*map(bool, key), device="cpu", chunk=5).numpy()
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max(), key
