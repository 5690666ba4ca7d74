"""Pins the CPU oracle (oracle/*.py) to the reference's own outputs stored in tests/golden/reference_vectors.npz.

Integer and structural results are compared bit-exactly; floating-point results to 1e-13 relative (the reference's
own cross-engine agreement is ~1e-15, `fastcpp.py:190-208`)."""

import numpy as np
import pytest

from conftest import max_rel, rel_err
from oracle import adrt_np as A
from oracle import oblique_np as O

TOL = 1e-13


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5])
def test_adrt_float(golden, n):
    assert rel_err(A.adrt(n, golden[f"adrt_x_{n}"]), golden[f"adrt_R_{n}"]) < TOL
    assert rel_err(A.adrt_T(n, golden[f"adrt_b_{n}"]), golden[f"adrt_RT_{n}"]) < TOL
    for m in range(1, n + 1):
        assert np.array_equal(A.S_apply(n, m, golden[f"level_f_{n}_{m}"]), golden[f"level_S_{n}_{m}"])
        assert np.array_equal(A.S_apply_T(n, m, golden[f"level_g_{n}_{m}"]), golden[f"level_ST_{n}_{m}"])


@pytest.mark.parametrize("n", [4, 6])
def test_adrt_int_exact(golden, n):
    xi = golden[f"adrt_int_x_{n}"]
    R = A.adrt(n, xi, dtype=np.int64)
    assert np.array_equal(R, golden[f"adrt_int_R_{n}"].astype(np.int64))
    RT = A.adrt_T(n, golden[f"adrt_int_b_{n}"], dtype=np.int64)
    assert np.array_equal(RT, golden[f"adrt_int_RT_{n}"].astype(np.int64))


def test_mask(golden):
    assert np.array_equal(A.mask_full(4), golden["mask_full_4"])


@pytest.mark.parametrize("n", [4, 6])
def test_butterflies(golden, n):
    V, z = golden[f"bf_V_{n}"], golden[f"bf_z_{n}"]
    assert max_rel(O.bfly(n, z, V), golden[f"bf_B_{n}"]) < TOL
    assert max_rel(O.bflyT(n, z, V), golden[f"bf_BT_{n}"]) < TOL
    assert max_rel(O.bfly_levels(n, z, V, 2, n), golden[f"bf_B2_{n}"]) < TOL
    assert max_rel(O.bflyT_levels(n, z, V, 2, n), golden[f"bf_BT2_{n}"]) < TOL
    assert max_rel(O.bfly_levels(n, z, V, 1, 1), golden[f"bf_B11_{n}"]) < TOL
    assert max_rel(O.bflyT_levels(n, z, V, 1, 1), golden[f"bf_BT11_{n}"]) < TOL
    for lo, hi in ((1, n), (2, n), (1, 1), (2, n - 1), (3, n)):
        assert max_rel(O.bfly_levels(n, z, V, lo, hi), golden[f"cpp_bfly_{n}_{lo}_{hi}_0"]) < TOL
        assert max_rel(O.bflyT_levels(n, z, V, lo, hi), golden[f"cpp_bfly_{n}_{lo}_{hi}_1"]) < TOL


@pytest.mark.parametrize("n", [4, 6])
@pytest.mark.parametrize("lo", [1, 2])
def test_cheb_rows(golden, n, lo):
    z = golden[f"bf_z_{n}"]
    N = 1 << n
    cnt = [0]
    Z = O.poly_apply_levels(n, z, golden[f"cheb_Y_{n}_{lo}"], golden[f"cheb_lam_{n}_{lo}"], 0.2 * N,
                            golden[f"cheb_deg_{n}_{lo}"], lo, n, cnt)
    assert max_rel(Z, golden[f"cheb_Z_{n}_{lo}"]) < 1e-12
    assert max_rel(Z, golden[f"cheb_poly_{n}_{lo}"]) < 1e-12
    assert cnt[0] == int(golden[f"cheb_steps_{n}_{lo}"])


@pytest.mark.parametrize("n", [4, 6])
@pytest.mark.parametrize("lo", [1, 2])
def test_power_iteration(golden, n, lo):
    lam = O.power_lam_max(n, O.offset_z(2 << n), lo, seeds=(0, 1))
    assert max_rel(lam, golden[f"power_{n}_{lo}"]) < 1e-10


@pytest.mark.parametrize("n", [4, 6, 8])
@pytest.mark.parametrize("lo", [1, 2])
def test_cert(golden, n, lo):
    oms = O.offset_freqs(2 << n)
    mine = np.array([O.cert_rowsum_levels(n, om, lo) for om in oms])
    assert max_rel(mine, golden[f"cert_np_{n}_{lo}"]) < TOL
    assert max_rel(mine, golden[f"cert_cpp_{n}_{lo}"]) < 1e-12


def test_explicit(golden):
    assert max_rel(O.explicit_lam_max(6, O.offset_freqs(128)), golden["explicit_6"]) < TOL


@pytest.mark.parametrize("n", [3, 5])
def test_stencils(golden, n):
    x = golden[f"st_x_{n}"]
    assert np.array_equal(O.G1_apply(x), golden[f"st_G1_{n}"])
    assert max_rel(O.Pi_apply(x), golden[f"st_Pi_{n}"]) < TOL
    assert max_rel(O.lorr_inv(x), golden[f"st_lorr_{n}"]) < TOL
    assert max_rel(O.g1_inv(x), golden[f"st_g1inv_{n}"]) < TOL


CASES = [("lp", {}), ("hyb", {}), ("hybd8", {"dense_cap": 8}), ("lpd8", {"dense_cap": 8}),
         ("hyblorr", {"precond": "lorr"})]


@pytest.mark.parametrize("n", [4, 6])
@pytest.mark.parametrize("name,kw", CASES)
def test_packed_inverses(golden, n, name, kw):
    k = f"{name}_{n}"
    lo, hi, D = golden[f"inv_outer_{k}"]
    cls = O.HybridOracle if name.startswith("hyb") else O.LpOracle
    P = cls(n, lam_max=golden[f"inv_lam_{k}"], outer=(lo, hi, D), **kw)
    assert np.array_equal(P.deg, golden[f"inv_deg_{k}"])
    assert P.eng.n_dense == int(golden[f"inv_ndense_{k}"])
    x, b = golden[f"inv_x_{n}"], golden[f"inv_b_{n}"]
    G = P.Gh if name.startswith("hyb") else P.frame_window
    assert max_rel(G(x), golden[f"inv_G_{k}"]) < 1e-12
    assert max_rel(P.backproject(b), golden[f"inv_bp_{k}"]) < 1e-12
    P.eng.count = [0]
    xr = P.apply(b)
    assert max_rel(xr, golden[f"inv_apply_{k}"]) < 1e-11
    assert P.eng.count[0] == int(golden[f"inv_count_{k}"])
    assert rel_err(xr, x) < 1e-9  # left-inverse identity L R x = x


def test_config0_capped_lp(golden):
    lo, hi, D = golden["c0_outer"]
    P = O.LpOracle(6, lam_max=golden["c0_lam"], deg_cap=16, outer=(lo, hi, D))
    assert np.array_equal(P.deg, golden["c0_deg"])
    assert P.deg.max() == 16
    assert max_rel(P.backproject(golden["c0_b"]), golden["c0_bp"]) < 1e-12
    assert rel_err(P.apply(golden["c0_b"]), golden["c0_apply"]) < 1e-12


def test_phantom_fixture_matches_generator(golden, pkg):
    assert np.array_equal(pkg.phantoms.ellipse_phantom(64, seed=0), golden["c0_x"])


def test_unpacked_references(golden):
    x, b = golden["spec_x"], golden["spec_b"]
    S = O.SpectralOracle(3, lam_max=golden["spec_lam"], outer=tuple(golden["spec_outer"]))
    assert np.array_equal(S.deg, golden["spec_deg"])
    assert max_rel(S.frame_window(x), golden["spec_fw"]) < 1e-12
    assert max_rel(S.apply(b), golden["spec_apply"]) < 1e-11
    H = O.HybridSpectralOracle(3, lam_max=golden["fhyb_lam"], outer=tuple(golden["fhyb_outer"]))
    assert np.array_equal(H.deg, golden["fhyb_deg"])
    assert max_rel(H.Gh(x), golden["fhyb_Gh"]) < 1e-12
    assert max_rel(H.apply(b), golden["fhyb_apply"]) < 1e-11


def test_outer_interval_recomputed(golden):
    """The oracle's own Lanczos setup reproduces the reference's outer interval at n=4 (tolerance of eigsh)."""
    k = "hyb_4"
    P = O.HybridOracle(4, lam_max=golden[f"inv_lam_{k}"])
    lo, hi, D = golden[f"inv_outer_{k}"]
    # eigsh runs at tol 1e-3 from ARPACK's process-dependent start vector: the enclosure agrees to a few 1e-3
    assert abs(P.lo - lo) < 5e-3 * lo and abs(P.hi - hi) < 5e-3 * hi
    assert abs(P.outer_deg - D) <= 1
