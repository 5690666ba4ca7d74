"""GPU setup (power iteration, certified bounds, Lanczos outer interval) and the spatial ADRT kernels."""

import numpy as np
import pytest

from conftest import max_rel
from oracle import adrt_np as A
from oracle import oblique_np as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [4, 6])
@pytest.mark.parametrize("lo", [1, 2])
def test_power_iteration_matches_reference(pkg, golden, n, lo):
    lam = pkg.power_lam_max(n, lo)
    assert max_rel(lam, golden[f"power_{n}_{lo}"]) < 1e-10


def test_cert_bounds(pkg, golden):
    for n in (4, 6, 8):
        for lo in (1, 2):
            assert max_rel(pkg.cert_lam_max(n, O.offset_freqs(2 << n), lo), golden[f"cert_cpp_{n}_{lo}"]) < 1e-12


@pytest.mark.parametrize("name", ["hyb", "lp"])
def test_outer_interval_on_gpu(pkg, golden, name):
    """Full GPU setup: same Lambda (power iteration), degrees and outer interval as the reference."""
    n = 6
    k = f"{name}_{n}"
    cls = pkg.FastHybridGpu if name == "hyb" else pkg.FastLpGpu
    P = cls(n, lam_max=golden[f"inv_lam_{k}"])
    lo, hi, D = golden[f"inv_outer_{k}"]
    assert np.array_equal(P.deg, golden[f"inv_deg_{k}"])
    # eigsh tol 1e-3 from ARPACK's process-dependent start vector: agreement to a few 1e-3
    assert abs(P.lo - lo) < 5e-3 * lo and abs(P.hi - hi) < 5e-3 * hi
    assert abs(P.outer_deg - int(D)) <= 1


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5])
def test_adrt_float_matches_reference(pkg, golden, n):
    ac = pkg.adrtcore
    assert max_rel(ac.adrt(n, golden[f"adrt_x_{n}"]), golden[f"adrt_R_{n}"]) < 1e-13
    assert max_rel(ac.adrt_T(n, golden[f"adrt_b_{n}"]), golden[f"adrt_RT_{n}"]) < 1e-13


@pytest.mark.parametrize("n", [4, 6])
def test_adrt_int_golden(pkg, golden, n):
    ac = pkg.adrtcore
    assert np.array_equal(ac.adrt(n, golden[f"adrt_int_x_{n}"], dtype=np.int32), golden[f"adrt_int_R_{n}"].astype(np.int32))
    assert np.array_equal(ac.adrt_T(n, golden[f"adrt_int_b_{n}"], dtype=np.int64), golden[f"adrt_int_RT_{n}"].astype(np.int64))


@pytest.mark.parametrize("n", [7, 8])
def test_adrt_int_bit_exact_batch(pkg, n):
    """int32 forward and int64 transpose on a batch of U{0..255} images: bit-exact against the oracle."""
    ac = pkg.adrtcore
    N = 1 << n
    xs = np.stack([pkg.phantoms.int_image(N, s) for s in range(3)])
    R = ac.adrt(n, xs, dtype=np.int32)
    for i in range(3):
        assert np.array_equal(R[i], A.adrt(n, xs[i], dtype=np.int64).astype(np.int32))
    RT = ac.adrt_T(n, R.astype(np.int64), dtype=np.int64)
    assert np.array_equal(RT[1], A.adrt_T(n, R[1].astype(np.int64), dtype=np.int64))


def test_adrt_adjoint_identity(pkg):
    ac = pkg.adrtcore
    n = 6
    N = 1 << n
    rng = np.random.default_rng(0)
    x = rng.standard_normal((N, N))
    b = rng.standard_normal((4, 2 * N - 1, N))
    lhs = np.sum(ac.adrt(n, x) * b)
    rhs = np.sum(x * ac.adrt_T(n, b))
    assert abs(lhs - rhs) < 1e-9 * abs(lhs)
