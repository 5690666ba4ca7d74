"""The oracle's restatements of pinv.py (CGLS, PCG) and of the gram_freq patch (gram_freq, gram, lstsq_cheb) against
golden vectors made by the reference itself (tests/golden/pinv_gram_vectors.npz: the reference's pinv.py and
adrtcore.py, and the patch's own C++ gram_freq compiled from the patch text). CPU only."""

import os

import numpy as np
import pytest

from conftest import REPO, rel_err
from oracle import pinv_np as P

GOLD = os.path.join(REPO, "tests", "golden", "pinv_gram_vectors.npz")


@pytest.fixture(scope="module")
def g():
    with np.load(GOLD) as f:
        return {k: f[k] for k in f.files}


@pytest.mark.parametrize("key", ["3_2000", "4_2000", "5_2000", "6_3000", "4_7"])
def test_cgls_matches_reference(g, key):
    n = int(key.split("_")[0])
    maxit = int(key.split("_")[1])
    x, h = P.cgls(n, g[f"cgls_b_{key}"], tol=float(g[f"cgls_tol_{key}"]), maxit=maxit)
    assert len(h) == len(g[f"cgls_hist_{key}"])
    assert rel_err(x, g[f"cgls_x_{key}"]) < 1e-10
    assert rel_err(h, g[f"cgls_hist_{key}"]) < 1e-9


def test_cgls_nonzero_start_matches_reference(g):
    x, h = P.cgls(4, g["cgls_x0_b"], tol=1e-10, maxit=2000, x0=g["cgls_x0_x0"])
    assert len(h) == len(g["cgls_x0_hist"]) and rel_err(x, g["cgls_x0_x"]) < 1e-10


@pytest.mark.parametrize("n", [3, 4, 5])
def test_pcg_matches_reference(g, n):
    N = 1 << n
    for tag, M in (("id", lambda v: v), ("sc", lambda v: v / (4.0 * N))):
        x, h = P.pcg_normal(n, g[f"pcg_b_{n}"], M, tol=1e-10, maxit=2000)
        assert len(h) == len(g[f"pcg_hist_{tag}_{n}"])
        assert rel_err(x, g[f"pcg_x_{tag}_{n}"]) < 1e-10


@pytest.mark.parametrize("n", range(1, 7))
def test_gram_freq_matches_patch_kernel(g, n):
    a, om = g[f"gf_a_{n}"], g[f"gf_om_{n}"]
    ref = P.gram_freq(a, om)
    assert rel_err(ref, g[f"gf_f64_{n}"]) < 1e-13
    assert rel_err(g[f"gf_f32_{n}"], g[f"gf_f64_{n}"]) < 2e-5  # the patch's own FP32 kernel, for the GPU bound


def test_gram_freq_any_frequency(g):
    assert rel_err(P.gram_freq(g["gf_a_any"], g["gf_om_any"]), g["gf_f64_any"]) < 1e-13


@pytest.mark.parametrize("n", range(1, 7))
def test_gram_is_normal_operator(g, n):
    assert rel_err(P.gram(g[f"gram_a_{n}"]), g[f"gram_{n}"]) < 1e-12


@pytest.mark.parametrize("n", [2, 3, 4])
def test_lstsq_cheb_matches_dense_lstsq(g, n):
    lo, hi = g[f"ls_eig_{n}"]
    x = P.lstsq_cheb(g[f"ls_b_{n}"], 0.99 * lo, 1.01 * hi, tol=1e-10)
    assert rel_err(x, g[f"ls_x_{n}"]) < 1e-8


def test_pinv_dense_reproduces_cgls(g):
    """The reference's self-check (pinv.py:91-104) on the golden dense pseudoinverses: CGLS (oracle) = R^+ b."""
    from oracle import adrt_np as A

    for n in (1, 2, 3):
        N = 1 << n
        b = np.random.default_rng(n).standard_normal((4, 2 * N - 1, N))
        xd = (g[f"pinv_dense_{n}"] @ b.ravel()).reshape(N, N)
        x1, _ = P.cgls(n, b, tol=1e-14)
        assert rel_err(x1, xd) < 1e-9
        assert A.adrt(n, xd).shape == b.shape


@pytest.mark.parametrize("shape", [(4, 8), (6, 6), (8,)])
def test_gpu_gram_rejects_bad_shape_before_any_device_work(pkg, shape):
    """The product's argument checks (host logic, as the patch's tests/test_gram.py states them)."""
    with pytest.raises(ValueError):
        pkg.gram.gram(np.zeros(shape))


def test_gpu_gram_rejects_int_and_bad_intervals(pkg):
    with pytest.raises(TypeError):
        pkg.gram.gram(np.zeros((8, 8), dtype=np.int64))
    with pytest.raises(ValueError):
        pkg.gram.lstsq_cheb(np.zeros((4, 15, 8)), lam_min=10.0, lam_max=5.0)
    with pytest.raises(ValueError):
        pkg.gram.lstsq_cheb(np.zeros((3, 15, 8)), lam_min=1.0, lam_max=5.0)
    with pytest.raises(TypeError):
        pkg.gram.gram_freq(np.zeros((4, 8), dtype=np.complex128), np.zeros(4, dtype=np.float32))
    with pytest.raises(ValueError):
        pkg.gram.gram_freq(np.zeros((4, 8), dtype=np.complex128), np.zeros(5))


def test_cgls_history_depends_on_summation_order(g):
    """Why the GPU CGLS tests compare solutions and early histories only: the reference's own algorithm, run with its
    inner products summed in another order (blocks of 37 terms), keeps the solution (<= 1e-7) and the history while
    the residual is above 1e-3 of its start, then the histories part (by tens of percent mid-run) and the stopping
    iteration can move by one."""
    orig = P._ip

    def blocked(a, c):
        v = (np.asarray(a) * np.asarray(c)).ravel()
        return float(sum(np.sum(v[i:i + 37]) for i in range(0, len(v), 37)))

    worst_mid = 0.0
    try:
        P._ip = blocked
        for key, tol, mx in (("4_2000", 1e-10, 2000), ("5_2000", 1e-8, 2000), ("6_3000", 1e-8, 3000)):
            x, h = P.cgls(int(key[0]), g[f"cgls_b_{key}"], tol=tol, maxit=mx)
            ref_h = g[f"cgls_hist_{key}"]
            m = min(len(h), len(ref_h))
            keep = ref_h[:m] > 1e-3 * ref_h[0]
            rel = np.abs(h[:m] - ref_h[:m]) / ref_h[:m]
            assert rel_err(x, g[f"cgls_x_{key}"]) < 1e-7 and rel[keep].max() < 1e-6
            assert abs(len(h) - len(ref_h)) <= 2
            worst_mid = max(worst_mid, rel.max())
    finally:
        P._ip = orig
    assert worst_mid > 1e-2  # the later history is not reproducible at any fixed tolerance
