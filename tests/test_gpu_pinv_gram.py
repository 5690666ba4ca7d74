"""GPU Moore-Penrose baselines (CGLS, PCG on the normal equations, the dense pseudoinverse; pinv.py:23-88) and the
row-wise normal operator of the gram_freq patch (gram_freq, gram, lstsq_cheb) against golden vectors made by the
reference itself (tests/golden/pinv_gram_vectors.npz).

Tolerances. CGLS / PCG in floating point lose orthogonality as they run: once the residual has fallen by about three
orders of magnitude, rounding differences of the inner products (NumPy's summation order against the library's
fixed partial sums) steer the later iterates and the residual history apart, while both runs converge to the same
solution. So: solutions within 1e-7 relative of the reference's, histories equal to 1e-6 while the reference's entry
is above 1e-3 of its first, and the iteration count within 10 % (exact where maxit stops the loop). Dense pseudoinverse and FP64 gram / gram_freq: 1e-10 .. 1e-12; the FP32 gram_freq / gram
within the patch's own FP32 bound (2e-5 of the largest entry)."""

import os

import numpy as np
import pytest

from conftest import REPO, rel_err

pytestmark = pytest.mark.gpu

GOLD = os.path.join(REPO, "tests", "golden", "pinv_gram_vectors.npz")


@pytest.fixture(scope="module")
def g():
    with np.load(GOLD) as f:
        return {k: f[k] for k in f.files}


def _check_iterative(x, h, ref_x, ref_h, exact_len=False):
    assert rel_err(x, ref_x) < 1e-7
    if exact_len:
        assert len(h) == len(ref_h)
    assert abs(len(h) - len(ref_h)) <= max(2, len(ref_h) // 10), (len(h), len(ref_h))
    m = min(len(h), len(ref_h))
    keep = ref_h[:m] > 1e-3 * ref_h[0]  # before rounding differences of the inner products steer the iterates
    assert np.max(np.abs(h[:m][keep] - ref_h[:m][keep]) / ref_h[:m][keep]) < 1e-6


@pytest.mark.parametrize("key", ["3_2000", "4_2000", "5_2000", "6_3000", "4_7"])
def test_cgls_matches_reference(pkg, g, key):
    n, maxit = (int(v) for v in key.split("_"))
    x, h = pkg.pinv.cgls(n, g[f"cgls_b_{key}"], tol=float(g[f"cgls_tol_{key}"]), maxit=maxit)
    _check_iterative(x, h, g[f"cgls_x_{key}"], g[f"cgls_hist_{key}"], exact_len=maxit < 100)


def test_cgls_batch_each_sinogram_as_alone(pkg, g):
    """Two sinograms with different starts and different iteration counts in one batch: each ends with the
    reference's iterate and history for it alone."""
    import torch

    b = np.stack([g["cgls_b_4_2000"], g["cgls_x0_b"]])
    x0 = np.stack([np.zeros((16, 16)), g["cgls_x0_x0"]])
    x, hs = pkg.pinv.cgls(4, torch.from_numpy(b).cuda(), tol=1e-10, maxit=2000, x0=x0)
    assert x.is_cuda and x.shape == (2, 16, 16)
    _check_iterative(x[0].cpu().numpy(), hs[0], g["cgls_x_4_2000"], g["cgls_hist_4_2000"])
    _check_iterative(x[1].cpu().numpy(), hs[1], g["cgls_x0_x"], g["cgls_x0_hist"])
    x1, h1 = pkg.pinv.cgls(4, g["cgls_b_4_2000"], tol=1e-10, maxit=2000)  # alone: the same arithmetic
    assert len(h1) == len(hs[0]) and np.array_equal(x1, x[0].cpu().numpy())


def test_cgls_callback_sees_every_iteration(pkg, g):
    seen = []
    x, h = pkg.pinv.cgls(3, g["cgls_b_3_2000"], tol=1e-10, maxit=2000,
                         callback=lambda it, x, gn: seen.append((it, gn)))
    assert [s[0] for s in seen] == list(range(len(h) - 1))
    assert rel_err(np.array([s[1] for s in seen]), h[1:]) == 0.0
    _check_iterative(x, h, g["cgls_x_3_2000"], g["cgls_hist_3_2000"])


def test_cgls_zero_data_stops_at_start(pkg):
    x, h = pkg.pinv.cgls(3, np.zeros((4, 15, 8)), tol=1e-10, maxit=50)
    assert len(h) == 1 and h[0] == 0.0 and not np.any(x)


@pytest.mark.parametrize("n", [3, 4, 5])
def test_pcg_matches_reference(pkg, g, n):
    N = 1 << n
    x, h = pkg.pinv.pcg_normal(n, g[f"pcg_b_{n}"], None, tol=1e-10, maxit=2000)
    _check_iterative(x, h, g[f"pcg_x_id_{n}"], g[f"pcg_hist_id_{n}"])
    x, h = pkg.pinv.pcg_normal(n, g[f"pcg_b_{n}"], lambda r: r / (4.0 * N), tol=1e-10, maxit=2000)
    _check_iterative(x, h, g[f"pcg_x_sc_{n}"], g[f"pcg_hist_sc_{n}"])


@pytest.mark.parametrize("n", [1, 2, 3])
def test_pinv_dense_matches_reference(pkg, g, n):
    assert rel_err(pkg.pinv.pinv_dense(n), g[f"pinv_dense_{n}"]) < 1e-10


@pytest.mark.parametrize("n", range(1, 7))
def test_gram_freq_matches_patch_kernel(pkg, g, n):
    a, om = g[f"gf_a_{n}"], g[f"gf_om_{n}"]
    out = pkg.gram.gram_freq(a, om)
    assert out.dtype == np.complex128 and out.shape == a.shape
    assert rel_err(out, g[f"gf_f64_{n}"]) < 1e-12
    out32 = pkg.gram.gram_freq(a.astype(np.complex64), om.astype(np.float32))
    ref = g[f"gf_f64_{n}"]
    assert out32.dtype == np.complex64
    assert np.abs(out32 - ref).max() <= 2e-5 * np.abs(ref).max()


def test_gram_freq_any_frequency(pkg, g):
    assert rel_err(pkg.gram.gram_freq(g["gf_a_any"], g["gf_om_any"]), g["gf_f64_any"]) < 1e-12


@pytest.mark.parametrize("n", range(1, 7))
def test_gram_is_normal_operator(pkg, g, n):
    a, ref = g[f"gram_a_{n}"], g[f"gram_{n}"]
    out = pkg.gram.gram(a)
    assert out.dtype == np.float64 and rel_err(out, ref) < 1e-11
    out32 = pkg.gram.gram(a.astype(np.float32))
    assert out32.dtype == np.float32 and np.abs(out32 - ref).max() <= 2e-5 * np.abs(ref).max()


def test_gram_batch(pkg, g):
    a = np.random.default_rng(0).standard_normal((3, 2, 16, 16))
    out = pkg.gram.gram(a)
    from oracle import pinv_np as P

    for i in range(3):
        for j in range(2):
            assert rel_err(out[i, j], P.gram(a[i, j])) < 1e-11


@pytest.mark.parametrize("n", [2, 3, 4])
def test_lstsq_cheb_matches_dense_lstsq(pkg, g, n):
    lo, hi = g[f"ls_eig_{n}"]
    x = pkg.gram.lstsq_cheb(g[f"ls_b_{n}"], lam_min=0.99 * lo, lam_max=1.01 * hi, tol=1e-10)
    assert rel_err(x, g[f"ls_x_{n}"]) < 1e-8


def test_lstsq_cheb_estimated_lam_max(pkg):
    """The patch's own check: with lam_max from the power iteration, the data of an image give the image back."""
    x = np.random.default_rng(3).standard_normal((8, 8))
    b = pkg.adrtcore.adrt(3, x)
    out = pkg.gram.lstsq_cheb(b, lam_min=15.0)
    assert np.linalg.norm(out - x) <= 1e-8 * np.linalg.norm(x)
