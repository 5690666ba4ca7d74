"""GPU inverses (FastLpGpu / FastHybridGpu) against the reference's golden outputs and the CPU oracle.

Tolerances: FP64 mode <= 1e-12 (operators) / 1e-11 (apply) relative, as the reference's own engines agree;
FP32 mode <= 1e-5 relative error vs FP64 (the accuracy target of the FP32 path)."""

import numpy as np
import pytest

from conftest import max_rel, rel_err
from oracle import cpu_engine as CE
from oracle import oblique_np as O

pytestmark = pytest.mark.gpu

CASES = [("lp", {}), ("hyb", {}), ("hybd8", {"dense_cap": 8}), ("lpd8", {"dense_cap": 8}),
         ("hyblorr", {"precond": "lorr"})]


def _cls(pkg, name):
    return pkg.FastHybridGpu if name.startswith("hyb") else pkg.FastLpGpu


@pytest.mark.parametrize("n", [4, 6])
@pytest.mark.parametrize("name,kw", CASES)
def test_fp64_matches_reference(pkg, golden, n, name, kw):
    k = f"{name}_{n}"
    P = _cls(pkg, name)(n, lam_max=golden[f"inv_lam_{k}"], outer=tuple(golden[f"inv_outer_{k}"]), precision="fp64", **kw)
    assert np.array_equal(P.deg, golden[f"inv_deg_{k}"])
    x, b = golden[f"inv_x_{n}"], golden[f"inv_b_{n}"]
    G = P.Gh if name.startswith("hyb") else P.frame_window
    assert max_rel(G(x), golden[f"inv_G_{k}"]) < 1e-12
    assert max_rel(P.backproject(b), golden[f"inv_bp_{k}"]) < 1e-12
    P.eng.count = [0]
    xr = P.apply(b)
    assert max_rel(xr, golden[f"inv_apply_{k}"]) < 1e-11
    assert P.eng.count[0] == int(golden[f"inv_count_{k}"])


def test_config0_lp_fp64_p16(pkg, golden):
    """L_p, FP64, N=64, p=16 on the noisy ellipse phantom: <= 1e-12 vs the reference's C++ engine."""
    P = pkg.FastLpGpu(6, lam_max=golden["c0_lam"], deg_cap=16, outer=tuple(golden["c0_outer"]), precision="fp64")
    assert np.array_equal(P.deg, golden["c0_deg"])
    assert rel_err(P.backproject(golden["c0_b"]), golden["c0_bp"]) < 1e-12
    assert rel_err(P.apply(golden["c0_b"]), golden["c0_apply"]) < 1e-12


@pytest.mark.parametrize("name,kw", CASES)
def test_fp32_within_1e5(pkg, golden, name, kw):
    n = 6
    k = f"{name}_{n}"
    P = _cls(pkg, name)(n, lam_max=golden[f"inv_lam_{k}"], outer=tuple(golden[f"inv_outer_{k}"]), precision="fp32", **kw)
    assert rel_err(P.apply(golden[f"inv_b_{n}"]), golden[f"inv_apply_{k}"]) < 1e-5


def test_packed_roundtrip_property(pkg):
    """With an empty row op list the packed pass is sum_q TqT(ifft(fft(Tq x))) = 4x (FFT round trip, Tq unitary)."""
    import torch

    for prec, tol in (("fp64", 1e-13), ("fp32", 1e-6)):
        for n in (3, 7, 9):
            N = 1 << n
            plan = pkg.Plan("lp", n, np.full(2 * N, 4.0), outer=(1.0, 2.0, 3))
            pipe = pkg.Pipeline(plan, 2, prec)
            x = torch.randn(2, N, N, dtype=torch.float64, device="cuda")
            pipe.packed_image(x, [])
            out = torch.empty_like(x)
            pipe.sum_parts(out)
            assert torch.max(torch.abs(out - 4 * x)).item() / torch.max(torch.abs(x)).item() < tol


def test_packed_sino_matches_oracle(pkg):
    import torch

    n = 5
    N = 1 << n
    rng = np.random.default_rng(2)
    b = rng.standard_normal((4, 2 * N - 1, N))
    plan = pkg.Plan("lp", n, np.full(2 * N, 4.0), outer=(1.0, 2.0, 3))
    pipe = pkg.Pipeline(plan, 1, "fp64")
    pipe.packed_sino(torch.from_numpy(b[None]).cuda(), [])
    out = torch.empty((1, N, N), dtype=torch.float64, device="cuda")
    pipe.sum_parts(out)

    class Ident:
        def run(self, Y, ops):
            return Y

    ref = O.packed(n, Ident(), lambda q: O.iota(n, b[q]), [])
    assert max_rel(out[0].cpu().numpy(), ref) < 1e-13


@pytest.fixture(scope="module")
def hybrid256(pkg):
    """N=256, p=32 hybrid, dense table for d_k > 16, plan computed on the GPU (power iteration + Lanczos)."""
    return pkg.FastHybridGpu(8, deg_cap=32, dense_cap=16, precision="fp32")


def test_n256_hybrid_fp32_vs_cpu_reference_engine(pkg, hybrid256):
    """N=256, p=32, FP32 on a noisy ellipse phantom: <= 1e-5 vs the FP64 C++-engine path on the same plan."""
    H = hybrid256
    n, N = 8, 256
    x = pkg.phantoms.ellipse_phantom(N, seed=7)
    b = pkg.phantoms.add_noise(pkg.adrtcore.adrt(n, x), 1e-3, seed=8)
    xg = H.apply(b)
    ref = CE.hybrid_cpu(n, dict(lam_max=H.lam_max, deg=H.deg, dense_cap=16, outer=(H.lo, H.hi, H.outer_deg)),
                        threads=16).apply(b)
    assert rel_err(xg, ref) < 1e-5
    assert rel_err(xg, x) < 0.05  # noisy data: close to the phantom


def test_n512_hybrid_fp32_vs_cpu_reference_engine(pkg):
    """N=512 (row programs with the warp-shuffle level), p=32, dense_cap 16, FP32: <= 1e-5 vs the FP64 C++-engine
    path on the same plan."""
    n, N = 9, 512
    H = pkg.FastHybridGpu(n, deg_cap=32, dense_cap=16, precision="fp32")
    x = pkg.phantoms.ellipse_phantom(N, seed=17)
    b = pkg.phantoms.add_noise(pkg.adrtcore.adrt(n, x), 1e-3, seed=18)
    ref = CE.hybrid_cpu(n, dict(lam_max=H.lam_max, deg=H.deg, dense_cap=16, outer=(H.lo, H.hi, H.outer_deg)),
                        threads=16).apply(b)
    assert rel_err(H.apply(b), ref) < 1e-5


def test_n256_fp32_without_dense_rows_precision(pkg):
    """Without the dense table the FP32 polynomial filter on the low-frequency rows limits the accuracy: recorded
    here (not hidden) so that a regression in the FP32 path shows."""
    H = pkg.FastHybridGpu(8, deg_cap=32, precision="fp32")
    n, N = 8, 256
    x = pkg.phantoms.ellipse_phantom(N, seed=7)
    b = pkg.phantoms.add_noise(pkg.adrtcore.adrt(n, x), 1e-3, seed=8)
    ref = CE.hybrid_cpu(n, dict(lam_max=H.lam_max, deg=H.deg, outer=(H.lo, H.hi, H.outer_deg)), threads=16).apply(b)
    assert rel_err(H.apply(b), ref) < 1e-4


def test_presplit_dense_rows_in_the_inverse(pkg, hybrid256):
    """Above 16 images the dense rows run on the complex-blocked tensor-core kernel over pre-split operators: the
    whole N=256 inverse of 20 sinograms equals the real-form tensor-core kernel's within 1e-6 and the FP64
    C++-engine path's within 1e-5."""
    import torch

    H = hybrid256
    n, N, B = 8, 256, 20
    bs = np.stack([pkg.phantoms.add_noise(pkg.adrtcore.adrt(n, pkg.phantoms.ellipse_phantom(N, seed=s)), 1e-3, seed=s + 70)
                   for s in range(B)])
    bd = torch.from_numpy(bs).cuda()
    pa = pkg.Pipeline(H.plan, B, "fp32")
    pb = pkg.Pipeline(H.plan, B, "fp32")
    pb.tables.split_dense = False
    assert pa.tables.dense_mode() == 3 and pb.tables.dense_mode() == 1
    xa = pa.apply(bd).clone()
    pa.tables.raise_if_error()
    xb = pb.apply(bd)
    for i in range(B):
        assert rel_err(xa[i].cpu().numpy(), xb[i].cpu().numpy()) < 1e-6
    ref = CE.hybrid_cpu(n, dict(lam_max=H.lam_max, deg=H.deg, dense_cap=16, outer=(H.lo, H.hi, H.outer_deg)),
                        threads=16).apply(bs[3])
    assert rel_err(xa[3].cpu().numpy(), ref) < 1e-5


def test_n256_left_inverse_and_linearity(pkg, hybrid256):
    import torch

    H = hybrid256
    n, N = 8, 256
    rng = np.random.default_rng(3)
    x = rng.standard_normal((2, N, N))
    b = pkg.adrtcore.adrt(n, x)
    xr = H.apply(b)
    assert rel_err(xr[0], x[0]) < 1e-5 and rel_err(xr[1], x[1]) < 1e-5  # L R x = x
    bt = torch.from_numpy(b).cuda()
    lin = H.apply(bt[0] + 2.0 * bt[1]).cpu().numpy()
    assert rel_err(lin, xr[0] + 2.0 * xr[1]) < 1e-5


def test_batch_equals_single(pkg, hybrid256):
    """Each result is the same alone and inside a batch, within 1e-6: the kernels do no cross-image arithmetic, but
    the dense-row matrix product may sum in a different order for a different batch width."""
    n, N = 8, 256
    bs = np.stack([pkg.phantoms.add_noise(pkg.adrtcore.adrt(n, pkg.phantoms.ellipse_phantom(N, seed=s)), 1e-3, seed=s + 100)
                   for s in range(3)])
    batch = hybrid256.apply(bs)
    for i in range(3):
        assert rel_err(batch[i], hybrid256.apply(bs[i])) < 1e-6


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("n,precond,nimg", [(5, "g1", 3), (8, "g1", 3), (8, "g1", 40), (8, "lorr", 3), (9, "g1", 3),
                                             (6, "none", 3)])
def test_fused_outer_step_matches_separate_kernels(pkg, prec, n, precond, nimg):
    """adrt_outer_step (residual + P + outer update, one clustered kernel) equals resid / g1 steps / outer kernels;
    3 images take 16-row bands (N <= 256), 40 images at N=256 the 32-row bands."""
    import torch

    if prec == "fp64" and n > 8:
        pytest.skip("FP64 fused step covers n <= 8")
    N = 1 << n
    method = "lp" if precond == "none" else "hybrid"
    plan = pkg.Plan(method, n, np.full(2 * N, 4.0), precond="g1" if precond == "none" else precond, outer=(1.0, 2.0, 3))
    pipe = pkg.Pipeline(plan, nimg, prec)
    assert pipe.fused_outer_ok()
    g = torch.Generator(device="cuda").manual_seed(n)
    y = torch.randn((nimg, N, N), dtype=torch.float64, device="cuda", generator=g)
    pipe.parts.normal_(generator=g)
    x = torch.randn((nimg, N, N), dtype=torch.float64, device="cuda", generator=g)
    xp = torch.randn((nimg, N, N), dtype=torch.float64, device="cuda", generator=g)
    out_f = torch.empty_like(x)
    out_s = torch.empty_like(x)
    pipe.fused_outer_step(y, True, x, xp, out_f, 0.7, 0.3, 0.0)
    s = pipe.resid(y)
    r = pipe.precond(s) if method == "hybrid" else s
    pipe.outer_step(x, xp, r, out_s, 0.7, 0.3, 0.0)
    tol = 1e-6 if prec == "fp32" else 1e-13
    assert (out_f - out_s).abs().max().item() / out_s.abs().max().item() < tol
    pipe.fused_outer_step(y, False, None, None, out_f, 0.0, 0.0, 0.25)
    r = pipe.precond(pipe.resid(y, with_parts=False)) if method == "hybrid" else y
    pipe.outer_step(None, None, r, out_s, 0.0, 0.0, 0.25)
    assert (out_f - out_s).abs().max().item() / out_s.abs().max().item() < tol


@pytest.mark.parametrize("precond", ["g1", "lorr", "none"])
@pytest.mark.parametrize("n,nimg,band", [(6, 3, 0), (7, 5, 16), (8, 3, 0), (8, 40, 0), (8, 40, 16), (9, 3, 32),
                                         (9, 2, 16)])
def test_register_outer_step_matches_shared_form(pkg, n, nimg, band, precond):
    """The register-resident fused outer step (FP32 stencil and partial images, 64 <= N <= 512: iterates in
    registers, column neighbours by warp shuffle, halo rows and warp-edge columns through shared memory) against the
    shared-memory form (ADRT_OS_SHARED) on the same inputs, with per-image outer coefficients: the same arithmetic
    term for term, so equal up to FP32 contraction differences (1e-6). The G_1 preconditioner alone against the
    oracle's g1_inv (fasthybrid.py:114-130) at FP32 accuracy (1e-5)."""
    import torch

    N = 1 << n
    method = "lp" if precond == "none" else "hybrid"
    plan = pkg.Plan(method, n, np.full(2 * N, 4.0), precond="g1" if precond == "none" else precond, outer=(1.0, 2.0, 3))
    pipe = pkg.Pipeline(plan, nimg, "fp32")
    assert pipe.fused_outer_ok()
    g = torch.Generator(device="cuda").manual_seed(n + band)
    y = torch.randn((nimg, N, N), dtype=torch.float64, device="cuda", generator=g)
    pipe.parts.normal_(generator=g)
    x = torch.randn((nimg, N, N), dtype=torch.float64, device="cuda", generator=g)
    xp = torch.randn((nimg, N, N), dtype=torch.float64, device="cuda", generator=g)
    om = torch.rand((nimg, 2), dtype=torch.float64, device="cuda", generator=g)
    outs = []
    for shared in (False, True):
        pipe.band = band | (pkg._lib.OS_SHARED if shared else 0)
        o1 = torch.empty_like(x)
        o2 = torch.empty_like(x)
        pipe.fused_outer_step(y, True, x, xp, o1, 0.0, 0.0, 0.0, om_img=om)
        pipe.fused_outer_step(y, False, None, None, o2, 0.0, 0.0, 0.5)
        outs.append((o1, o2))
    pipe.band = 0
    for a, b in zip(*outs):
        assert (a - b).abs().max().item() / b.abs().max().item() < 1e-6
    if precond == "g1":
        got = outs[0][1].cpu().numpy()
        yh = y.cpu().numpy()
        for i in range(min(nimg, 3)):
            assert rel_err(got[i], 0.5 * O.g1_inv(yh[i])) < 1e-5


def _ff_planes(v):
    """FP64 images (B, N, N) -> float-float planes (B, 2, N, N): hi = fl32(v), lo = fl32(v - hi)."""
    import torch

    hi = v.float()
    return torch.stack([hi, (v - hi.double()).float()], 1).contiguous()


@pytest.mark.parametrize("n,nimg,precond,per_image", [(6, 3, "g1", False), (8, 5, "g1", True), (8, 40, "lorr", False),
                                                      (9, 2, "g1", False), (7, 4, "none", True)])
def test_float_float_state_outer_step(pkg, n, nimg, precond, per_image):
    """adrt_outer_step_ff (outer state as float-float planes, FP32 y, FP32 arithmetic only) against the FP64-state
    fused step on the same values. The residual and the preconditioner are the same FP32 computation (y - sum of
    the parts rounds once either way), so the new states differ only by the FP32 rounding of the update
    om_a r + om_1 (x - x_prev): within 1e-6 of the update. The first step a0 P(y) is a float-float product (1e-12)."""
    import torch

    N = 1 << n
    method = "lp" if precond == "none" else "hybrid"
    plan = pkg.Plan(method, n, np.full(2 * N, 4.0), precond="g1" if precond == "none" else precond, outer=(1.0, 2.0, 3))
    pipe = pkg.Pipeline(plan, nimg, "fp32")
    assert pipe.ff_state and pipe.fused_outer_ok()
    g = torch.Generator(device="cuda").manual_seed(n + nimg)
    y32 = torch.randn((nimg, N, N), dtype=torch.float32, device="cuda", generator=g)
    pipe.parts.normal_(generator=g)
    x = torch.randn((nimg, N, N), dtype=torch.float64, device="cuda", generator=g)
    xp = x + 0.1 * torch.randn((nimg, N, N), dtype=torch.float64, device="cuda", generator=g)
    om = torch.rand((nimg, 2), dtype=torch.float64, device="cuda", generator=g) if per_image else None
    out64 = torch.empty_like(x)
    outff = torch.empty((nimg, 2, N, N), dtype=torch.float32, device="cuda")
    pipe.fused_outer_step(y32.double(), True, x, xp, out64, 0.7, 0.3, 0.0, om_img=om)
    pipe.fused_outer_step(y32, True, _ff_planes(x), _ff_planes(xp), outff, 0.7, 0.3, 0.0, om_img=om)
    got = pipe.result(outff, torch.empty_like(x))
    assert ((got - out64).abs().max() / (out64 - x).abs().max()).item() < 1e-6
    pipe.fused_outer_step(y32.double(), False, None, None, out64, 0.0, 0.0, 0.37)
    pipe.fused_outer_step(y32, False, None, None, outff, 0.0, 0.0, 0.37)
    got = pipe.result(outff, torch.empty_like(x))
    assert ((got - out64).abs().max() / out64.abs().max()).item() < 1e-12
    # the float-float result keeps hi = fl32(hi + lo): its planes are normalised
    assert torch.equal(outff[:, 0], (outff[:, 0].double() + outff[:, 1].double()).float())


def test_pack_reads_hi_plane_of_float_float_images(pkg):
    """The pack of float-float images (B, 2, N, N) reads the hi planes (image stride 2 N^2): the same packed rows as
    the pack of the hi planes alone."""
    import torch

    n, B = 7, 3
    N = 1 << n
    plan = pkg.Plan("hybrid", n, np.full(2 * N, 4.0), outer=(1.0, 2.0, 3))
    pipe = pkg.Pipeline(plan, B, "fp32")
    x = torch.randn((B, 2, N, N), dtype=torch.float32, device="cuda")
    pipe.pack(x, sino=False)
    y1 = pipe.Y.clone()
    pipe.pack(x[:, 0].contiguous(), sino=False)
    assert torch.equal(y1, pipe.Y)


def test_float_float_state_inverse_matches_fp64_state(pkg, hybrid256):
    """The whole N=256 hybrid inverse with the float-float outer state (the default) against the same pipeline with
    the FP64 outer state: both compute the rows, FFTs and stencil in FP32, so they agree far inside the 1e-5
    accuracy target (1e-6)."""
    import torch

    n, N, B = 8, 256, 4
    bs = np.stack([pkg.phantoms.add_noise(pkg.adrtcore.adrt(n, pkg.phantoms.ellipse_phantom(N, seed=s)), 1e-3, seed=s + 50)
                   for s in range(B)])
    bd = torch.from_numpy(bs).cuda()
    pa = pkg.Pipeline(hybrid256.plan, B, "fp32")
    pb = pkg.Pipeline(hybrid256.plan, B, "fp32", state="fp64")
    assert pa.ff_state and not pb.ff_state
    xa = pa.apply(bd).clone()
    xb = pb.apply(bd)
    for i in range(B):
        assert rel_err(xa[i].cpu().numpy(), xb[i].cpu().numpy()) < 1e-6


@pytest.mark.parametrize("sprec,tol", [("fp64", 1e-12), ("ff", 1e-10)])
@pytest.mark.parametrize("n,nimg", [(4, 2), (6, 3), (8, 3), (8, 40)])
def test_fused_cross_quadrant_inverse_high_precision(pkg, sprec, tol, n, nimg):
    """The fused outer step of an FP32 pipeline with the cross-quadrant preconditioner in FP64 or float-float:
    x_new = a0 g1_inv(y) against the oracle's g1_inv (fasthybrid.py:114-130, pinned to the reference's golden
    values) image by image; FP64 to 1e-12, float-float to 1e-10. With FP32 partial images the residual is
    y - (p0 + p1 + p2) summed in FP32 and differenced in FP64, checked on the same images."""
    import torch

    N = 1 << n
    plan = pkg.Plan("hybrid", n, np.full(2 * N, 4.0), precond="g1", outer=(1.0, 2.0, 3))
    pipe = pkg.Pipeline(plan, nimg, "fp32", stencil_precision=sprec)
    assert pipe.fused_outer_ok()
    rng = np.random.default_rng(n + nimg)
    y = rng.standard_normal((nimg, N, N))
    out = torch.empty((nimg, N, N), dtype=torch.float64, device="cuda")
    pipe.fused_outer_step(torch.from_numpy(y).cuda(), False, None, None, out, 0.0, 0.0, 0.5)
    got = out.cpu().numpy()
    for i in range(nimg):
        assert rel_err(got[i], 0.5 * O.g1_inv(y[i])) < tol
    pipe.parts.normal_()
    pipe.fused_outer_step(torch.from_numpy(y).cuda(), True, None, None, out, 0.0, 0.0, 1.0)
    parts = pipe.parts.cpu().numpy()
    s = y - ((parts[0] + parts[1]) + parts[2]).astype(np.float64)
    got = out.cpu().numpy()
    for i in range(min(nimg, 3)):
        assert rel_err(got[i], O.g1_inv(s[i])) < tol


@pytest.mark.parametrize("cap", [16, 8])
def test_n256_compensated_rows_without_dense_operators(pkg, cap):
    """The rows with d_k > cap keep the polynomial filter, evaluated in float-float (compensated) arithmetic, and
    no dense operator is stored: the FP32 inverse against the reference's C++-engine path on the same plan (every
    row polynomial, FP64) stays within 1e-5, where the plain FP32 polynomial rows give about 3e-5."""
    H = pkg.FastHybridGpu(8, deg_cap=32, dense_cap=cap, precision="fp32", high_rows="ff")
    n, N = 8, 256
    assert H.eng.n_dense > 0 and H.pipeline(1).tables.high_ff
    x = pkg.phantoms.ellipse_phantom(N, seed=7)
    b = pkg.phantoms.add_noise(pkg.adrtcore.adrt(n, x), 1e-3, seed=8)
    ref = CE.hybrid_cpu(n, dict(lam_max=H.lam_max, deg=H.deg, outer=(H.lo, H.hi, H.outer_deg)), threads=16).apply(b)
    got = H.apply(b)
    assert not H.pipeline(1).tables._dense_dev  # no operator was built
    assert rel_err(got, ref) < 1e-5


@pytest.mark.parametrize("method", ["lp", "hybrid"])
def test_compensated_rows_match_fp64_rows(pkg, method):
    """Row level: both op lists of each method on the high rows in float-float equal the FP64 row engine to about
    FP32 output rounding (2e-7), well below the FP32 polynomial rows' error on the same rows."""
    import torch

    from adrt_pinv_gb300.device import RowTables, _op_lists

    n, N = 6, 64
    cls = pkg.FastLpGpu if method == "lp" else pkg.FastHybridGpu
    H = cls(n, deg_cap=32, dense_cap=8, precision="fp32", high_rows="ff")
    plan = H.plan
    t32 = RowTables(plan, torch.float32, torch.device("cuda"))
    t64 = RowTables(plan, torch.float64, torch.device("cuda"))
    rows = t32.rows_dense.long()
    g = torch.Generator(device="cuda").manual_seed(1)
    Y = torch.randn((2, 4 * N, N), dtype=torch.complex128, device="cuda", generator=g)
    for ops in _op_lists(plan).values():
        ref = Y.clone()
        t64.run(ref, ops)
        got = Y.to(torch.complex64)
        t32.run(got, ops)
        err = ((got.to(torch.complex128) - ref)[:, rows].abs().max() / ref[:, rows].abs().max()).item()
        assert err < 2e-6, (ops, err)


@pytest.mark.parametrize("n", [6, 8, 9])
def test_fft_narrow_columns_same_result(pkg, n):
    """The offset FFTs with a quarter of the default strip columns per CTA (a tile shape the autotuner may pick) give
    the same packed pass: every column is transformed by the same arithmetic whatever the CTA shape."""
    import torch

    from adrt_pinv_gb300 import tune

    N = 1 << n
    plan = pkg.Plan("hybrid", n, np.full(2 * N, 4.0), outer=(1.0, 2.0, 3))
    x = torch.randn((3, N, N), dtype=torch.float64, device="cuda", generator=torch.Generator("cuda").manual_seed(n))
    outs = []
    for cols in (0, tune.fft_cols_default(N, torch.float32) // 4):
        pipe = pkg.Pipeline(plan, 3, "fp32")
        pipe.fft_cols = cols
        pipe.packed_image(x, [("B", 1, n), ("BT", 1, n)])
        out = torch.empty_like(x)
        pipe.sum_parts(out)
        outs.append(out)
    assert torch.equal(outs[0], outs[1])
