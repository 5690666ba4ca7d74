"""Generate the golden fixtures in this directory by running the reference implementation (dsrim/adrt-pinv).

Run from the repository root with the path of a read-only reference checkout (no default):

    python tests/golden/make_golden.py REF          (or ADRT_PINV_REF=REF python tests/golden/make_golden.py)

The reference is copied to a temporary directory first because its C++ engine (`fastcpp.py:19-21`) compiles
`cpp/liboblique.so` next to its own source. Every array in the fixtures comes from the reference's own code
(adrtcore, fastspec, fasthybrid, fastops, fastcpp); the only inputs made here are seeded Gaussians and the
seeded ellipse phantom of this package. The fixtures are small (n <= 6) so that the oracle tests finish in
seconds on a CPU.
"""

import importlib.util
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def _load_phantoms():
    spec = importlib.util.spec_from_file_location("phantoms", os.path.join(REPO, "adrt-pinv_gb300", "phantoms.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _import_reference(ref):
    tmp = tempfile.mkdtemp(prefix="adrt_ref_")
    dst = os.path.join(tmp, "ref")
    shutil.copytree(ref, dst)
    for root, dirs, files in os.walk(dst):
        for f in files:
            os.chmod(os.path.join(root, f), 0o644)
        os.chmod(root, 0o755)
    sys.path.insert(0, dst)
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    import adrtcore as ac  # noqa: E402
    import fastcpp as fc  # noqa: E402
    import fasthybrid as fh  # noqa: E402
    import fastops as fo  # noqa: E402
    import fastspec as fs  # noqa: E402

    return ac, fs, fh, fo, fc


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ADRT_PINV_REF")
    if not ref:
        sys.exit("usage: make_golden.py REF (the path of a reference checkout; or set ADRT_PINV_REF)")
    ac, fs, fh, fo, fc = _import_reference(ref)
    ph = _load_phantoms()
    out = {}

    # ---- spatial ADRT (adrtcore.py:122-137), float and integer images
    for n in range(1, 6):
        N = 1 << n
        rng = np.random.default_rng(100 + n)
        x = rng.standard_normal((N, N))
        b = rng.standard_normal((4, 2 * N - 1, N))
        out[f"adrt_x_{n}"] = x
        out[f"adrt_R_{n}"] = ac.adrt(n, x)
        out[f"adrt_b_{n}"] = b
        out[f"adrt_RT_{n}"] = ac.adrt_T(n, b)
        for m in range(1, n + 1):
            f = rng.standard_normal(ac.level_shape(n, m - 1))
            g = rng.standard_normal(ac.level_shape(n, m))
            out[f"level_f_{n}_{m}"] = f
            out[f"level_S_{n}_{m}"] = ac.S_apply(n, m, f)
            out[f"level_g_{n}_{m}"] = g
            out[f"level_ST_{n}_{m}"] = ac.S_apply_T(n, m, g)
    for n in (4, 6):
        N = 1 << n
        xi = ph.int_image(N, 7 + n)
        bi = np.random.default_rng(8 + n).integers(0, 256, size=(4, 2 * N - 1, N)).astype(np.int64)
        out[f"adrt_int_x_{n}"] = xi
        out[f"adrt_int_R_{n}"] = ac.adrt(n, xi)
        out[f"adrt_int_b_{n}"] = bi
        out[f"adrt_int_RT_{n}"] = ac.adrt_T(n, bi)
    out["mask_full_4"] = ac.mask_full(4)

    # ---- butterflies (fastspec.py:21-52, fasthybrid.py:23-54) and the C++ row kernels (cpp/oblique.cpp)
    for n in (4, 6):
        N, L = 1 << n, 2 << n
        rng = np.random.default_rng(200 + n)
        zall = np.exp(1j * 2 * np.pi * np.fft.fftfreq(L))
        rows = np.arange(0, L, 1 if n < 6 else 4)  # every frequency at n=4, every 4th at n=6 (rows are independent)
        z = zall[rows]
        K = len(rows)
        V = rng.standard_normal((K, N)) + 1j * rng.standard_normal((K, N))
        out[f"bf_rows_{n}"] = rows
        out[f"bf_V_{n}"] = V
        out[f"bf_z_{n}"] = z
        out[f"bf_B_{n}"] = fs.bfly(n, z, V)
        out[f"bf_BT_{n}"] = fs.bflyT(n, z, V)
        out[f"bf_B2_{n}"] = fh.bfly_levels(n, z, V, 2, n)
        out[f"bf_BT2_{n}"] = fh.bflyT_levels(n, z, V, 2, n)
        out[f"bf_B11_{n}"] = fh.bfly_levels(n, z, V, 1, 1)
        out[f"bf_BT11_{n}"] = fh.bflyT_levels(n, z, V, 1, 1)
        zc = np.ascontiguousarray(z)
        for lo, hi in ((1, n), (2, n), (1, 1), (2, n - 1), (3, n)):
            for tr in (0, 1):
                X = V.copy()
                fc.lib().bfly_rows(n, K, fc._ptr(zc), fc._ptr(X), lo, hi, tr, 1)
                out[f"cpp_bfly_{n}_{lo}_{hi}_{tr}"] = X
        # cheb_rows with power-iteration bounds and default degrees, levels 1..n and 2..n
        tau = 0.2 * N
        for lo in (1, 2):
            lam_all = fc.power_lam_max(n, zall, lo, threads=1)
            out[f"power_{n}_{lo}"] = lam_all
            lam = np.maximum(fo._sym(lam_all), 1.0)[rows]
            kap = 1.0 + lam / tau
            rate = (np.sqrt(kap) - 1) / (np.sqrt(kap) + 1)
            deg = np.maximum(2, np.ceil(np.log(0.1 / 2.0) / np.log(np.maximum(rate, 1e-12)))).astype(np.int32)
            c, a = fs.cheb_coeffs(lam, tau)
            Y = rng.standard_normal((K, N)) + 1j * rng.standard_normal((K, N))
            Z = np.empty_like(Y)
            steps = fc.ctypes.c_longlong(0)
            fc.lib().cheb_rows(
                n, K, fc._ptr(zc), fc._ptr(np.ascontiguousarray(deg)), fc._ptr(np.ascontiguousarray(a)),
                fc._ptr(np.ascontiguousarray(c)), tau, fc._ptr(Y), fc._ptr(Z), lo, n, 1, fc.ctypes.byref(steps),
            )
            out[f"cheb_lam_{n}_{lo}"] = lam
            out[f"cheb_deg_{n}_{lo}"] = deg
            out[f"cheb_Y_{n}_{lo}"] = Y
            out[f"cheb_Z_{n}_{lo}"] = Z
            out[f"cheb_steps_{n}_{lo}"] = np.array(steps.value)
            out[f"cheb_poly_{n}_{lo}"] = fh.poly_apply_levels(n, z, Y, lam, tau, deg, lo, n)

    # ---- certified bounds (cpp/oblique.cpp:108-130, fasthybrid.py:134-150)
    for n in (4, 6, 8):
        oms = 2 * np.pi * np.fft.fftfreq(2 << n)
        for lo in (1, 2):
            out[f"cert_cpp_{n}_{lo}"] = fc.cert_lam_max(n, oms, lo, 1)
            out[f"cert_np_{n}_{lo}"] = np.array([fh.cert_rowsum_levels(n, om, lo) for om in oms])
    out["explicit_6"] = fc.explicit_lam_max(6, 2 * np.pi * np.fft.fftfreq(128))

    # ---- level-1 stencils (fasthybrid.py:81-130)
    for n in (3, 5):
        N = 1 << n
        x = np.random.default_rng(300 + n).standard_normal((N, N))
        out[f"st_x_{n}"] = x
        out[f"st_G1_{n}"] = fh.G1_apply(x)
        out[f"st_Pi_{n}"] = fh.Pi_apply(x)
        out[f"st_lorr_{n}"] = fh.lorr_inv(x)
        out[f"st_g1inv_{n}"] = fh.g1_inv(x)

    # ---- packed inverses (fastops.py:261-338) and the C++ engine (fastcpp.py:137-169)
    for n in (4, 6):
        N = 1 << n
        rng = np.random.default_rng(1)
        x = rng.standard_normal((N, N))
        b = ac.adrt(n, x)
        out[f"inv_x_{n}"] = x
        out[f"inv_b_{n}"] = b
        for name, ctor in (
            ("lp", lambda n=n: fo.FastLp(n, eps_in=0.1, threads=1)),
            ("hyb", lambda n=n: fo.FastHybrid(n, eps_in=0.1, threads=1)),
            ("hybd8", lambda n=n: fo.FastHybrid(n, eps_in=0.1, threads=1, dense_cap=8)),
            ("lpd8", lambda n=n: fo.FastLp(n, eps_in=0.1, threads=1, dense_cap=8)),
            ("hyblorr", lambda n=n: fo.FastHybrid(n, eps_in=0.1, threads=1, precond="lorr")),
        ):
            P = ctor()
            k = f"{name}_{n}"
            out[f"inv_lam_{k}"] = P.lam_max
            out[f"inv_deg_{k}"] = P.deg
            out[f"inv_outer_{k}"] = np.array([P.lo, P.hi, P.outer_deg])
            G = P.Gh if name.startswith("hyb") else P.frame_window
            out[f"inv_G_{k}"] = G(x)
            out[f"inv_bp_{k}"] = P.backproject(b)
            P.eng.count = [0]
            out[f"inv_apply_{k}"] = P.apply(b)
            out[f"inv_count_{k}"] = np.array(P.eng.count[0])
            out[f"inv_ndense_{k}"] = np.array(P.eng.n_dense)

    # ---- L_p in FP64 at N = 64 with degrees capped at p = 16 on a noisy ellipse phantom (C++ engine)
    n, p = 6, 16
    N = 1 << n

    class CappedLpCpp(fc.FastLpCpp):
        def _degrees(self, lam_max, eps_in, dense_cap=None, p_levels=(1, None)):
            fo._Base._degrees(self, lam_max, eps_in, dense_cap, p_levels)
            self.deg = np.minimum(self.deg, p)
            self.eng = self.engine_cls(self.n, self.z, self.deg, self.lam_max, self.tau, self.threads, copies=2,
                                       dense_cap=dense_cap, p_levels=p_levels)

    x0 = ph.ellipse_phantom(N, seed=0)
    b0 = ph.add_noise(ac.adrt(n, x0), 1e-3, seed=1)
    P = CappedLpCpp(n, eps_in=0.1, threads=1)
    out["c0_x"] = x0
    out["c0_b"] = b0
    out["c0_lam"] = P.lam_max
    out["c0_deg"] = P.deg
    out["c0_outer"] = np.array([P.lo, P.hi, P.outer_deg])
    out["c0_apply"] = P.apply(b0)
    out["c0_bp"] = P.backproject(b0)

    # ---- the unpacked NumPy references (fastspec.py:90-215, fasthybrid.py:153-309)
    n = 3
    N = 1 << n
    x = np.random.default_rng(5).standard_normal((N, N))
    b = ac.adrt(n, x)
    S = fs.FastSpectralInverse(n, 0.2, eps=1e-10)
    out["spec_x"] = x
    out["spec_b"] = b
    out["spec_lam"] = S.lam_max
    out["spec_deg"] = S.deg
    out["spec_outer"] = np.array([S.lo, S.hi, S.outer_deg])
    out["spec_fw"] = S.frame_window(x)
    out["spec_apply"] = S.apply(b)
    H = fh.FastHybridInverse(n, 0.2, eps=1e-10)
    out["fhyb_lam"] = H.lam_max
    out["fhyb_deg"] = H.deg
    out["fhyb_outer"] = np.array([H.lo, H.hi, H.outer_deg])
    out["fhyb_Gh"] = H.Gh(x)
    out["fhyb_apply"] = H.apply(b)

    path = os.path.join(HERE, "reference_vectors.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path}: {len(out)} arrays, {os.path.getsize(path) / 1e6:.2f} MB")


if __name__ == "__main__":
    main()
