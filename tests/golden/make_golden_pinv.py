"""Generate tests/golden/pinv_gram_vectors.npz from the reference implementation (dsrim/adrt-pinv).

Run from the repository root with the path of a read-only reference checkout (no default):

    python tests/golden/make_golden_pinv.py REF       (or ADRT_PINV_REF=REF python tests/golden/make_golden_pinv.py)

Sources of every array:
  * pinv.cgls / pinv.pcg_normal / pinv.pinv_dense (pinv.py:23-88) and adrtcore (adrtcore.adrt, adrt_T, adrt_dense)
    of the reference, imported from a temporary copy;
  * gram_freq: the C++ kernel of patches/adrt-gram-freq.patch (the added file src/adrt/adrt_cdefs_gram.hpp), cut out
    of the patch text into a temporary directory and compiled with g++ beside a small stand-in for the few helpers it
    takes from the absent `adrt` package (a span element accessor, a size_t literal, the restrict and OpenMP macros),
    then called through ctypes on seeded inputs, in both of its precisions;
  * gram: R^T R a from the reference's adrtcore (adrt_T of adrt), the identity the patch's own tests check;
  * lstsq_cheb: the least-squares solution from the reference's dense ADRT (np.linalg.lstsq) and the extreme
    eigenvalues of its Gram matrix, as the patch's own test builds them.
Inputs made here: seeded Gaussians and this package's seeded ellipse phantoms. Sizes stay small (N <= 64).
"""

import ctypes
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import _import_reference, _load_phantoms  # noqa: E402

SHIM = r"""
#pragma once
#include <cstddef>
#include <span>
#define ADRT_RESTRICT __restrict__
#define ADRT_OPENMP(x)
namespace adrt { namespace _common {
template <std::size_t I, typename S> constexpr auto get(const S& s) { return s[I]; }
} }
constexpr std::size_t operator""_uz(unsigned long long v) { return static_cast<std::size_t>(v); }
"""

WRAP = r"""
#include <complex>
#include <span>
#include "adrt_cdefs_gram.hpp"
extern "C" void gram_freq_f64(const double* a, size_t b, size_t r, size_t n, const double* om, double* out) {
    const std::array<size_t, 3> s{b, r, n};
    adrt::gram_freq(reinterpret_cast<const std::complex<double>*>(a), std::span<const size_t, 3>(s), om,
                    reinterpret_cast<std::complex<double>*>(out));
}
extern "C" void gram_freq_f32(const float* a, size_t b, size_t r, size_t n, const float* om, float* out) {
    const std::array<size_t, 3> s{b, r, n};
    adrt::gram_freq(reinterpret_cast<const std::complex<float>*>(a), std::span<const size_t, 3>(s), om,
                    reinterpret_cast<std::complex<float>*>(out));
}
"""


def _patch_file(patch_text, path):
    """The added file `path` of a git patch, its lines without the leading '+'."""
    lines, on = [], False
    for line in patch_text.splitlines():
        if line.startswith("+++ b/"):
            on = line[len("+++ b/"):] == path
            continue
        if on and line.startswith("diff --git"):
            break
        if on and line.startswith("+"):
            lines.append(line[1:])
    return "\n".join(lines) + "\n"


def _build_gram_freq(ref):
    tmp = tempfile.mkdtemp(prefix="adrt_gram_")
    with open(os.path.join(ref, "patches", "adrt-gram-freq.patch")) as f:
        text = f.read()
    with open(os.path.join(tmp, "adrt_cdefs_gram.hpp"), "w") as f:
        f.write(_patch_file(text, "src/adrt/adrt_cdefs_gram.hpp"))
    with open(os.path.join(tmp, "adrt_cdefs_common.hpp"), "w") as f:
        f.write(SHIM)
    with open(os.path.join(tmp, "wrap.cpp"), "w") as f:
        f.write(WRAP)
    so = os.path.join(tmp, "libgram.so")
    subprocess.check_call(["g++", "-O2", "-std=c++20", "-fPIC", "-shared", "-I", tmp, "-o", so,
                           os.path.join(tmp, "wrap.cpp")])
    lib = ctypes.CDLL(so)
    P, S = ctypes.c_void_p, ctypes.c_size_t
    for name in ("gram_freq_f64", "gram_freq_f32"):
        getattr(lib, name).argtypes = [P, S, S, S, P, P]
        getattr(lib, name).restype = None
    return lib, tmp


def _call_gram_freq(lib, a, om):
    a = np.ascontiguousarray(a)
    out = np.empty_like(a)
    fn = lib.gram_freq_f64 if a.dtype == np.complex128 else lib.gram_freq_f32
    p = lambda x: x.ctypes.data_as(ctypes.c_void_p)
    fn(p(a), a.shape[0], a.shape[1], a.shape[2], p(np.ascontiguousarray(om)), p(out))
    return out


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ADRT_PINV_REF")
    if not ref:
        sys.exit("usage: make_golden_pinv.py REF (the path of a reference checkout; or set ADRT_PINV_REF)")
    ac, _, _, _, _ = _import_reference(ref)
    import pinv  # noqa: E402  (the reference's module, on the path after _import_reference)

    ph = _load_phantoms()
    out = {}

    # ---- CGLS (pinv.py:23-48): noisy phantoms, tolerances and iteration caps as the experiments use them
    for n, tol, maxit in ((3, 1e-10, 2000), (4, 1e-10, 2000), (5, 1e-8, 2000), (6, 1e-8, 3000), (4, 1e-12, 7)):
        N = 1 << n
        x = ph.ellipse_phantom(N, seed=40 + n)
        b = ph.add_noise(ac.adrt(n, x), 1e-2, seed=50 + n)
        key = f"{n}_{maxit}"
        xc, h = pinv.cgls(n, b, tol=tol, maxit=maxit)
        out[f"cgls_b_{key}"], out[f"cgls_x_{key}"], out[f"cgls_hist_{key}"] = b, xc, h
        out[f"cgls_tol_{key}"] = np.array(tol)
    # a nonzero start
    n = 4
    N = 1 << n
    b = np.random.default_rng(60).standard_normal((4, 2 * N - 1, N))
    x0 = np.random.default_rng(61).standard_normal((N, N))
    xc, h = pinv.cgls(n, b, tol=1e-10, maxit=2000, x0=x0)
    out["cgls_x0_b"], out["cgls_x0_x0"], out["cgls_x0_x"], out["cgls_x0_hist"] = b, x0, xc, h

    # ---- PCG on the normal equations (pinv.py:51-82), identity and a scaled-identity preconditioner
    for n in (3, 4, 5):
        N = 1 << n
        b = ph.add_noise(ac.adrt(n, ph.ellipse_phantom(N, seed=70 + n)), 1e-2, seed=80 + n)
        for tag, M in (("id", lambda v: v), ("sc", lambda v, N=N: v / (4.0 * N))):
            xp, h = pinv.pcg_normal(n, b, M, tol=1e-10, maxit=2000)
            out[f"pcg_b_{n}"], out[f"pcg_x_{tag}_{n}"], out[f"pcg_hist_{tag}_{n}"] = b, xp, h

    # ---- dense pseudoinverse (pinv.py:85-88) and the reference's own self-check (pinv.py:91-104)
    for n in (1, 2, 3):
        out[f"pinv_dense_{n}"] = pinv.pinv_dense(n)

    # ---- gram_freq: the patch's C++ kernel, compiled from the patch text
    lib, tmp = _build_gram_freq(ref)
    try:
        for n in range(1, 7):
            N = 1 << n
            rng = np.random.default_rng(90 + n)
            rows = 2 * N
            a = rng.standard_normal((3, rows, N)) + 1j * rng.standard_normal((3, rows, N))
            om = 2 * np.pi * np.fft.fftfreq(rows)
            out[f"gf_a_{n}"], out[f"gf_om_{n}"] = a, om
            out[f"gf_f64_{n}"] = _call_gram_freq(lib, a.astype(np.complex128), om.astype(np.float64))
            out[f"gf_f32_{n}"] = _call_gram_freq(lib, a.astype(np.complex64), om.astype(np.float32))
        # arbitrary frequencies (not only the offset grid)
        n = 5
        N = 1 << n
        rng = np.random.default_rng(99)
        a = rng.standard_normal((2, 7, N)) + 1j * rng.standard_normal((2, 7, N))
        om = rng.uniform(-np.pi, np.pi, 7)
        out["gf_a_any"], out["gf_om_any"] = a, om
        out["gf_f64_any"] = _call_gram_freq(lib, a, om)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)

    # ---- gram: R^T R a from the reference's spatial transform
    for n in range(1, 7):
        N = 1 << n
        a = np.random.default_rng(100 + n).standard_normal((N, N))
        out[f"gram_a_{n}"], out[f"gram_{n}"] = a, ac.adrt_T(n, ac.adrt(n, a))

    # ---- lstsq_cheb: the dense least-squares solution and the Gram matrix's extreme eigenvalues
    for n in (2, 3, 4):
        N = 1 << n
        rng = np.random.default_rng(N)
        mat = ac.adrt_dense(n)
        eig = np.linalg.eigvalsh(mat.T @ mat)
        b = ac.adrt(n, rng.standard_normal((N, N))) + 0.1 * rng.standard_normal((4, 2 * N - 1, N))
        out[f"ls_b_{n}"] = b
        out[f"ls_eig_{n}"] = np.array([eig[0], eig[-1]])
        out[f"ls_x_{n}"] = np.linalg.lstsq(mat, b.ravel(), rcond=None)[0].reshape(N, N)

    path = os.path.join(HERE, "pinv_gram_vectors.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {len(out)} arrays to {path}")


if __name__ == "__main__":
    main()
