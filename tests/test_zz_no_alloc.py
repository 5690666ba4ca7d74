"""The allocation-free bfly_rows (adrt_bfly_rows_noalloc) against the regular host-pointer bfly_rows.

Some callers cannot allocate device memory: a process that has given the whole GPU to its own memory pool, code that
must not let cudaMalloc/cudaFree synchronize the device, threads that may not enter the CUDA allocator. For them the
library offers bfly_rows on device pointers with its scratch in a fixed device array. This checks, through the C ABI,
two calls in a row (different sizes and directions, the second reusing the array the first left behind) against the
regular entry point and against the reference's own outputs (golden vectors), to the FP64 tolerance of the other
row-kernel tests, that the device's free memory does not change across calls, and that oversized calls are refused.
Collected last on purpose, so that a failure here comes after every other test has run."""

import ctypes

import numpy as np
import pytest

from conftest import max_rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib(pkg):
    import __graft_entry__ as ge

    ge.build()
    lib = pkg._lib.load()
    P, I = ctypes.c_void_p, ctypes.c_int
    lib.adrt_bfly_rows_noalloc.argtypes = [I, I, P, P, I, I, I, P]
    lib.adrt_bfly_rows_noalloc.restype = I
    return lib


def _host_ref(lib, n, z, V, lo, hi, tr):
    X = V.copy()
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    assert lib.bfly_rows(n, len(z), p(np.ascontiguousarray(z)), p(X), lo, hi, tr, 1) == 0, lib.adrt_last_error()
    return X


def test_noalloc_matches_bfly_rows_two_calls(lib):
    import torch

    for n, lo, hi, tr, seed in ((8, 2, 8, 0, 1), (6, 1, 6, 1, 2)):
        N, L = 1 << n, 2 << n
        rng = np.random.default_rng(seed)
        z = np.exp(2j * np.pi * np.arange(L) / L)
        V = rng.standard_normal((L, N)) + 1j * rng.standard_normal((L, N))
        zd = torch.from_numpy(z).cuda()
        Xd = torch.from_numpy(V).cuda()
        torch.cuda.synchronize()
        rc = lib.adrt_bfly_rows_noalloc(n, L, zd.data_ptr(), Xd.data_ptr(), lo, hi, tr, None)
        assert rc == 0, lib.adrt_last_error()
        torch.cuda.synchronize()
        assert max_rel(Xd.cpu().numpy(), _host_ref(lib, n, z, V, lo, hi, tr)) < 1e-12


def test_noalloc_matches_reference_golden_and_allocates_nothing(lib, golden):
    """Against the reference's own compiled bfly_rows (golden cpp_bfly_* vectors, cpp/oblique.cpp:56-70), two
    calls in a row per size, and the device's free memory is the same before and after the calls (the entry point
    allocates nothing)."""
    import torch

    # one call first, so that the library's lazily loaded device code and the array are resident before the
    # free-memory reading (the CUDA runtime loads a module on its first use, which takes device memory once)
    V4 = torch.from_numpy(np.ascontiguousarray(golden["bf_V_4"])).cuda()
    z4 = torch.from_numpy(np.ascontiguousarray(golden["bf_z_4"])).cuda()
    assert lib.adrt_bfly_rows_noalloc(4, V4.shape[0], z4.data_ptr(), V4.data_ptr(), 1, 4, 0, None) == 0
    torch.cuda.synchronize()
    for n in (4, 6):
        V = golden[f"bf_V_{n}"]
        z = np.ascontiguousarray(golden[f"bf_z_{n}"])
        zd = torch.from_numpy(z).cuda()
        cases = [(lo, hi, tr) for lo, hi in ((1, n), (2, n - 1)) for tr in (0, 1)]
        Xs = [torch.from_numpy(np.ascontiguousarray(V)).cuda() for _ in cases]
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        for (lo, hi, tr), Xd in zip(cases, Xs):
            rc = lib.adrt_bfly_rows_noalloc(n, V.shape[0], zd.data_ptr(), Xd.data_ptr(), lo, hi, tr, None)
            assert rc == 0, lib.adrt_last_error()
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free0
        for (lo, hi, tr), Xd in zip(cases, Xs):
            assert max_rel(Xd.cpu().numpy(), golden[f"cpp_bfly_{n}_{lo}_{hi}_{tr}"]) < 1e-12, (n, lo, hi, tr)


def test_noalloc_rejects_oversized_calls(lib):
    import torch

    n, K = 11, 512  # 512 rows x 1025 twiddles x 16 B > 4 MiB
    zd = torch.ones(K, dtype=torch.complex128, device="cuda")
    Xd = torch.zeros((K, 1 << n), dtype=torch.complex128, device="cuda")
    assert lib.adrt_bfly_rows_noalloc(n, K, zd.data_ptr(), Xd.data_ptr(), 1, n, 0, None) == 1
    assert b"scratch" in lib.adrt_last_error()
