"""Dense low-frequency rows (adrt_dense_rows): tensor-core 3xTF32 kernel and CUDA-core kernel against an FP64
NumPy product, through the C ABI. 3xTF32 with per-chunk promotion to FP32 registers keeps FP32 accuracy: the
norm-wise relative error of every output row is at most 5e-7 (1e-6 for the CUDA-core kernel's sequential sums)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,nimg,nrows", [(8, 64, 6), (6, 5, 3), (9, 20, 2), (7, 100, 2)])
def test_dense_rows_tc_and_simt(pkg, n, nimg, nrows):
    import torch

    C = pkg._lib
    C.load()
    N, R = 1 << n, 16
    rng = np.random.default_rng(n)
    W = (rng.standard_normal((nrows, N, N)) + 1j * rng.standard_normal((nrows, N, N))) / np.sqrt(N)
    Y = rng.standard_normal((nimg, R, N)) + 1j * rng.standard_normal((nimg, R, N))
    rows = np.array(sorted(rng.choice(R, nrows, replace=False)), dtype=np.int32)
    ref = Y.copy()
    for i, r in enumerate(rows):
        ref[:, r, :] = Y[:, r, :] @ W[i].T
    for use_tc, tile in ((1, 0), (1, 16), (1, 64), (0, 0)):
        Wd = torch.from_numpy(W).to("cuda", torch.complex64)
        Yd = torch.from_numpy(Y).to("cuda", torch.complex64)
        rd = torch.from_numpy(rows).cuda()
        Zd = torch.empty((nrows, nimg, N), dtype=torch.complex64, device="cuda")
        err = torch.zeros(1, dtype=torch.int32, device="cuda")
        C.call("adrt_dense_rows", C.F32, n, nimg, nrows, C.ptr(rd), C.ptr(Wd), C.ptr(Yd), R * N, C.ptr(Zd), C.ptr(err),
               use_tc, tile, C.stream_handle())
        torch.cuda.synchronize()
        assert int(err.item()) == 0
        out = Yd.cpu().numpy()
        for r in range(R):
            e = np.linalg.norm(out[:, r, :] - ref[:, r, :]) / np.linalg.norm(ref[:, r, :])
            assert e < (5e-7 if use_tc else 1e-6), (use_tc, r, e)  # sequential FP32 sum over K = 2N on CUDA cores
    # FP64 CUDA-core path
    Wd = torch.from_numpy(W).cuda()
    Yd = torch.from_numpy(Y).cuda()
    Zd = torch.empty((nrows, nimg, N), dtype=torch.complex128, device="cuda")
    C.call("adrt_dense_rows", C.F64, n, nimg, nrows, C.ptr(torch.from_numpy(rows).cuda()), C.ptr(Wd), C.ptr(Yd), R * N,
           C.ptr(Zd), None, 0, 0, C.stream_handle())
    torch.cuda.synchronize()
    assert np.abs(Yd.cpu().numpy() - ref).max() / np.abs(ref).max() < 1e-13


@pytest.mark.parametrize("n,nimg,nrows,tile", [(8, 64, 6, 0), (8, 100, 3, 0), (7, 40, 4, 32), (9, 20, 2, 16),
                                               (8, 64, 5, 64), (10, 33, 1, 0)])
def test_dense_rows_presplit_complex_blocked(pkg, n, nimg, nrows, tile):
    """The complex-blocked tensor-core kernel on operators pre-split by adrt_dense_split (use_tc = 3: Re / Im W in
    TF32 hi + lo, z = (ReW Re y - ImW Im y) + i (ImW Re y + ReW Im y), each product 3xTF32 with per-chunk promotion)
    against the FP64 product: every output row within 5e-7 (norm-wise), images beyond nimg untouched; partial image
    tiles (nimg not a multiple of the tile) included."""
    import torch

    C = pkg._lib
    C.load()
    N, R = 1 << n, 12
    rng = np.random.default_rng(n + nimg)
    W = (rng.standard_normal((nrows, N, N)) + 1j * rng.standard_normal((nrows, N, N))) / np.sqrt(N)
    Y = rng.standard_normal((nimg, R, N)) + 1j * rng.standard_normal((nimg, R, N))
    rows = np.array(sorted(rng.choice(R, nrows, replace=False)), dtype=np.int32)
    ref = Y.copy()
    for i, r in enumerate(rows):
        ref[:, r, :] = Y[:, r, :] @ W[i].T
    Wd = torch.from_numpy(W).to("cuda", torch.complex64)
    Ws = torch.empty((nrows, 4 * N * N), dtype=torch.float32, device="cuda")
    assert C.load().adrt_dense_split(n, nrows, C.ptr(Wd), C.ptr(Ws), C.stream_handle()) == 0
    Yd = torch.from_numpy(Y).to("cuda", torch.complex64)
    rd = torch.from_numpy(rows).cuda()
    Zd = torch.empty((nrows, nimg, N), dtype=torch.complex64, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    C.call("adrt_dense_rows", C.F32, n, nimg, nrows, C.ptr(rd), C.ptr(Ws), C.ptr(Yd), R * N, C.ptr(Zd), C.ptr(err), 3,
           tile, C.stream_handle())
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    out = Yd.cpu().numpy()
    for r in range(R):
        e = np.linalg.norm(out[:, r, :] - ref[:, r, :]) / np.linalg.norm(ref[:, r, :])
        assert e < 5e-7, (r, e)
    # the split table: tile element (o, i) of (row, 128-row block, 16-column chunk); hi + lo (two TF32 values, about
    # 22 significant bits together) reproduces the FP32 entry to 2^-21
    Wh = Ws.cpu().numpy().reshape(nrows, N // 128, N // 16, 4, 2048).astype(np.float64)
    o, i = 130 % N, 37
    t = Wh[0, o // 128, i // 16]
    off = ((o % 128) // 8 * 4 + (i % 16) // 4) * 32 + (o % 8) * 4 + i % 4
    w32 = np.complex64(W[0, o, i])
    assert abs(t[0, off] + t[1, off] - float(w32.real)) <= 2.0 ** -21 * abs(float(w32.real))
    assert abs(t[2, off] + t[3, off] - float(w32.imag)) <= 2.0 ** -21 * abs(float(w32.imag))


@pytest.mark.parametrize("n,nimg,nrows", [(6, 1, 3), (8, 3, 5), (9, 8, 2), (11, 2, 1), (7, 13, 3), (10, 16, 1)])
def test_dense_rows_streaming_small_batch(pkg, n, nimg, nrows):
    """The small-batch streaming kernel (use_tc = 2, operators transposed, passes of 8 images) against the FP64
    product; it refuses more than 16 images."""
    import torch

    C = pkg._lib
    C.load()
    N, R = 1 << n, 8
    rng = np.random.default_rng(n + nimg)
    W = (rng.standard_normal((nrows, N, N)) + 1j * rng.standard_normal((nrows, N, N))) / np.sqrt(N)
    Y = rng.standard_normal((nimg, R, N)) + 1j * rng.standard_normal((nimg, R, N))
    rows = np.array(sorted(rng.choice(R, nrows, replace=False)), dtype=np.int32)
    ref = Y.copy()
    for i, r in enumerate(rows):
        ref[:, r, :] = Y[:, r, :] @ W[i].T
    WT = torch.from_numpy(np.ascontiguousarray(W.transpose(0, 2, 1))).to("cuda", torch.complex64)
    Yd = torch.from_numpy(Y).to("cuda", torch.complex64)
    rd = torch.from_numpy(rows).cuda()
    Zd = torch.empty((nrows, nimg, N), dtype=torch.complex64, device="cuda")
    C.call("adrt_dense_rows", C.F32, n, nimg, nrows, C.ptr(rd), C.ptr(WT), C.ptr(Yd), R * N, C.ptr(Zd), None, 2, 0,
           C.stream_handle())
    out = Yd.cpu().numpy()
    for r in range(R):
        e = np.linalg.norm(out[:, r, :] - ref[:, r, :]) / np.linalg.norm(ref[:, r, :])
        assert e < 1e-6, (r, e)
    Z9 = torch.empty((nrows, 17, N), dtype=torch.complex64, device="cuda")
    Y9 = torch.zeros((17, R, N), dtype=torch.complex64, device="cuda")
    rc = C.load().adrt_dense_rows(C.F32, n, 17, nrows, C.ptr(rd), C.ptr(WT), C.ptr(Y9), R * N, C.ptr(Z9), None, 2, 0,
                                  C.stream_handle())
    assert rc != 0


@pytest.mark.parametrize("method", ["hybrid", "lp"])
def test_device_built_dense_operators_match_host(pkg, method):
    """Dense-row operators built on the device (FP64 row kernels on unit vectors + Cholesky, used for n >= 9) equal
    the host eigendecomposition form for every folding."""
    import numpy as np

    from adrt_pinv_gb300.device import dense_row_operator_device
    from adrt_pinv_gb300.plan import Plan

    n, N = 6, 64
    plan = Plan(method, n, np.full(2 * N, 50.0 * N), 0.2, 0.1, 1e-10, dense_cap=8)
    for key in [(a, b, c, d) for a in (0, 1) for b in (0, 1) for c in (0, 1) for d in (0, 1)]:
        ref = plan.dense_row_operator(*map(bool, key))
        got = np.concatenate([T.cpu().numpy() for _, T in
                              dense_row_operator_device(plan, *map(bool, key), device="cuda", chunk=37)])
        assert np.abs(got - ref).max() <= 1e-11 * np.abs(ref).max(), key
