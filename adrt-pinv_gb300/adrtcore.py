"""GPU ADRT in the reference's sinogram layout: drop-in for adrtcore.adrt / adrt_T (adrtcore.py:122-137).

Inputs may be NumPy or torch arrays, one image (N, N) / sinogram (4, 2N-1, N) or a batch with a leading axis.
The arithmetic type follows the reference unless given: float64 (adrtcore casts to float, adrtcore.py:106,124);
dtype=int32 / int64 gives the exact integer transform (sums only). NumPy in -> NumPy out, torch in -> torch out.
"""

import numpy as np
import torch

from . import _lib as C

_TORCH = {np.dtype("float32"): torch.float32, np.dtype("float64"): torch.float64, np.dtype("int32"): torch.int32,
          np.dtype("int64"): torch.int64}


def _prep(a, dtype, device):
    is_torch = isinstance(a, torch.Tensor)
    t = a if is_torch else torch.from_numpy(np.ascontiguousarray(np.asarray(a)))
    want = _TORCH[np.dtype(dtype)] if dtype is not None else torch.float64
    return is_torch, t.to(device=device, dtype=want).contiguous()


def _finish(out, is_torch, single):
    out = out[0] if single else out
    return out if is_torch else out.cpu().numpy()


def adrt(n, x, dtype=None, device="cuda"):
    """R x: (..., N, N) -> (..., 4, 2N-1, N)."""
    N = 1 << n
    is_torch, xt = _prep(x, dtype, device)
    single = xt.dim() == 2
    xt = xt.reshape(-1, N, N)
    B = xt.shape[0]
    out = torch.empty((B, 4, 2 * N - 1, N), dtype=xt.dtype, device=xt.device)
    scratch = torch.empty(2 * B * 4 * (2 * N - 1) * N, dtype=xt.dtype, device=xt.device)
    C.call("adrt_forward", C.dtype_code(xt.dtype), n, B, C.ptr(xt), C.ptr(out), C.ptr(scratch), C.stream_handle())
    return _finish(out, is_torch, single)


def adrt_T(n, b, dtype=None, device="cuda"):
    """R^T b: (..., 4, 2N-1, N) -> (..., N, N)."""
    N = 1 << n
    is_torch, bt = _prep(b, dtype, device)
    single = bt.dim() == 3
    bt = bt.reshape(-1, 4, 2 * N - 1, N)
    B = bt.shape[0]
    out = torch.empty((B, N, N), dtype=bt.dtype, device=bt.device)
    scratch = torch.empty(2 * B * 4 * (2 * N - 1) * N, dtype=bt.dtype, device=bt.device)
    C.call("adrt_transpose", C.dtype_code(bt.dtype), n, B, C.ptr(bt), C.ptr(out), C.ptr(scratch), C.stream_handle())
    return _finish(out, is_torch, single)


def mask_full(n):
    """Structurally non-zero sinogram entries (adrtcore.py:140-146), host boolean array."""
    N = 1 << n
    h = np.arange(2 * N - 1)[:, None] - (N - 1)
    return np.broadcast_to(h >= -np.arange(N)[None, :], (4, 2 * N - 1, N)).copy()
