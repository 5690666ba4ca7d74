"""ctypes binding of libadrt_pinv_gb300.so (the C ABI in include/adrt_pinv_gb300.h).

The library is loaded from this directory; there is no fallback: if it is missing or fails to load, every GPU
entry point raises. Device-pointer calls take torch CUDA tensors (data_ptr) and the current torch stream.
"""

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libadrt_pinv_gb300.so")

F32, F64, I32, I64, F32X2 = 0, 1, 2, 3, 4
OS_SHARED = 0x100  # band flag of adrt_outer_step: the shared-memory form
OP_B, OP_BT, OP_M, OP_P = 0, 1, 2, 3
MAX_OPS = 8
STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of device memory", 4: "unsupported"}


class RowJob(ctypes.Structure):
    """Mirror of `adrt_row_job` (include/adrt_pinv_gb300.h)."""

    _fields_ = [
        ("dtype", ctypes.c_int),
        ("n", ctypes.c_int),
        ("nimg", ctypes.c_int),
        ("nsel", ctypes.c_int),
        ("img_stride", ctypes.c_int64),
        ("X", ctypes.c_void_p),
        ("rows", ctypes.c_void_p),
        ("freq_mod", ctypes.c_int),
        ("roots", ctypes.c_void_p),
        ("twtab", ctypes.c_void_p),
        ("deg", ctypes.c_void_p),
        ("coef", ctypes.c_void_p),
        ("coef_stride", ctypes.c_int),
        ("tau", ctypes.c_double),
        ("nops", ctypes.c_int),
        ("op", ctypes.c_int * MAX_OPS),
        ("lo", ctypes.c_int * MAX_OPS),
        ("hi", ctypes.c_int * MAX_OPS),
        ("counter", ctypes.c_void_p),
        ("grid", ctypes.c_int),
    ]


class CglsState(ctypes.Structure):
    """Mirror of `adrt_cgls` (include/adrt_pinv_gb300.h)."""

    _fields_ = [("n", ctypes.c_int), ("nimg", ctypes.c_int), ("maxit", ctypes.c_int), ("nblk", ctypes.c_int),
                ("tol", ctypes.c_double)] + [(f, ctypes.c_void_p) for f in
                                             ("x", "p", "s", "r", "q", "scratch", "partial", "scal", "it", "active",
                                              "hist")]


class PcgState(ctypes.Structure):
    """Mirror of `adrt_pcg` (include/adrt_pinv_gb300.h)."""

    _fields_ = [("n", ctypes.c_int), ("nimg", ctypes.c_int), ("maxit", ctypes.c_int), ("nblk", ctypes.c_int),
                ("tol", ctypes.c_double)] + [(f, ctypes.c_void_p) for f in
                                             ("x", "r", "z", "p", "q", "t", "scratch", "partial", "scal", "it",
                                              "active", "hist")]


_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_L = ctypes.c_longlong
PROTOTYPES = {
    "bfly_rows": [_I, _I, _P, _P, _I, _I, _I, _I],
    "cheb_rows": [_I, _I, _P, _P, _P, _P, _D, _P, _P, _I, _I, _I, _P],
    "cert_rowsum": [_I, _I, _P, _I, _P, _I],
    "omp_max_threads": [],
    "adrt_last_error": [],
    "adrt_abi_version": [],
    "adrt_launch_count": [],
    "adrt_fp32_probe": [_I, _I, _I, _P, _P],
    "adrt_rows_run": [ctypes.POINTER(RowJob), _P],
    "adrt_rows_ff_run": [ctypes.POINTER(RowJob), _P],
    "adrt_rows_multi_code": [ctypes.POINTER(RowJob)],
    "adrt_rows_lanes_per_row": [_I],
    "adrt_rows_run_multi": [_P, _P, _P, _I, _P, _I, _P],
    "adrt_twiddle_table": [_I, _I, _I, _P, _P, _P],
    "adrt_power_rows": [_I, _I, _I, _P, _P, _I, _I, _D, _P, _P, _P],
    "adrt_cert_rowsum_dev": [_I, _I, _P, _I, _P, _P],
    "adrt_pack_fft": [_I, _I, _I, _I, _I, _P, _L, _P, _P, _I, _P],
    "adrt_ifft_unpack": [_I, _I, _I, _P, _P, _P, _P, _P, _I, _P],
    "adrt_resid": [_I, _I, _I, _I, _P, _P, _P, _P, _P, _P],
    "adrt_g1_step": [_I, _I, _I, _P, _P, _P, _P, _D, _D, _D, _P],
    "adrt_lorr": [_I, _I, _I, _P, _P, _P],
    "adrt_outer_update": [_I, _I, _I, _P, _P, _P, _I, _P, _D, _D, _D, _P, _P],
    "adrt_sum3": [_I, _I, _I, _P, _P, _P, _P, _I, _P],
    "adrt_outer_step": [_I, _I, _I, _I, _P, _P, _P, _P, _P, _P, _P, _D, _D, _D, _I, _I, _P, _P, _I, _P],
    "adrt_outer_step_max_n": [_I],
    "adrt_outer_step_ff": [_I, _I, _P, _P, _P, _P, _P, _P, _P, _D, _D, _D, _I, _I, _P, _P, _I, _P],
    "adrt_ff_to_f64": [_I, _I, _P, _P, _P],
    "adrt_dense_rows": [_I, _I, _I, _I, _P, _P, _P, ctypes.c_longlong, _P, _P, _I, _I, _P],
    "adrt_dense_split": [_I, _I, _P, _P, _P],
    "adrt_forward": [_I, _I, _I, _P, _P, _P, _P],
    "adrt_transpose": [_I, _I, _I, _P, _P, _P, _P],
    "adrt_cgls_start": [ctypes.POINTER(CglsState), _P, _P],
    "adrt_cgls_iterate": [ctypes.POINTER(CglsState), _I, _P],
    "adrt_pcg_start": [ctypes.POINTER(PcgState), _P, _P],
    "adrt_pcg_rho": [ctypes.POINTER(PcgState), _P],
    "adrt_pcg_step": [ctypes.POINTER(PcgState), _P],
    "adrt_pcg_direction": [ctypes.POINTER(PcgState), _P],
}

_lib = None


def load(path=LIB_PATH):
    """Load the library (once). Raises if it has not been built (`__graft_entry__.build()`)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(path)
    for name, args in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = {"adrt_last_error": ctypes.c_char_p, "adrt_launch_count": ctypes.c_longlong}.get(name, ctypes.c_int)
    _lib = lib
    return lib


def check(rc, what):
    if rc != 0:
        msg = load().adrt_last_error().decode(errors="replace")
        raise RuntimeError(f"{what} failed ({STATUS.get(rc, rc)}): {msg}")


def call(name, *args):
    """Call a C ABI function and raise on a non-zero status."""
    check(getattr(load(), name)(*args), name)


def ptr(t):
    """Device pointer of a torch tensor (or None -> NULL)."""
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def stream_handle():
    import torch

    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def dtype_code(dt):
    import torch

    return {torch.float32: F32, torch.float64: F64, torch.int32: I32, torch.int64: I64,
            torch.complex64: F32, torch.complex128: F64}[dt]
