"""GB300-native explicit oblique inverses of the ADRT: a drop-in for the fastops / fastcpp / adrtcore path of
dsrim/adrt-pinv, with every hot operation in hand-written sm_103a CUDA kernels (libadrt_pinv_gb300.so).

    from adrt_pinv_gb300 import FastHybridGpu
    H = FastHybridGpu(8, deg_cap=32)          # plan: power iteration + Lanczos on the GPU
    x = H.apply(b)                            # b: (4, 2N-1, N) or (B, 4, 2N-1, N), NumPy or CUDA tensor

Submodules: fastgpu (fastcpp drop-in), adrtcore (GPU ADRT), pinv (CGLS / PCG Moore-Penrose baselines), gram (the
row-wise normal operator and its Chebyshev least squares), plan, device (pipeline), serve (request server), uneven
(uneven batches in one graph), tune (autotuner), phantoms (seeded inputs).
"""

from . import phantoms  # noqa: F401
from . import plan  # noqa: F401
from .plan import Plan  # noqa: F401


def __getattr__(name):
    # torch-dependent modules load on first use so that host-only tooling does not import CUDA
    import importlib

    if name in ("fastgpu", "adrtcore", "device", "inverse", "stencils", "_lib", "build", "pinv", "gram", "serve",
                "uneven", "tune"):
        return importlib.import_module(f".{name}", __name__)
    if name in ("FastLpGpu", "FastHybridGpu", "power_lam_max", "cert_lam_max", "explicit_lam_max"):
        return getattr(importlib.import_module(".inverse", __name__), name)
    if name in ("Pipeline",):
        return getattr(importlib.import_module(".device", __name__), name)
    raise AttributeError(name)
