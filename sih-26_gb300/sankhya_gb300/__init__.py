"""GB300-native restarted PDHG for SANKHYA LPs.

The engine is CUDA (sm_103a) behind the C ABI of include/sankhya_gb300.h; this package is
its Python face: ``solve_pdhg_gpu`` (the reference seam's contract), ``PdhgEngine`` (load
once, solve many times), the LP container and the synthetic planted-optimum generators.
"""
from .model import LP, from_dense  # noqa: F401

__all__ = ["LP", "from_dense", "capi", "lpgen", "build"]


def __getattr__(name):
    # Import the ctypes layers lazily so that importing the package never needs a built
    # library (the build step itself lives in this package).
    if name in ("capi", "lpgen", "build"):
        import importlib

        return importlib.import_module(f"{__name__}.{name}")
    if name in ("solve_pdhg_gpu", "PdhgEngine", "EngineError"):
        from . import capi

        return getattr(capi, name)
    raise AttributeError(name)
