"""corrfunc_gb300 -- Corrfunc's gridded pair counting on one GB300 GPU.

Drop-in for the Corrfunc 2.5.3 pair-counting C API (include/corrfunc_gb300.h) and its Python
front ends: ``corrfunc_gb300.theory.{DD, DDrppi, DDsmu, wp, xi}`` and
``corrfunc_gb300.mocks.DDtheta_mocks``.  The counting runs in sm_103a CUDA kernels; there is no
CPU fallback.
"""
from . import _capi  # noqa: F401

__version__ = "2.5.3"


def library():
    """ctypes handle of libcorrfunc_gb300.so (raises if it has not been built)."""
    return _capi.library()


def set_precision(mode):
    """'fp32_refine' (default) or 'fp64' counting; both give identical pair counts."""
    m = {"fp32_refine": _capi.PRECISION_FP32_REFINE, "fp64": _capi.PRECISION_FP64}[mode]
    if library().cf_gpu_set_precision(m) != 0:
        raise RuntimeError("could not set precision")


def get_precision():
    return {0: "fp32_refine", 1: "fp64"}[library().cf_gpu_get_precision()]


def set_autotune(on):
    """Single-count autotuner for DD(r) and xi: the first count of each shape times the splits of
    the j lattice's columns and later counts of that shape use the fastest (counts are identical
    for every split).  Off by default; turning it off forgets the shapes."""
    library().cf_gpu_set_autotune(1 if on else 0)


def get_autotune():
    return bool(library().cf_gpu_get_autotune())


def last_stats():
    """Kernel statistics of the most recent call (CUDA-event times, pairs evaluated/refined)."""
    import ctypes
    s = _capi.GpuStats()
    library().cf_gpu_last_stats(ctypes.byref(s))
    return {k: getattr(s, k) for k, _ in s._fields_}
