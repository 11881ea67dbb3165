"""gpi_project_gb300 -- SOFI2D's time-stepping hot path as sm_103a CUDA kernels.

The native library (libsofigpu.so, C ABI in include/sofigpu.h) is the product;
this package holds its in-tree build and a thin Python face of the same
interface (``TimeLoop``) used by tests and the benchmark.
"""
from ._native import SofiConfig, SofiError, UnstableError, load  # noqa: F401
from .timeloop import COMP, WEQ, TimeLoop, device_bytes, make_config  # noqa: F401

__all__ = ["TimeLoop", "make_config", "SofiConfig", "SofiError", "UnstableError", "load", "device_bytes"]
