"""GB300 (sm_103a) per-time-step solver core of DRD-Micro.

The CUDA library (csrc/, built into libdrd_gb300.so) is the product; this package is its
host-side mirror of the reference's subroutine interface (api.DRDContext) plus the input
builders used by the tests and the benchmark.
"""
from . import abi, layout  # noqa: F401

__all__ = ["abi", "layout"]
