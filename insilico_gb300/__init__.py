"""insilico_gb300 — GB300-native (sm_103a) stiffness/force assembly and Krylov
solve for the inSilico finite-element hot path.

The compute path is libisl_gpu.so (C-ABI in include/isl_gpu.h, CUDA sources in
insilico_gb300/csrc/); this package only binds it (ctypes) and mirrors the
reference's call sequence (:class:`System`) and benchmark inputs
(:mod:`workloads`).  There is no CPU fallback.
"""
from . import _abi as abi  # noqa: F401
from ._abi import IslError  # noqa: F401
from .system import System  # noqa: F401

__all__ = ["System", "IslError", "abi"]
