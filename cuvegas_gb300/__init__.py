"""cuvegas_gb300 -- GB300-native VEGAS+ adaptive Monte Carlo integration.

The hot path (sampling, grid map, integrand, accumulation, reallocation and
grid refinement) runs in libcuvegas.so, hand-written CUDA for sm_103a behind a
C ABI (include/cuvegas.h).  This package is the Python side of that boundary:
``integrate`` mirrors the reference's ``vegas_cuda_extension.python_wrapper
.integrate``; ``runtime`` exposes contexts, integrands and step-level runs.
"""
from . import _lib
from ._lib import CuvegasError
from .python_wrapper import integrate

__all__ = ["integrate", "CuvegasError", "build"]


def build(force=False):
    """Compile libcuvegas.so in-tree for sm_103a."""
    from . import _build
    return _build.build(force=force)
