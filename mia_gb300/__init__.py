"""mia_gb300 — GB300 (sm_103a) implementation of MIA's B-spline
nonrigid-registration cost+gradient path (spline transformation, image full
cost with ssd/ncc, divcurl penalty, bspline:d=3 interpolation).

The compute runs in libmgr.so (hand-written CUDA behind the C ABI of
include/mgr.h).  Importing this package does not touch the GPU; creating a
``Level`` does, and fails loudly when libmgr.so or the GPU is missing.
"""
from ._lib import MgrError, lib  # noqa: F401
from .level import Level  # noqa: F401

__all__ = ["Level", "MgrError", "lib"]
