"""GB300-native RSF (region-scalable fitting) level-set evolution.

The evolution runs in librsf_gb300.so (hand-written sm_103a CUDA behind the C
ABI of include/rsf.h); this package is its Python face.
"""
from ._lib import RsfError  # noqa: F401
from .api import Params, Workspace, copy_async, gaussian_taps  # noqa: F401

__all__ = ["Params", "RsfError", "Workspace", "copy_async", "gaussian_taps"]
