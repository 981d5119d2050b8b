"""blitzen_gb300 — GB300-native (sm_103a) GPU-driven culling for the Blitzen renderer's cull path.

The product is libblz_cull.so (C ABI in include/blz_cull.h, CUDA kernels in csrc/). This package
holds its build script, ctypes bindings (abi), the host-side mirror of the reference's cull
interface (culler.Culler) and seeded synthetic scenes (scenes).
"""
from . import abi  # noqa: F401
from .abi import BlzError, CameraViewData, load, pyramid_layout, view_setup  # noqa: F401

__all__ = ["abi", "BlzError", "CameraViewData", "load", "pyramid_layout", "view_setup"]
