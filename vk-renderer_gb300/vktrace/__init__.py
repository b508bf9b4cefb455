"""vktrace: GB300-native (sm_103a) path tracer behind a C ABI.

The drop-in for the compute dispatch of stickyfingies/vk-renderer
(Assets/Tracer.comp); see include/tracer_abi.h for the boundary.
"""
from . import scene
from .abi import (AOV_PRIMARY_HIT, AOV_RGBA8, AOV_RGBA32F, AOV_STATS, KERNEL_AUTO, KERNEL_WAVEFRONT, KERNEL_PLAIN,
                  TIES_REFERENCE, TIES_STRICT, Tracer, TracerError, build_bvh, load_library, validate_bvh)

__all__ = ["scene", "Tracer", "TracerError", "build_bvh", "validate_bvh", "load_library", "AOV_RGBA8", "AOV_RGBA32F",
           "AOV_PRIMARY_HIT", "AOV_STATS", "KERNEL_AUTO", "KERNEL_PLAIN", "KERNEL_WAVEFRONT", "TIES_REFERENCE",
           "TIES_STRICT"]
