"""vira_gb300: a GB300-native (sm_103a) spectral ray-tracing hot path for Vira.

Camera ray generation, BVH build and traversal, watertight ray/triangle intersection, sun
next-event estimation with shadow rays, Lambertian shading and per-band film accumulation run
as hand-written CUDA kernels behind the C ABI of include/vgb.h (libvgb.so).  This package is
the host side: scene, FP64 poses and ephemeris, rebasing, and the reference-shaped API.
"""
from . import capi, spectral, synthetic
from .scene import BatchFrame, Camera, Instance, Mesh, PathTracer, PathTracerOptions, RenderPasses, Scene, SphereLight
from .spectral import EIGHT_BAND, FOUR_BAND, SpectralBands, black_body_radiance

__all__ = [
    "capi", "spectral", "synthetic", "BatchFrame", "Camera", "Instance", "Mesh", "PathTracer", "PathTracerOptions",
    "RenderPasses", "Scene", "SphereLight", "SpectralBands", "black_body_radiance", "FOUR_BAND", "EIGHT_BAND",
]
