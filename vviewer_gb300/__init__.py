"""GB300-native drop-in for vengine's offline path-traced renderer.

The compute path is libvvpt.so (hand-written sm_103a CUDA kernels behind the C
ABI of include/vvpt.h); this package is the host-side mirror of the reference's
scene and renderer API plus scene generators and I/O.
"""
from .renderer import Context, GpuScene, RenderInfo, RendererPathTracing, RenderResult  # noqa: F401
from .scene import (DirectionalLight, Engine, EnvironmentType, LightType, MaterialLambert,  # noqa: F401
                    MaterialPBRStandard, MaterialVolume, PerspectiveCamera, PointLight, Scene, SceneObject,
                    Transform, radians)

__all__ = [
    "Context", "GpuScene", "RenderInfo", "RendererPathTracing", "RenderResult", "DirectionalLight", "Engine",
    "EnvironmentType", "LightType", "MaterialLambert", "MaterialPBRStandard", "MaterialVolume",
    "PerspectiveCamera", "PointLight", "Scene", "SceneObject", "Transform", "radians",
]
