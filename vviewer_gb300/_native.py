"""ctypes binding of include/vvpt.h (libvvpt.so).

The structures below mirror the C declarations field for field. Loading fails
loudly when the library is missing; there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libvvpt.so"

VVPT_OK = 0
TIMEOUT = 4
BUDGET_EXCEEDED = 3
NOT_READY = 6
STATUS_NAMES = {
    0: "VVPT_OK", 1: "VVPT_ERR_INVALID_ARG", 2: "VVPT_ERR_OOM", 3: "VVPT_ERR_BUDGET_EXCEEDED",
    4: "VVPT_ERR_TIMEOUT", 5: "VVPT_ERR_DEVICE", 6: "VVPT_ERR_NOT_READY", 7: "VVPT_ERR_EMPTY_SCENE",
    8: "VVPT_ERR_UNSUPPORTED",
}

BVH_BUILDER_AUTO, BVH_BUILDER_HOST, BVH_BUILDER_GPU = 0, 1, 2

MATERIAL_PBR_STANDARD = 0
MATERIAL_LAMBERT = 2
MATERIAL_VOLUME = 3
INSTANCE_IN_TLAS = 1
TEXTURE_RGBA8_LINEAR = 0
TEXTURE_RGBA8_SRGB = 1
TEXTURE_RGBA32F = 2
RENDER_WANT_BATCH_M2 = 1
RENDER_ENV_IS = 4
RENDER_SAMPLER_PMJ = 8
RENDER_REDUCE_FP64 = 16
PMJ_SEQUENCES = 16
PMJ_SAMPLES = 16384
BLUE_NOISE_TEXTURES = 48
BLUE_NOISE_RES = 128


class VvptError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class Vertex(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("uv", C.c_float * 2), ("normal", C.c_float * 3),
                ("color", C.c_float * 3), ("tangent", C.c_float * 3), ("bitangent", C.c_float * 3)]


class MeshDesc(C.Structure):
    _fields_ = [("vertices", C.c_void_p), ("num_vertices", C.c_uint32), ("indices", C.c_void_p),
                ("num_triangles", C.c_uint32)]


class Material(C.Structure):
    _fields_ = [("albedo", C.c_float * 4), ("metallic_roughness_ao", C.c_float * 4), ("emissive", C.c_float * 4),
                ("textures1", C.c_uint32 * 4), ("textures2", C.c_uint32 * 4), ("uv_tiling", C.c_float * 4),
                ("padding", C.c_uint32 * 8)]


class Instance(C.Structure):
    _fields_ = [("model", C.c_float * 16), ("id", C.c_float * 4), ("material_index", C.c_uint32),
                ("mesh_index", C.c_uint32), ("num_triangles", C.c_uint32), ("flags", C.c_uint32)]


class LightData(C.Structure):
    _fields_ = [("color", C.c_float * 4), ("type", C.c_uint32 * 4), ("padding", C.c_uint32 * 8)]


class LightInstance(C.Structure):
    _fields_ = [("info", C.c_uint32 * 4), ("position", C.c_float * 4), ("position1", C.c_float * 4),
                ("position2", C.c_float * 4)]


class TextureDesc(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("format", C.c_uint32), ("reserved", C.c_uint32),
                ("data", C.c_void_p)]


class SceneDesc(C.Structure):
    _fields_ = [("meshes", C.POINTER(MeshDesc)), ("num_meshes", C.c_uint32),
                ("instances", C.POINTER(Instance)), ("num_instances", C.c_uint32),
                ("materials", C.POINTER(Material)), ("num_materials", C.c_uint32),
                ("light_data", C.POINTER(LightData)), ("num_light_data", C.c_uint32),
                ("lights", C.POINTER(LightInstance)), ("num_lights", C.c_uint32),
                ("textures", C.POINTER(TextureDesc)), ("num_textures", C.c_uint32),
                ("environment", C.POINTER(TextureDesc))]


class SceneData(C.Structure):
    _fields_ = [("view", C.c_float * 16), ("view_inverse", C.c_float * 16), ("projection", C.c_float * 16),
                ("projection_inverse", C.c_float * 16), ("exposure", C.c_float * 4), ("background", C.c_float * 4),
                ("volumes", C.c_float * 4)]


class RenderInfo(C.Structure):
    _fields_ = [("samples", C.c_uint32), ("depth", C.c_uint32), ("batch_size", C.c_uint32), ("width", C.c_uint32),
                ("height", C.c_uint32), ("flags", C.c_uint32)]


class Outputs(C.Structure):
    _fields_ = [("radiance", C.c_void_p), ("albedo", C.c_void_p), ("normal", C.c_void_p),
                ("radiance_m2", C.c_void_p), ("on_device", C.c_int32)]


class Ray(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("tmin", C.c_float), ("direction", C.c_float * 3), ("tmax", C.c_float)]


class Hit(C.Structure):
    _fields_ = [("t", C.c_float), ("u", C.c_float), ("v", C.c_float), ("instance", C.c_uint32),
                ("primitive", C.c_uint32)]


class RenderStats(C.Structure):
    _fields_ = [("kernel_launches", C.c_uint64), ("iterations", C.c_uint64), ("segments", C.c_uint64),
                ("shadow_rays", C.c_uint64), ("emitter_rays", C.c_uint64), ("paths", C.c_uint64),
                ("device_ms", C.c_double)]


class Tuning(C.Structure):
    _fields_ = [("slots", C.c_uint32), ("blocks_per_sm", C.c_uint32), ("threads_per_block", C.c_uint32),
                ("iterations_per_graph", C.c_uint32)]


class KernelProfileEntry(C.Structure):
    _fields_ = [("name", C.c_char * 24), ("launches", C.c_uint64), ("units", C.c_uint64), ("total_ms", C.c_double),
                ("bytes_per_unit", C.c_double)]


class KernelProfile(C.Structure):
    _fields_ = [("count", C.c_uint32), ("kernels", KernelProfileEntry * 8)]


RENDER_PROFILE_KERNELS = 2


# every symbol include/vvpt.h declares, with its ctypes signature
class JobInfo(C.Structure):
    _fields_ = [("state", C.c_uint32), ("status", C.c_int32), ("submit_ms", C.c_double), ("start_ms", C.c_double),
                ("end_ms", C.c_double), ("paths", C.c_uint64), ("device_bytes", C.c_uint64)]


class EngineStats(C.Structure):
    _fields_ = [("fixed_bytes", C.c_uint64), ("job_bytes", C.c_uint64), ("queued", C.c_uint32),
                ("running", C.c_uint32), ("finished", C.c_uint32), ("slots", C.c_uint32)]


class DenoiseBatch(C.Structure):
    _fields_ = [("radiance", C.c_void_p), ("albedo", C.c_void_p), ("normal", C.c_void_p), ("target", C.c_void_p),
                ("count", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32)]


JOB_QUEUED, JOB_RUNNING, JOB_DONE, JOB_FAILED = 0, 1, 2, 3

_SIGNATURES = {
    "vvpt_version": (C.c_char_p, []),
    "vvpt_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "vvpt_destroy": (C.c_int, [C.c_void_p]),
    "vvpt_last_error": (C.c_char_p, [C.c_void_p]),
    "vvpt_scene_upload": (C.c_int, [C.c_void_p, C.POINTER(SceneDesc), C.POINTER(C.c_void_p)]),
    "vvpt_scene_release": (C.c_int, [C.c_void_p, C.c_void_p]),
    "vvpt_scene_device_bytes": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_uint64)]),
    "vvpt_render": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(SceneData), C.POINTER(RenderInfo),
                              C.POINTER(Outputs)]),
    "vvpt_progress": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "vvpt_trace_closest": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_int32]),
    "vvpt_last_render_stats": (C.c_int, [C.c_void_p, C.POINTER(RenderStats)]),
    "vvpt_set_tuning": (C.c_int, [C.c_void_p, C.POINTER(Tuning)]),
    "vvpt_get_tuning": (C.c_int, [C.c_void_p, C.POINTER(Tuning)]),
    "vvpt_last_kernel_profile": (C.c_int, [C.c_void_p, C.POINTER(KernelProfile)]),
    "vvpt_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "vvpt_render_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(SceneData), C.POINTER(RenderInfo),
                                      C.POINTER(Outputs)]),
    "vvpt_submit": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(SceneData), C.POINTER(RenderInfo),
                              C.POINTER(Outputs), C.POINTER(C.c_uint64)]),
    "vvpt_poll": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(JobInfo)]),
    "vvpt_wait": (C.c_int, [C.c_void_p, C.c_uint64, C.c_double]),
    "vvpt_job_release": (C.c_int, [C.c_void_p, C.c_uint64]),
    "vvpt_set_budget": (C.c_int, [C.c_void_p, C.c_uint64]),
    "vvpt_set_bvh_builder": (C.c_int, [C.c_void_p, C.c_int]),
    "vvpt_autotune": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(SceneData), C.POINTER(RenderInfo), C.c_double,
                                C.POINTER(Tuning)]),
    "vvpt_engine_stats_get": (C.c_int, [C.c_void_p, C.POINTER(EngineStats)]),
    "vvpt_denoiser_create": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(C.c_void_p)]),
    "vvpt_denoiser_destroy": (C.c_int, [C.c_void_p]),
    "vvpt_denoiser_num_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64)]),
    "vvpt_denoiser_get_params": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64]),
    "vvpt_denoiser_set_params": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64]),
    "vvpt_denoiser_gradients": (C.c_int, [C.c_void_p, C.POINTER(DenoiseBatch), C.c_void_p, C.c_uint64,
                                          C.POINTER(C.c_float)]),
    "vvpt_denoiser_train_step": (C.c_int, [C.c_void_p, C.POINTER(DenoiseBatch), C.c_float, C.POINTER(C.c_float)]),
    "vvpt_denoiser_set_kernels": (C.c_int, [C.c_void_p, C.c_int]),
    "vvpt_denoiser_inject_wait_timeout": (C.c_int, [C.c_void_p]),
    "vvpt_denoiser_apply": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32,
                                      C.c_uint32]),
    "vvpt_render_batch": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(C.c_void_p), C.POINTER(SceneData),
                                    C.POINTER(RenderInfo), C.POINTER(Outputs)]),
    "vvpt_sampler_tables": (C.c_int, [C.c_void_p, C.c_void_p]),
    "vvpt_jpeg_decode": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                   C.POINTER(C.c_uint32), C.c_void_p, C.c_uint64]),
}

_lib = None


def load(path: Path | None = None):
    """Loads libvvpt.so (building it first if it is missing) and binds every entry point."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        from . import build as _build
        _build.build()
    if not p.exists():
        raise RuntimeError(f"libvvpt.so not found at {p}; run vviewer_gb300/build.py")
    lib = C.CDLL(str(p))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def declared_symbols() -> list[str]:
    return list(_SIGNATURES)


def check(status: int, ctx=None) -> None:
    if status != VVPT_OK:
        msg = ""
        if ctx is not None and _lib is not None:
            raw = _lib.vvpt_last_error(ctx)
            msg = raw.decode() if raw else ""
        raise VvptError(status, msg)


def as_ptr(a: np.ndarray) -> int:
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data
