"""RendererPathTracing adapter over the C ABI.

Mirrors src/lib/vengine/core/Renderer.hpp:11-39 (RenderInfo, render,
renderProgress, isRayTracingEnabled) and the output step of
src/lib/vengine/vulkan/renderers/VulkanRendererPathTracing.cpp:958-1027 and
src/lib/vengine/core/ImageUtils.cpp:39-76 (exposure for PNG, RGBE or sRGB PNG).
"""
from __future__ import annotations

import ctypes as C
import struct
import warnings
import zlib
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import _native as N
from .assets import srgb_encode, write_hdr
from .scene import Engine, FlatScene


def _sampler_flag(sampler: str) -> int:
    if sampler not in ("rtgems", "pmj"):
        raise ValueError("sampler must be 'rtgems' or 'pmj'")
    return N.RENDER_SAMPLER_PMJ if sampler == "pmj" else 0


def sampler_tables() -> tuple[np.ndarray, np.ndarray]:
    """The PMJ sampler's tables (vvpt_sampler_tables): (16, 16384, 2) (0,2)
    sequence points and (48, 128, 128) blue-noise values, float32."""
    lib = N.load()
    pmj = np.zeros((N.PMJ_SEQUENCES, N.PMJ_SAMPLES, 2), dtype=np.float32)
    bn = np.zeros((N.BLUE_NOISE_TEXTURES, N.BLUE_NOISE_RES, N.BLUE_NOISE_RES), dtype=np.float32)
    st = lib.vvpt_sampler_tables(pmj.ctypes.data, bn.ctypes.data)
    if st != 0:
        raise N.VvptError(st, "vvpt_sampler_tables failed")
    return pmj, bn


@dataclass
class RenderInfo:
    samples: int = 256
    depth: int = 9
    batch_size: int = 4
    filename: str = "test"
    file_type: str = "hdr"  # "hdr" or "png"
    exposure: float = 0.0
    width: int = 1080
    height: int = 1080
    denoise: bool = False
    write_all_files: bool = False
    write_files: bool = True


@dataclass
class RenderResult:
    radiance: np.ndarray  # H x W x 4 float32
    albedo: np.ndarray
    normal: np.ndarray
    radiance_m2: np.ndarray | None
    stats: N.RenderStats
    batches: int


class Context:
    """One CUDA device context of the library (vvpt_create / vvpt_destroy)."""

    def __init__(self, device: int = 0):
        self.lib = N.load()
        h = C.c_void_p()
        st = self.lib.vvpt_create(device, C.byref(h))
        if st != N.VVPT_OK:
            raise N.VvptError(st, "vvpt_create failed (no usable CUDA device)")
        self.handle = h

    def close(self) -> None:
        if self.handle:
            self.lib.vvpt_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, st: int) -> None:
        N.check(st, self.handle)

    def upload(self, flat: FlatScene) -> "GpuScene":
        d = flat.desc()
        h = C.c_void_p()
        self.check(self.lib.vvpt_scene_upload(self.handle, C.byref(d), C.byref(h)))
        return GpuScene(self, h, flat)

    def set_tuning(self, slots=0, blocks_per_sm=0, threads_per_block=0, iterations_per_graph=0) -> None:
        t = N.Tuning(slots, blocks_per_sm, threads_per_block, iterations_per_graph)
        self.check(self.lib.vvpt_set_tuning(self.handle, C.byref(t)))

    def stats(self) -> N.RenderStats:
        s = N.RenderStats()
        self.check(self.lib.vvpt_last_render_stats(self.handle, C.byref(s)))
        return s

    def kernel_profile(self) -> list[dict]:
        """Per-kernel profile of the last render made with profile=True."""
        p = N.KernelProfile()
        self.check(self.lib.vvpt_last_kernel_profile(self.handle, C.byref(p)))
        return [{"name": k.name.decode(), "launches": int(k.launches), "units": int(k.units),
                 "total_ms": float(k.total_ms), "bytes_per_unit": float(k.bytes_per_unit)}
                for k in p.kernels[:p.count]]

    def set_budget(self, nbytes: int) -> None:
        """Device-memory budget of the job engine (0: no limit)."""
        self.check(self.lib.vvpt_set_budget(self.handle, int(nbytes)))

    def engine_stats(self) -> N.EngineStats:
        es = N.EngineStats()
        self.check(self.lib.vvpt_engine_stats_get(self.handle, C.byref(es)))
        return es

    def set_stream(self, cuda_stream: int | None) -> None:
        """Runs the context's work on a caller-owned CUDA stream (None: its own)."""
        self.check(self.lib.vvpt_set_stream(self.handle, cuda_stream or None))


class GpuScene:
    """A scene resident on the device (vvpt_scene_upload)."""

    def __init__(self, ctx: Context, handle, flat: FlatScene):
        self.ctx = ctx
        self.handle = handle
        self.flat = flat

    def release(self) -> None:
        """Frees the device copy; raises (VVPT_ERR_NOT_READY) while
        submitted jobs still use the scene."""
        if self.handle:
            self.ctx.check(self.ctx.lib.vvpt_scene_release(self.ctx.handle, self.handle))
            self.handle = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass

    def device_bytes(self) -> int:
        b = C.c_uint64()
        self.ctx.check(self.ctx.lib.vvpt_scene_device_bytes(self.ctx.handle, self.handle, C.byref(b)))
        return int(b.value)

    def render(self, scene_data: N.SceneData, info: RenderInfo, want_m2: bool = False,
               outputs: dict | None = None, profile: bool = False,
               host_outputs: dict | None = None, env_is: bool = False,
               sampler: str = "rtgems", reduce_fp64: bool = False) -> RenderResult | None:
        """Renders into new host arrays, into caller-provided host arrays
        (`host_outputs`), or into device pointers when `outputs` maps
        radiance/albedo/normal/radiance_m2 to device addresses. env_is: the
        environment is importance sampled as a light (VVPT_RENDER_ENV_IS).
        sampler: 'rtgems' (the reference's default xorshift stream) or 'pmj'
        (its low-discrepancy sampler, VVPT_RENDER_SAMPLER_PMJ). reduce_fp64:
        the batch sums are added in double precision (VVPT_RENDER_REDUCE_FP64)."""
        flags = ((N.RENDER_WANT_BATCH_M2 if want_m2 else 0) | (N.RENDER_PROFILE_KERNELS if profile else 0) |
                 (N.RENDER_ENV_IS if env_is else 0) | _sampler_flag(sampler) |
                 (N.RENDER_REDUCE_FP64 if reduce_fp64 else 0))
        ri = N.RenderInfo(info.samples, info.depth, info.batch_size, info.width, info.height, flags)
        if host_outputs is not None:
            o = N.Outputs(host_outputs.get("radiance"), host_outputs.get("albedo"), host_outputs.get("normal"),
                          host_outputs.get("radiance_m2"), 0)
            self.ctx.check(self.ctx.lib.vvpt_render(self.ctx.handle, self.handle, C.byref(scene_data), C.byref(ri),
                                                    C.byref(o)))
            return None
        if outputs is not None:
            o = N.Outputs(outputs.get("radiance"), outputs.get("albedo"), outputs.get("normal"),
                          outputs.get("radiance_m2"), 1)
            self.ctx.check(self.ctx.lib.vvpt_render(self.ctx.handle, self.handle, C.byref(scene_data), C.byref(ri),
                                                    C.byref(o)))
            return None
        H, W = info.height, info.width
        rad = np.zeros((H, W, 4), dtype=np.float32)
        alb = np.zeros((H, W, 4), dtype=np.float32)
        nrm = np.zeros((H, W, 4), dtype=np.float32)
        m2 = np.zeros((H, W, 4), dtype=np.float32) if want_m2 else None
        o = N.Outputs(rad.ctypes.data, alb.ctypes.data, nrm.ctypes.data, m2.ctypes.data if want_m2 else None, 0)
        self.ctx.check(self.ctx.lib.vvpt_render(self.ctx.handle, self.handle, C.byref(scene_data), C.byref(ri),
                                                C.byref(o)))
        return RenderResult(rad, alb, nrm, m2, self.ctx.stats(), info.samples // info.batch_size)

    def submit(self, scene_data: N.SceneData, info: RenderInfo, want_m2: bool = False,
               outputs: dict | None = None, env_is: bool = False, sampler: str = "rtgems") -> "Job":
        """Queues a render on the context's job engine (vvpt_submit). Outputs go
        to new host arrays, or to device pointers when `outputs` maps
        radiance/albedo/normal/radiance_m2 to device addresses."""
        flags = ((N.RENDER_WANT_BATCH_M2 if want_m2 else 0) | (N.RENDER_ENV_IS if env_is else 0) |
                 _sampler_flag(sampler))
        ri = N.RenderInfo(info.samples, info.depth, info.batch_size, info.width, info.height, flags)
        job = Job(self, info, want_m2)
        if outputs is not None:
            o = N.Outputs(outputs.get("radiance"), outputs.get("albedo"), outputs.get("normal"),
                          outputs.get("radiance_m2"), 1)
        else:
            H, W = info.height, info.width
            job.radiance = np.zeros((H, W, 4), dtype=np.float32)
            job.albedo = np.zeros((H, W, 4), dtype=np.float32)
            job.normal = np.zeros((H, W, 4), dtype=np.float32)
            job.radiance_m2 = np.zeros((H, W, 4), dtype=np.float32) if want_m2 else None
            o = N.Outputs(job.radiance.ctypes.data, job.albedo.ctypes.data, job.normal.ctypes.data,
                          job.radiance_m2.ctypes.data if want_m2 else None, 0)
        jid = C.c_uint64()
        self.ctx.check(self.ctx.lib.vvpt_submit(self.ctx.handle, self.handle, C.byref(scene_data), C.byref(ri),
                                                C.byref(o), C.byref(jid)))
        job.id = int(jid.value)
        return job

    def autotune(self, scene_data: N.SceneData, info: RenderInfo, budget_ms: float = 3000.0,
                 env_is: bool = False) -> dict:
        """Picks the context's tuning for requests like `info` (vvpt_autotune)."""
        flags = N.RENDER_ENV_IS if env_is else 0
        ri = N.RenderInfo(info.samples, info.depth, info.batch_size, info.width, info.height, flags)
        t = N.Tuning()
        self.ctx.check(self.ctx.lib.vvpt_autotune(self.ctx.handle, self.handle, C.byref(scene_data), C.byref(ri),
                                                  float(budget_ms), C.byref(t)))
        return {"slots": t.slots, "blocks_per_sm": t.blocks_per_sm, "threads_per_block": t.threads_per_block,
                "iterations_per_graph": t.iterations_per_graph}

    def trace_closest(self, rays: np.ndarray) -> np.ndarray:
        """rays: N x 8 float32 (origin, tmin, direction, tmax) -> structured hits."""
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        n = rays.shape[0]
        hits = np.zeros(n, dtype=HIT_DTYPE)
        self.ctx.check(self.ctx.lib.vvpt_trace_closest(self.ctx.handle, self.handle, rays.ctypes.data, n,
                                                       hits.ctypes.data, 0))
        return hits


class Job:
    """A render submitted to the job engine; its host outputs (if any) are
    filled when the job is done."""

    def __init__(self, scene: GpuScene, info: RenderInfo, want_m2: bool):
        self.scene = scene
        self.ctx = scene.ctx
        self.info = info
        self.want_m2 = want_m2
        self.id = 0
        self.radiance = self.albedo = self.normal = self.radiance_m2 = None

    def poll(self) -> N.JobInfo:
        ji = N.JobInfo()
        self.ctx.check(self.ctx.lib.vvpt_poll(self.ctx.handle, self.id, C.byref(ji)))
        return ji

    def done(self) -> bool:
        return self.poll().state in (N.JOB_DONE, N.JOB_FAILED)

    def wait(self, timeout_ms: float = -1.0) -> bool:
        """True when done; False on timeout; raises if the job failed."""
        st = self.ctx.lib.vvpt_wait(self.ctx.handle, self.id, float(timeout_ms))
        if st == N.TIMEOUT:
            return False
        self.ctx.check(st)
        return True

    def result(self) -> RenderResult:
        self.wait()
        return RenderResult(self.radiance, self.albedo, self.normal, self.radiance_m2, None,
                            self.info.samples // self.info.batch_size)

    def release(self) -> None:
        if self.id:
            self.ctx.check(self.ctx.lib.vvpt_job_release(self.ctx.handle, self.id))
            self.id = 0


HIT_DTYPE = np.dtype([("t", np.float32), ("u", np.float32), ("v", np.float32), ("instance", np.uint32),
                      ("primitive", np.uint32)])


def write_png(path: str | Path, rgba8: np.ndarray) -> None:
    """Minimal PNG writer (8-bit RGBA, no filtering)."""
    h, w, c = rgba8.shape
    raw = b"".join(b"\x00" + rgba8[y].tobytes() for y in range(h))

    def chunk(tag: bytes, data: bytes) -> bytes:
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    color_type = 6 if c == 4 else 2
    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, color_type, 0, 0, 0))
    png += chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b"")
    Path(path).write_bytes(png)


def write_to_disk(data: np.ndarray, filename: str, file_type: str) -> None:
    """ImageUtils.cpp:51-76. "png": every channel, alpha included, becomes
    uint8(255 * linearToSRGB(clamp(v, 0, 1))) (truncation, float32), written
    as an 8-bit RGBA PNG; "hdr": RGBE of the first three channels (the
    Radiance format has no alpha)."""
    if file_type == "png":
        rgba = np.asarray(data, dtype=np.float32)
        write_png(filename + ".png", (np.float32(255.0) * srgb_encode(rgba)).astype(np.uint8))
    elif file_type == "hdr":
        write_hdr(filename + ".hdr", data)
    else:
        raise ValueError("writeToDisk(): Unsupported file type")


def apply_exposure(data: np.ndarray, exposure: float) -> np.ndarray:
    """ImageUtils.cpp:34-49: v * 2^exposure on the first three channels."""
    out = np.array(data, dtype=np.float32, copy=True)
    out[..., :3] = out[..., :3] * np.float32(np.power(np.float32(2.0), np.float32(exposure)))
    return out


class RendererPathTracing:
    """engine.renderer().rendererPathTracing() of the reference."""

    def __init__(self, engine: Engine, device: int = 0, context: Context | None = None, denoiser=None):
        self.engine = engine
        # denoise=True runs this (the OIDN step of storeToDisk): any object
        # with denoise(radiance, albedo, normal) -> radiance over H x W x 4
        # float32 arrays, e.g. DenoiserStep over a trained Denoiser
        self.denoiser = denoiser
        self._ctx = context
        self._device = device
        self._info = RenderInfo()
        self._progress = 0.0
        self._in_progress = False
        self.last_result: RenderResult | None = None

    def render_info(self) -> RenderInfo:
        return self._info

    @property
    def context(self) -> Context:
        if self._ctx is None:
            self._ctx = Context(self._device)
        return self._ctx

    def is_ray_tracing_enabled(self) -> bool:
        try:
            return self.context.handle is not None
        except N.VvptError:
            return False

    def render_progress(self) -> float:
        if self._ctx is None:
            return self._progress
        p = C.c_float()
        self._ctx.lib.vvpt_progress(self._ctx.handle, C.byref(p))
        return float(p.value)

    def render(self) -> RenderResult | None:
        if self._in_progress:
            return None
        scene = self.engine.scene
        if not scene.objects_flat():
            warnings.warn("Trying to render an empty scene")
            return None
        self._in_progress = True
        try:
            info = self._info
            flat = scene.build()
            gpu = self.context.upload(flat)
            try:
                res = gpu.render(scene.scene_data(info.width, info.height), info)
            finally:
                gpu.release()
            self.last_result = res
            if info.write_files:
                self.store_to_disk(res)
            return res
        finally:
            self._in_progress = False

    def store_to_disk(self, res: RenderResult) -> None:
        """VulkanRendererPathTracing.cpp:958-1027: with writeAllFiles the
        albedo and normal AOVs as HDR; without denoising the radiance, exposed
        for PNG only; with denoising also the noisy radiance as
        `<name>_radiance.hdr`, then the denoised image, exposed for PNG."""
        info = self._info
        if info.write_all_files:
            write_to_disk(res.albedo, info.filename + "_albedo", "hdr")
            write_to_disk(res.normal, info.filename + "_normal", "hdr")
        radiance = res.radiance
        if info.denoise:
            if self.denoiser is None:
                raise ValueError("denoise=True needs a denoiser: set RendererPathTracing.denoiser "
                                 "(e.g. DenoiserStep over a trained Denoiser)")
            if info.write_all_files:
                write_to_disk(radiance, info.filename + "_radiance", "hdr")
            radiance = np.asarray(self.denoiser.denoise(res.radiance, res.albedo, res.normal), dtype=np.float32)
        if info.file_type == "png" and info.exposure != 0.0:
            radiance = apply_exposure(radiance, info.exposure)
        write_to_disk(radiance, info.filename, info.file_type)
