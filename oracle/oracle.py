"""ORACLE — test infrastructure only (tests/, the smoke check, and bench.py's
CPU-baseline leg). ctypes wrapper of liboracle.so, the CPU restatement of the
reference's path-tracing shaders in vvpt_oracle.cpp.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"


def build() -> Path:
    src = HERE / "vvpt_oracle.cpp"
    hdr = HERE.parent / "include" / "vvpt.h"
    if not LIB.exists() or LIB.stat().st_mtime < max(src.stat().st_mtime, hdr.stat().st_mtime):
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB))
        lib.oracle_render.restype = C.c_int
        lib.oracle_render.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_int, C.c_int,
                                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.oracle_trace_closest.restype = C.c_int
        lib.oracle_trace_closest.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]
        lib.oracle_set_sampler_tables.restype = None
        lib.oracle_set_sampler_tables.argtypes = [C.c_void_p, C.c_void_p]
        _lib = lib
    return _lib


_tables = None


def _sampler_tables(lib):
    """The PMJ sampler's tables, the same data the library renders with
    (vvpt_sampler_tables), handed to the oracle once and kept alive here."""
    global _tables
    if _tables is None:
        from vviewer_gb300.renderer import sampler_tables
        _tables = sampler_tables()
        lib.oracle_set_sampler_tables(_tables[0].ctypes.data, _tables[1].ctypes.data)
    return _tables


def render(flat_scene, scene_data, info, pixels: np.ndarray | None = None, threads: int = 0, fp64: bool = False,
           env_is: bool = False, sampler: str = "rtgems", alt_order: bool = False):
    """Renders with the oracle. Returns dict of H x W x 4 float32 arrays
    (radiance, albedo, normal, radiance_m2); pixels not in `pixels` stay 0.
    sampler: 'rtgems' or 'pmj' (VVPT_RENDER_SAMPLER_PMJ).
    alt_order: also return 'radiance_alt', the same render with every
    BSDF-direction emitter ray's any-hit candidates taken in
    instance-box-entry order rather than nearest first (the two ends of the
    orders a hardware traversal may report them in; the paths are the same,
    only those rays' contributions differ)."""
    from vviewer_gb300 import _native as N

    lib = load()
    desc = flat_scene.desc()
    flags = N.RENDER_ENV_IS if env_is else 0
    if sampler == "pmj":
        _sampler_tables(lib)
        flags |= N.RENDER_SAMPLER_PMJ
    elif sampler != "rtgems":
        raise ValueError("sampler must be 'rtgems' or 'pmj'")
    ri = N.RenderInfo(info.samples, info.depth, info.batch_size, info.width, info.height, flags)
    H, W = info.height, info.width
    keys = ("radiance", "albedo", "normal", "radiance_m2") + (("radiance_alt",) if alt_order else ())
    out = {k: np.zeros((H, W, 4), dtype=np.float32) for k in keys}
    px = None
    n = 0
    if pixels is not None:
        px = np.ascontiguousarray(pixels, dtype=np.uint32)
        n = px.shape[0]
    threads = threads or (os.cpu_count() or 1)
    st = lib.oracle_render(C.addressof(desc), C.addressof(scene_data), C.addressof(ri),
                           px.ctypes.data if px is not None else None, n, threads,
                           (1 if fp64 else 0) | (2 if alt_order else 0),
                           out["radiance"].ctypes.data, out["albedo"].ctypes.data, out["normal"].ctypes.data,
                           out["radiance_m2"].ctypes.data, out["radiance_alt"].ctypes.data if alt_order else None)
    if st != 0:
        raise RuntimeError(f"oracle_render failed with {st}")
    return out


def trace_closest(flat_scene, rays: np.ndarray) -> np.ndarray:
    from vviewer_gb300.renderer import HIT_DTYPE

    lib = load()
    desc = flat_scene.desc()
    rays = np.ascontiguousarray(rays, dtype=np.float32)
    hits = np.zeros(rays.shape[0], dtype=HIT_DTYPE)
    st = lib.oracle_trace_closest(C.addressof(desc), rays.ctypes.data, rays.shape[0], hits.ctypes.data)
    if st != 0:
        raise RuntimeError(f"oracle_trace_closest failed with {st}")
    return hits
