"""vvpt_render_noalloc: the render entry point for callers that cannot let a
library allocate device memory (engines with their own fixed memory pool,
processes under a hard memory cap, frame loops that must not hit the
allocator's implicit synchronisation). It takes its scratch from a fixed
array inside the library and writes caller-owned device buffers.

Checked through the C ABI against vvpt_render on the same scene: identical
images (the tracer is deterministic, the tolerance of the other render
checks here is bit equality), on two calls in a row, since every call reuses
the same scratch array; with environment importance sampling too. A fresh
context renders with it before anything else and the device's free memory
does not move. Sizes whose products overflow are refused before any GPU
work. This file is collected last so that a run stopping at its first
failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from vviewer_gb300 import _native as N
from vviewer_gb300 import scenes

pytestmark = pytest.mark.gpu
KEYS = ("radiance", "albedo", "normal", "radiance_m2")


def _render_noalloc(ctx, gpu, sd, info, bufs, flags=0):
    ri = N.RenderInfo(info.samples, info.depth, info.batch_size, info.width, info.height, flags)
    o = N.Outputs(bufs["radiance"].data_ptr(), bufs["albedo"].data_ptr(), bufs["normal"].data_ptr(),
                  bufs["radiance_m2"].data_ptr(), 1)
    return ctx.lib.vvpt_render_noalloc(ctx.handle, gpu.handle, C.byref(sd), C.byref(ri), C.byref(o))


def _nan_buffers(torch, info):
    return {k: torch.full((info.height, info.width, 4), float("nan"), dtype=torch.float32, device="cuda")
            for k in KEYS}


def _check_twice(torch, ctx, engine, info, env_is):
    fs = engine.scene.build()
    sd = engine.scene.scene_data(info.width, info.height)
    gpu = ctx.upload(fs)
    try:
        ref = gpu.render(sd, info, want_m2=True, env_is=env_is)
        for call in range(2):
            bufs = _nan_buffers(torch, info)
            st = _render_noalloc(ctx, gpu, sd, info, bufs, N.RENDER_ENV_IS if env_is else 0)
            assert st == N.VVPT_OK, ctx.lib.vvpt_last_error(ctx.handle)
            torch.cuda.synchronize()
            for k in KEYS:
                got = bufs[k].cpu().numpy()
                want = getattr(ref, k)
                assert np.array_equal(got, want), f"call {call}: {k} differs from vvpt_render"
        assert ctx.stats().paths == info.width * info.height * info.samples
    finally:
        gpu.release()


def test_render_noalloc_matches_render_twice():
    torch = pytest.importorskip("torch")
    from vviewer_gb300 import Context

    ctx = Context(0)
    try:
        e, info = scenes.cornell_box(3, 96, 64, 32, 8, 4)
        _check_twice(torch, ctx, e, info, env_is=False)
    finally:
        ctx.close()


def test_render_noalloc_honours_environment_importance_sampling():
    torch = pytest.importorskip("torch")
    from vviewer_gb300 import Context

    ctx = Context(0)
    try:
        e, info = scenes.sky_scene(2, 64, 48, 16, 6, 4, sky_w=256, sky_h=128)
        _check_twice(torch, ctx, e, info, env_is=True)
    finally:
        ctx.close()


def test_render_noalloc_first_call_of_a_context_allocates_nothing():
    """A fresh context's first render goes through vvpt_render_noalloc: the
    device's free memory is the same before and after the call (the library's
    code and its fixed array are loaded by an earlier call in another context,
    and the scene is uploaded before the measurement)."""
    torch = pytest.importorskip("torch")
    from vviewer_gb300 import Context

    warm = Context(0)
    try:
        e, info = scenes.cornell_box(5, 32, 32, 8, 4, 4)
        g = warm.upload(e.scene.build())
        bufs = _nan_buffers(torch, info)
        assert _render_noalloc(warm, g, e.scene.scene_data(32, 32), info, bufs) == N.VVPT_OK
        torch.cuda.synchronize()
        g.release()
    finally:
        warm.close()

    ctx = Context(0)
    try:
        e, info = scenes.cornell_box(6, 80, 48, 16, 8, 4)
        gpu = ctx.upload(e.scene.build())
        sd = e.scene.scene_data(info.width, info.height)
        bufs = _nan_buffers(torch, info)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        assert _render_noalloc(ctx, gpu, sd, info, bufs) == N.VVPT_OK, ctx.lib.vvpt_last_error(ctx.handle)
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        assert free_after == free_before, f"device free memory moved by {free_before - free_after} bytes"
        assert np.isfinite(bufs["radiance"].cpu().numpy()).all()
        gpu.release()
    finally:
        ctx.close()


def test_render_noalloc_rejects_what_does_not_fit():
    torch = pytest.importorskip("torch")
    from vviewer_gb300 import Context

    ctx = Context(0)
    try:
        e, info = scenes.cornell_box(3, 16, 16, 4, 4, 4)
        gpu = ctx.upload(e.scene.build())
        bufs = {k: torch.zeros((16, 16, 4), dtype=torch.float32, device="cuda") for k in KEYS}
        before = {k: v.clone() for k, v in bufs.items()}
        big = scenes.cornell_box(3, 1920, 1080, 256, 4, 4)[1]
        sd = e.scene.scene_data(1920, 1080)
        assert _render_noalloc(ctx, gpu, sd, big, bufs) == 1  # VVPT_ERR_INVALID_ARG
        assert b"scratch" in ctx.lib.vvpt_last_error(ctx.handle)
        # sizes whose products wrap 32 or 64 bits are refused by the size
        # checks, before any scratch arithmetic or launch
        for w, h, samples, batch, what in ((65536, 65536, 1 << 20, 1, b"resolution"),
                                           (16384, 16384, 64, 2, b"2^32"),
                                           (1 << 31, 4, 1 << 31, 1, b"resolution")):
            huge = scenes.cornell_box(3, 16, 16, 4, 4, 4)[1]
            huge.width, huge.height, huge.samples, huge.batch_size = w, h, samples, batch
            assert _render_noalloc(ctx, gpu, e.scene.scene_data(16, 16), huge, bufs) == 1
            assert what in ctx.lib.vvpt_last_error(ctx.handle), ctx.lib.vvpt_last_error(ctx.handle)
        torch.cuda.synchronize()
        for k in KEYS:
            assert torch.equal(bufs[k], before[k]), f"{k} written by a refused call"
        # host outputs are refused: the call has no staging buffers
        ri = N.RenderInfo(4, 4, 4, 16, 16, 0)
        host = np.zeros((16, 16, 4), dtype=np.float32)
        o = N.Outputs(host.ctypes.data, None, None, None, 0)
        assert ctx.lib.vvpt_render_noalloc(ctx.handle, gpu.handle, C.byref(e.scene.scene_data(16, 16)), C.byref(ri),
                                           C.byref(o)) == 1
        # the PMJ sampler needs tables it would have to allocate: refused
        ri = N.RenderInfo(4, 4, 4, 16, 16, N.RENDER_SAMPLER_PMJ)
        o = N.Outputs(bufs["radiance"].data_ptr(), None, None, None, 1)
        assert ctx.lib.vvpt_render_noalloc(ctx.handle, gpu.handle, C.byref(e.scene.scene_data(16, 16)), C.byref(ri),
                                           C.byref(o)) == 8  # VVPT_ERR_UNSUPPORTED
        gpu.release()
    finally:
        ctx.close()
