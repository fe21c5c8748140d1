"""vvpt_render_noalloc: the render entry point for callers that cannot let a
library allocate device memory (engines with their own fixed memory pool,
processes under a hard memory cap, frame loops that must not hit the
allocator's implicit synchronisation). It takes its scratch from a fixed
array inside the library and writes caller-owned device buffers.

Checked through the C ABI against vvpt_render on the same scene: identical
images (the tracer is deterministic, the tolerance of the other render
checks here is bit equality), on two calls in a row, since every call reuses
the same scratch array. This file is collected last so that a run stopping
at its first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from vviewer_gb300 import _native as N
from vviewer_gb300 import scenes

pytestmark = pytest.mark.gpu


def _render_noalloc(ctx, gpu, sd, info, bufs):
    ri = N.RenderInfo(info.samples, info.depth, info.batch_size, info.width, info.height, 0)
    o = N.Outputs(bufs["radiance"].data_ptr(), bufs["albedo"].data_ptr(), bufs["normal"].data_ptr(),
                  bufs["radiance_m2"].data_ptr(), 1)
    return ctx.lib.vvpt_render_noalloc(ctx.handle, gpu.handle, C.byref(sd), C.byref(ri), C.byref(o))


def test_render_noalloc_matches_render_twice():
    torch = pytest.importorskip("torch")
    from vviewer_gb300 import Context

    ctx = Context(0)
    try:
        e, info = scenes.cornell_box(3, 96, 64, 32, 8, 4)
        fs = e.scene.build()
        sd = e.scene.scene_data(info.width, info.height)
        gpu = ctx.upload(fs)
        ref = gpu.render(sd, info, want_m2=True)
        keys = ("radiance", "albedo", "normal", "radiance_m2")
        for call in range(2):
            bufs = {k: torch.full((info.height, info.width, 4), float("nan"), dtype=torch.float32, device="cuda")
                    for k in keys}
            st = _render_noalloc(ctx, gpu, sd, info, bufs)
            assert st == N.VVPT_OK, ctx.lib.vvpt_last_error(ctx.handle)
            torch.cuda.synchronize()
            for k in keys:
                got = bufs[k].cpu().numpy()
                want = getattr(ref, k)
                assert np.array_equal(got, want), f"call {call}: {k} differs from vvpt_render"
        assert ctx.stats().paths == info.width * info.height * info.samples
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
        bufs = {k: torch.zeros((16, 16, 4), dtype=torch.float32, device="cuda")
                for k in ("radiance", "albedo", "normal", "radiance_m2")}
        big = scenes.cornell_box(3, 1920, 1080, 256, 4, 4)[1]
        sd = e.scene.scene_data(1920, 1080)
        assert _render_noalloc(ctx, gpu, sd, big, bufs) == 1  # VVPT_ERR_INVALID_ARG
        assert b"scratch" in ctx.lib.vvpt_last_error(ctx.handle)
        # host outputs are refused: the call has no staging buffers
        ri = N.RenderInfo(4, 4, 4, 16, 16, 0)
        host = np.zeros((16, 16, 4), dtype=np.float32)
        o = N.Outputs(host.ctypes.data, None, None, None, 0)
        assert ctx.lib.vvpt_render_noalloc(ctx.handle, gpu.handle, C.byref(e.scene.scene_data(16, 16)), C.byref(ri),
                                           C.byref(o)) == 1
        gpu.release()
    finally:
        ctx.close()
