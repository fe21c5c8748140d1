"""Job engine (vvpt_submit / vvpt_poll / vvpt_wait / vvpt_render_batch): jobs
rendered together, with the work items of all jobs in one hand-out sequence
and fused per-stage queues, give images bit-identical to rendering each job
alone; admission respects the device budget; waits time out; scenes in use
cannot be released."""
import ctypes as C

import numpy as np
import pytest

from vviewer_gb300 import _native as N
from vviewer_gb300 import scenes
from vviewer_gb300.renderer import RenderInfo

pytestmark = pytest.mark.gpu


def _same(a, b):
    for k in ("radiance", "albedo", "normal"):
        x, y = getattr(a, k), getattr(b, k)
        assert np.array_equal(x, y), f"{k}: {np.count_nonzero(x != y)} values differ"


@pytest.fixture(scope="module")
def mixed_jobs(ctx):
    """Three scenes (the Cornell room, a room with a medium and displaced
    spheres, a seeded random scene) at different resolutions and sample
    counts."""
    e1, i1 = scenes.cornell_box(3, 64, 48, 16, 6, 4)
    e2, i2 = scenes.cornell_medium(2, 80, 40, 8, 8, 2, freq=6, spheres=3)
    e3 = scenes.random_scene(5, min_tris=2_000, max_tris=20_000)
    i3 = RenderInfo(samples=12, depth=7, batch_size=3, width=40, height=72, write_files=False)
    out = []
    for e, info in ((e1, i1), (e2, i2), (e3, i3)):
        g = ctx.upload(e.scene.build())
        out.append((g, e.scene.scene_data(info.width, info.height), info))
    yield out
    for g, _, _ in out:
        g.release()


def test_jobs_in_a_mix_equal_single_renders(ctx, mixed_jobs):
    alone = [g.render(sd, info) for g, sd, info in mixed_jobs]
    jobs = []
    for rep in range(3):
        for g, sd, info in mixed_jobs:
            jobs.append(g.submit(sd, info))
    for k, j in enumerate(jobs):
        r = j.result()
        _same(r, alone[k % len(mixed_jobs)])
        ji = j.poll()
        assert ji.state == N.JOB_DONE and ji.status == 0
        assert ji.submit_ms <= ji.start_ms <= ji.end_ms
        info = j.info
        assert ji.paths == info.width * info.height * (info.samples // info.batch_size) * info.batch_size
        j.release()


def test_jobs_with_different_samplers_in_one_mix(ctx, mixed_jobs):
    """Jobs of both samplers (RTGEMS and PMJ) and with the environment as a
    light share the fused queues: each job's sampler and estimator travel
    with its parameters, so every image still equals its single render."""
    flavours = [dict(sampler="pmj"), dict(sampler="rtgems"), dict(sampler="pmj", env_is=True)]
    alone = [g.render(sd, info, **kw) for (g, sd, info), kw in zip(mixed_jobs, flavours)]
    jobs = [g.submit(sd, info, **kw) for (g, sd, info), kw in zip(mixed_jobs, flavours)]
    for k, j in enumerate(jobs):
        _same(j.result(), alone[k])
        j.release()
    # and the PMJ images differ from the RTGEMS ones of the same requests
    g, sd, info = mixed_jobs[0]
    assert not np.array_equal(g.render(sd, info).radiance, alone[0].radiance)


def test_many_small_jobs_and_device_outputs(ctx, mixed_jobs):
    torch = pytest.importorskip("torch")
    g, sd, info = mixed_jobs[0]
    ref = g.render(sd, info)
    bufs = [{k: torch.zeros((info.height, info.width, 4), dtype=torch.float32, device="cuda")
             for k in ("radiance", "albedo", "normal")} for _ in range(24)]
    jobs = [g.submit(sd, info, outputs={k: v.data_ptr() for k, v in b.items()}) for b in bufs]
    for j in jobs:
        assert j.wait()
        j.release()
    torch.cuda.synchronize()
    for b in bufs:
        for k, v in b.items():
            assert np.array_equal(v.cpu().numpy(), getattr(ref, k))


def test_budget_admission_and_rejection(ctx, mixed_jobs):
    g, sd, info = mixed_jobs[0]
    ref = g.render(sd, info)
    fixed = ctx.engine_stats().fixed_bytes
    assert fixed > 0
    ctx.set_budget(fixed // 2)  # below the engine's own pool: every job is rejected
    with pytest.raises(N.VvptError) as ei:
        g.submit(sd, info)
    assert ei.value.status == N.BUDGET_EXCEEDED
    # room for about one job beside the pool: jobs are admitted one after another
    items = info.width * info.height * (info.samples // info.batch_size)
    per_job = 3 * (-(-items * 16 // 256) * 256) + 3 * (-(-info.width * info.height * 16 // 256) * 256)
    ctx.set_budget(fixed + per_job + per_job // 2)
    jobs = [g.submit(sd, info) for _ in range(6)]
    peak = 0
    while not all(j.done() for j in jobs):
        peak = max(peak, ctx.engine_stats().job_bytes)
    assert peak <= per_job + per_job // 2
    for j in jobs:
        _same(j.result(), ref)
        j.release()
    ctx.set_budget(0)


def test_zero_work_job_clears_outputs(ctx, mixed_jobs):
    g, sd, _ = mixed_jobs[0]
    info = RenderInfo(samples=2, depth=4, batch_size=4, width=16, height=8, write_files=False)
    j = g.submit(sd, info)
    r = j.result()
    assert not r.radiance.any() and not r.albedo.any()
    j.release()


def test_wait_timeout_and_scene_in_use(ctx):
    e, _ = scenes.cornell_box(4)
    g = ctx.upload(e.scene.build())
    info = RenderInfo(samples=256, depth=8, batch_size=4, width=512, height=512, write_files=False)
    sd = e.scene.scene_data(512, 512)
    j = g.submit(sd, info)
    assert j.wait(0.01) is False  # a 67M-path job is not done after 10 ms
    st = ctx.lib.vvpt_scene_release(ctx.handle, g.handle)
    assert st == N.NOT_READY
    with pytest.raises(N.VvptError):
        j.release()  # still running
    assert j.wait()
    j.release()
    g.release()


def test_render_batch_entry_point(ctx, mixed_jobs):
    alone = [g.render(sd, info) for g, sd, info in mixed_jobs]
    n = len(mixed_jobs)
    handles = (C.c_void_p * n)(*[g.handle for g, _, _ in mixed_jobs])
    sds = (N.SceneData * n)(*[sd for _, sd, _ in mixed_jobs])
    ris = (N.RenderInfo * n)(*[N.RenderInfo(i.samples, i.depth, i.batch_size, i.width, i.height, 0)
                               for _, _, i in mixed_jobs])
    outs_np = [{k: np.zeros((i.height, i.width, 4), np.float32) for k in ("radiance", "albedo", "normal")}
               for _, _, i in mixed_jobs]
    outs = (N.Outputs * n)(*[N.Outputs(o["radiance"].ctypes.data, o["albedo"].ctypes.data, o["normal"].ctypes.data,
                                       None, 0) for o in outs_np])
    ctx.check(ctx.lib.vvpt_render_batch(ctx.handle, n, handles, sds, ris, outs))
    for o, a in zip(outs_np, alone):
        for k in ("radiance", "albedo", "normal"):
            assert np.array_equal(o[k], getattr(a, k))
