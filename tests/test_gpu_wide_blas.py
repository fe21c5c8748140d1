"""The compressed 8-wide BLAS layout (build option VVPT_BLAS_WIDE=1,
csrc/bvh_wide.cpp) on the GPU. The library is built a second time with the
option, in-tree beside the default build, and driven from a child process
(one process loads one libvvpt.so). Closest hits must be bit-identical to the oracle's, and
renders bit-identical to the default (binary BLAS) build's: the hit and
any-hit candidate orders are fixed by (t, instance, primitive), not by the
BVH, so the node layout cannot change an image."""
import subprocess
import sys
import textwrap
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle
from raygen import HIT_SCENES, make_near_rays, make_rays
from vviewer_gb300 import scenes

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent
HIT_NAMES = ("cornell", "volume_cube", "displaced_spheres")


def _render_cases():
    return {"cornell": scenes.cornell_box(6, 64, 64, 32, 8, 4),
            "medium": scenes.cornell_medium(2, 48, 32, 16, 12, 4, freq=12, spheres=8)}


CHILD = textwrap.dedent("""
    import sys
    import numpy as np
    sys.path[:0] = [sys.argv[3], sys.argv[3] + "/tests"]
    from vviewer_gb300 import _native as N
    N.load(sys.argv[1])
    from vviewer_gb300 import Context
    from raygen import HIT_SCENES, make_near_rays, make_rays
    import test_gpu_wide_blas as T
    ctx = Context(0)
    out = {}
    for name in T.HIT_NAMES:
        build, (lo, hi) = HIT_SCENES[name]
        fs = build().scene.build()
        g = ctx.upload(fs)
        h = g.trace_closest(np.concatenate([make_rays(fs, 60_000, 7, lo, hi), make_near_rays(fs, 20_000, 11)]))
        for f in h.dtype.names:
            out[f"hit_{name}_{f}"] = h[f]
        g.release()
    for name, (e, info) in T._render_cases().items():
        fs = e.scene.build()
        g = ctx.upload(fs)
        r = g.render(e.scene.scene_data(info.width, info.height), info)
        out[f"rad_{name}"] = r.radiance
        out[f"alb_{name}"] = r.albedo
        g.release()
    ctx.close()
    np.savez(sys.argv[2], **out)
""")


def test_wide_blas_build_matches_oracle_and_binary_build(ctx, tmp_path):
    from vviewer_gb300 import build as B

    # in-tree, beside the default build (vviewer_gb300/_lib, _build: not committed)
    lib = B.build(force=True, defines=["VVPT_BLAS_WIDE=1"], out=B.OUT_DIR / "variants" / "libvvpt_wide.so",
                  build_dir=B.BUILD_DIR / "wide")
    res_file = tmp_path / "wide.npz"
    script = tmp_path / "child.py"
    script.write_text(CHILD)
    run = subprocess.run([sys.executable, str(script), str(lib), str(res_file), str(ROOT)], capture_output=True,
                         text=True, timeout=900)
    assert run.returncode == 0, run.stderr[-4000:]
    wide = np.load(res_file)
    for name in HIT_NAMES:
        build, (lo, hi) = HIT_SCENES[name]
        fs = build().scene.build()
        ho = oracle.trace_closest(fs, np.concatenate([make_rays(fs, 60_000, 7, lo, hi),
                                                      make_near_rays(fs, 20_000, 11)]))
        assert (wide[f"hit_{name}_instance"] != 0xFFFFFFFF).mean() > 0.3
        for f in ("instance", "primitive", "t", "u", "v"):
            eq = wide[f"hit_{name}_{f}"] == ho[f]
            assert eq.all(), f"{name} {f}: {np.count_nonzero(~eq)} differ"
    for name, (e, info) in _render_cases().items():
        fs = e.scene.build()
        g = ctx.upload(fs)
        r = g.render(e.scene.scene_data(info.width, info.height), info)
        g.release()
        assert np.array_equal(r.radiance, wide[f"rad_{name}"]), name
        assert np.array_equal(r.albedo, wide[f"alb_{name}"]), name
