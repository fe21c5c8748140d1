"""The device traversal (traverse.cuh) compiled for the host over the packed
scene arrays vvpt_scene_upload uploads, against the oracle: closest hits
bit-identical. This checks the traversal's bookkeeping (single stack across
TLAS and BLAS, instance entry and return, child order, culling margins)
without a GPU; the GPU parity tests repeat the comparison on the kernel."""
import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle
from raygen import HIT_SCENES, make_near_rays, make_rays, many_lights_scene
from vviewer_gb300.renderer import HIT_DTYPE

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "vviewer_gb300" / "csrc"
HARNESS = Path(__file__).resolve().parent / "host_traverse" / "host_traverse.cpp"
OUT = Path(__file__).resolve().parent / "_build" / "libhost_traverse.so"


def _lib_path(wide):
    return OUT.with_name(f"libhost_traverse_{'wide' if wide else 'binary'}.so")


def _cuda_include():
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "include" / "vector_types.h").exists():
            return str(Path(cand) / "include")
    pytest.skip("CUDA headers (vector_types.h) not found")


@pytest.fixture(scope="module", params=[True, False], ids=["wide_blas", "binary_blas"])
def host_lib(request):
    """The harness built for both BLAS layouts: compressed 8-wide nodes (the
    default) and binary nodes (VVPT_BLAS_WIDE=0)."""
    wide = request.param
    out = _lib_path(wide)
    srcs = [HARNESS, CSRC / "scene_pack.cpp", CSRC / "bvh_build.cpp", CSRC / "bvh_wide.cpp"]
    deps = srcs + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "vvpt.h"]
    if not out.exists() or out.stat().st_mtime < max(p.stat().st_mtime for p in deps):
        out.parent.mkdir(exist_ok=True)
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread",
               f"-DVVPT_BLAS_WIDE={int(wide)}", "-I", _cuda_include(), "-I", str(ROOT / "include"), "-I", str(CSRC),
               *map(str, srcs), "-o", str(out)]
        subprocess.run(cmd, check=True, capture_output=True)
    lib = C.CDLL(str(out))
    lib.host_trace_closest.restype = C.c_int
    lib.host_trace_closest.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.POINTER(C.c_uint32),
                                       C.c_char_p, C.c_int]
    lib.host_may_reach_emitter.restype = C.c_int
    lib.host_may_reach_emitter.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.POINTER(C.c_uint32),
                                           C.c_char_p, C.c_int]
    return lib


def host_trace(lib, fs, rays):
    desc = fs.desc()
    rays = np.ascontiguousarray(rays, dtype=np.float32)
    hits = np.zeros(rays.shape[0], dtype=HIT_DTYPE)
    err = C.c_uint32(0)
    msg = C.create_string_buffer(256)
    st = lib.host_trace_closest(C.addressof(desc), rays.ctypes.data, rays.shape[0], hits.ctypes.data, C.byref(err),
                                msg, 256)
    assert st == 0, msg.value
    assert err.value == 0, f"traversal status bits {err.value}"
    return hits


def assert_hits_equal(hh, ho):
    for f in ("instance", "primitive", "t", "u", "v"):
        eq = hh[f] == ho[f]
        assert eq.all(), f"{f}: {np.count_nonzero(~eq)} of {len(eq)} differ, first {np.nonzero(~eq)[0][:5]}"


@pytest.mark.parametrize("name", list(HIT_SCENES))
def test_host_traversal_matches_oracle(host_lib, name):
    build, (lo, hi) = HIT_SCENES[name]
    fs = build().scene.build()
    n = 40_000 if name != "shared_components" else 10_000
    rays = np.concatenate([make_rays(fs, n, 7, lo, hi), make_near_rays(fs, n // 4, 11)])
    hh = host_trace(host_lib, fs, rays)
    ho = oracle.trace_closest(fs, rays)
    assert (hh["instance"] != 0xFFFFFFFF).mean() > 0.3
    assert_hits_equal(hh, ho)


def test_hit_just_above_coplanar_faces(host_lib):
    """A ray from 1.5 mm below the Cornell floor, where a box's bottom face is
    coplanar with the floor: the floor's t is 2 ulps smaller than the box's,
    but the floor's slab entry exceeds both by 1.2e-5 relative, so a purely
    relative culling margin drops the floor whenever the box is found first."""
    from vviewer_gb300 import scenes

    fs = scenes.cornell_box(1)[0].scene.build()
    ray = np.array([[0.18627457, -0.001458, 0.42422411, 0.0, 0.55179465, 0.43452245, -0.71183771, 1e4]],
                   dtype=np.float32)
    hh = host_trace(host_lib, fs, ray)
    ho = oracle.trace_closest(fs, ray)
    assert_hits_equal(hh, ho)
    assert hh["instance"][0] == 0


def _emissive_instances(fs):
    out = np.zeros(len(fs.instances), dtype=bool)
    for k, inst in enumerate(fs.instances):
        m = fs.materials[inst.material_index]
        e = [abs(m.emissive[c] * m.emissive[3]) for c in range(3)]
        out[k] = bool(inst.flags & 1) and max(e) > 0.05
    return out


@pytest.mark.parametrize("name", ["cornell", "two_balls_mesh_light", "displaced_spheres", "many_lights"])
def test_emitter_prefilter_keeps_every_ray_that_reaches_an_emitter(host_lib, name):
    """The emitter-ray prefilter (traverse.cuh may_reach_emitter over the
    packed emissive boxes) must pass every ray whose closest hit is an
    emissive instance: those are the rays whose emitter contribution can be
    non-zero. Rays start anywhere, on surfaces, and just off surfaces."""
    if name == "many_lights":
        fs, lo, hi = many_lights_scene()[0].scene.build(), -0.2, 1.2
    else:
        build, (lo, hi) = HIT_SCENES[name]
        fs = build().scene.build()
    rays = np.concatenate([make_rays(fs, 40_000, 3, lo, hi), make_near_rays(fs, 20_000, 5)])
    hits = host_trace(host_lib, fs, rays)
    desc = fs.desc()
    r = np.ascontiguousarray(rays, dtype=np.float32)
    may = np.zeros(r.shape[0], dtype=np.uint8)
    nb = C.c_uint32(0)
    msg = C.create_string_buffer(256)
    assert host_lib.host_may_reach_emitter(C.addressof(desc), r.ctypes.data, r.shape[0], may.ctypes.data,
                                           C.byref(nb), msg, 256) == 0, msg.value
    emissive = _emissive_instances(fs)
    hit = hits["instance"] != 0xFFFFFFFF
    reach = np.zeros(len(hits), dtype=bool)
    reach[hit] = emissive[hits["instance"][hit].astype(np.int64)]
    assert reach.sum() > 50, reach.sum()
    assert may[reach].all(), f"{np.count_nonzero(may[reach] == 0)} rays reach an emitter but were rejected"
    assert 1 <= nb.value <= 32
    if name == "many_lights":
        assert nb.value == 32  # 41 emissive instances merged into 32 boxes
    if name in ("cornell", "displaced_spheres"):
        # one small ceiling light: most rays are rejected
        assert may.mean() < 0.5, may.mean()
