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
from raygen import HIT_SCENES, make_near_rays, make_rays
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
