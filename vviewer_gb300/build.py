"""Builds libvvpt.so in-tree for sm_103a.

Translation units compile in parallel (nvcc for .cu, g++ for host-only .cpp)
and link into vviewer_gb300/_lib/libvvpt.so with the CUDA runtime linked
statically. Rebuilds only when a source or header is newer than the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_lib"
BUILD_DIR = PKG / "_build"
LIB = OUT_DIR / "libvvpt.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -ffp-contract=off on the host compilers: the scene packing (inverse
# transforms, baked small-instance triangles) rounds the same on x86 and Arm
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-I", str(ROOT / "include"), "-I", str(CSRC)]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off", "-I", str(ROOT / "include"),
             "-I", str(CSRC)]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libvvpt.so")


def _sources():
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _newest_input() -> float:
    files = list(CSRC.glob("*")) + list((ROOT / "include").glob("*.h")) + [Path(__file__)]
    return max(f.stat().st_mtime for f in files if f.is_file())


def _compile(src: Path, nvcc: str, extra: list[str], defines: list[str], build_dir: Path = BUILD_DIR) -> Path:
    obj = build_dir / (src.stem + src.suffix.replace(".", "_") + ".o")
    dflags = [f"-D{d}" for d in defines]
    if src.suffix == ".cu":
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, *dflags, *extra, "-c", str(src), "-o", str(obj)]
    else:
        cmd = ["g++", *CXX_FLAGS, *dflags, "-I", str(Path(nvcc).parent.parent / "include"), "-c", str(src), "-o",
               str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False, extra_nvcc: list[str] | None = None,
          defines: list[str] | None = None, out: Path | None = None, build_dir: Path | None = None) -> Path:
    """Compiles and links libvvpt.so if it is missing or stale; returns its path.
    `defines` (NAME=VALUE) reach both compilers, e.g. VVPT_BLAS_WIDE=1 for the
    compressed 8-wide BLAS layout; `extra_nvcc` only nvcc. `out` and
    `build_dir` put a variant build beside the default one (the library path
    and the object folder)."""
    lib = Path(out) if out else LIB
    objdir = Path(build_dir) if build_dir else BUILD_DIR
    if lib.exists() and not force and lib.stat().st_mtime >= _newest_input():
        return lib
    nvcc = _nvcc()
    lib.parent.mkdir(parents=True, exist_ok=True)
    objdir.mkdir(parents=True, exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(lambda s: _compile(s, nvcc, extra_nvcc or [], defines or [], objdir), srcs))
    tmp = lib.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, lib)
    if verbose:
        print(f"built {lib}")
    return lib


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
