"""Generates tests/golden/reference_assets.npz from the reference tree.

Contents: the parsed OBJ arrays of assets/models/{cube,plane,uvsphere}.obj
(positions, uvs, normals, triangulated corner indices) and the RGBE bytes of
the twelve golden images of src/bin/unittests/RenderTests.cpp whose scenes
can be rebuilt from assets present in the reference tree. The GPU machines do
not have the reference tree, so the tests read this file instead.

Run: python tests/golden/make_fixtures.py <reference_root>
(reference_root: the top of a kwstanths/vviewer checkout)
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from vviewer_gb300.assets import obj_arrays, read_hdr_rgbe  # noqa: E402

GOLDENS = ["FurnacePBR", "FurnaceLambert", "PointLight", "DirectionalLight", "MeshLight", "Volume3", "Volume4",
           "Volume5", "Volume7", "Volume8", "Volume9", "SharedComponents"]
MODELS = ["cube", "plane", "uvsphere"]


def main(ref_root: str) -> None:
    ref = Path(ref_root)
    out = {}
    for m in MODELS:
        a = obj_arrays(ref / "assets" / "models" / f"{m}.obj")
        out[f"{m}_name"] = np.array(a["name"])
        out[f"{m}_v"] = a["v"].astype(np.float32)
        out[f"{m}_vt"] = a["vt"].astype(np.float32)
        out[f"{m}_vn"] = a["vn"].astype(np.float32)
        out[f"{m}_f"] = a["f"].astype(np.int32)
    for g in GOLDENS:
        out[f"golden_{g}"] = read_hdr_rgbe(ref / "assets" / "unittests" / f"{g}_ref.hdr")
    np.savez_compressed(Path(__file__).with_name("reference_assets.npz"), **out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_fixtures.py <reference_root>")
    main(sys.argv[1])
