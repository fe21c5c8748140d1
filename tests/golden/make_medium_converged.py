"""Generates tests/golden/medium_converged.npz: the CPU oracle's converged,
FP64-accumulated render of a small view of the headline scene, the reference
of the GPU's converged-image test.

Scene: scenes.cornell_medium(seed 4) at its full geometry (the Cornell room
filled with the homogeneous medium, eight displaced icospheres at frequency
79, 998,560 triangles), depth 12, seen through a 12-degree field of view
(spheres and back wall, not the light) at 3 x 2 pixels. The oracle renders
2^25 samples per pixel in batches of 256 with double-precision accumulation;
the file holds each pixel's mean radiance and its Monte Carlo standard error
from the batch sums. About 13 minutes on 8 cores.

Run: python tests/golden/make_medium_converged.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle  # noqa: E402
from vviewer_gb300 import scenes  # noqa: E402

SAMPLES = 1 << 25
BATCH = 256


def scene(samples: int, batch: int):
    """The converged test's scene and render info."""
    e, info = scenes.cornell_medium(4, 3, 2, samples, 12, batch, freq=79, spheres=8)
    e.scene.camera.fov = 12.0
    return e, info


def mean_and_se(img, m2, batches):
    """Per-pixel mean (the image: the sum of the batch contributions) and
    its standard error from the sum of the batch contributions' squares."""
    x = img[..., :3].astype(np.float64)
    var = np.maximum(batches * m2[..., :3].astype(np.float64) - x * x, 0.0) / max(batches - 1, 1)
    return x, np.sqrt(var)


def main() -> None:
    e, info = scene(SAMPLES, BATCH)
    fs = e.scene.build()
    sd = e.scene.scene_data(info.width, info.height)
    out = oracle.render(fs, sd, info, fp64=True)
    mean, se = mean_and_se(out["radiance"], out["radiance_m2"], info.samples // info.batch_size)
    np.savez_compressed(Path(__file__).with_name("medium_converged.npz"), mean=mean, se=se,
                        samples=np.int64(SAMPLES), batch=np.int64(BATCH))
    print("relative RMSE of the reference (noise):", float(np.sqrt((se ** 2).sum() / (mean ** 2).sum())))


if __name__ == "__main__":
    main()
