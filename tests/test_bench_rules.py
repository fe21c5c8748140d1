"""bench.py's host-side rules that need no GPU: the operating point of the
converged workload and the image error it is measured with."""
import sys
from pathlib import Path

import numpy as np
import torch

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
import bench  # noqa: E402


def _sweep(errs, gains):
    return [{"spp": s, "rel_rmse_denoised": e, "gain_at_equal_error": g}
            for s, e, g in zip((4, 8, 16, 32, 64), errs, gains)]


def test_operating_point_is_the_fewest_spp_meeting_the_target():
    sw = _sweep([0.5, 0.02, 0.009, 0.008, 0.005], [9.0, 8.0, 7.0, 5.0, 2.0])
    pick, rule = bench.pick_operating_point(sw, 0.01)
    assert pick["spp"] == 16 and rule.startswith("fewest")


def test_operating_point_without_the_target_takes_the_largest_equal_error_gain():
    sw = _sweep([0.6, 0.5, 0.45, 0.44, 0.41], [8.0, 10.7, 7.3, None, 2.6])
    pick, rule = bench.pick_operating_point(sw, 0.01)
    assert pick["spp"] == 8 and "largest gain" in rule


def test_rel_rmse_is_image_level_over_rgb():
    ref = torch.zeros((2, 2, 4), dtype=torch.float32)
    ref[..., :3] = torch.tensor([1.0, 2.0, 3.0])
    img = ref.clone()
    img[0, 0, :3] += 1.0
    img[..., 3] = 7.0  # alpha is not measured
    expect = np.sqrt(3.0 / (4 * (1 + 4 + 9)))
    assert abs(bench._rel_rmse(img, ref) - expect) < 1e-12
