"""Generates tests/golden/meshlight_orders.npz with the CPU oracle.

The reference's MeshLight scene (src/bin/unittests/RenderTests.cpp:643-689)
has an emissive plane that cuts into the glossy sphere. A BSDF-direction
emitter ray that reaches the plane's front can go on to hit the sphere behind
it, and the reference's any-hit shader for these rays
(shaders/pt/rayNEE.rahit.glsl:43-131) keeps whichever candidate the hardware
traversal reports first: the emitter (radiance added) or the sphere (ray
stopped, nothing added). The oracle renders the scene with both ends of the
possible orders in one pass (oracle.render(..., alt_order=True)): nearest
candidate first, the defined order of this library, and instance-box-entry
order. The pixels where the two images differ and both images' values there
are stored, so that the GPU tests can check the reference's golden against
the bracket without the multi-minute CPU render.

Run: python tests/golden/make_meshlight_orders.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import reference_scenes as R  # noqa: E402
from oracle import oracle  # noqa: E402


def render_orders():
    """Full-image MeshLight render in both candidate orders (oracle)."""
    e, info, _ = R.BUILDERS["MeshLight"]()
    fs = e.scene.build()
    sd = e.scene.scene_data(info.width, info.height)
    out = oracle.render(fs, sd, info, alt_order=True)
    return out["radiance"][..., :3], out["radiance_alt"][..., :3]


def main() -> None:
    near, alt = render_orders()
    diff = (near != alt).any(-1).reshape(-1)
    pix = np.nonzero(diff)[0].astype(np.uint32)
    np.savez_compressed(Path(__file__).with_name("meshlight_orders.npz"), pixels=pix,
                        nearest=near.reshape(-1, 3)[pix].astype(np.float32),
                        alt=alt.reshape(-1, 3)[pix].astype(np.float32))
    print(f"{pix.size} order-dependent pixels")


if __name__ == "__main__":
    main()
