"""Seeded ray sets for the closest-hit parity tests (GPU kernel and the
host-compiled traversal against the oracle)."""
import numpy as np

import reference_scenes as R
from vviewer_gb300 import scenes


def world_triangles(fs):
    """World-space vertices of every TLAS triangle: (T x 3 x 3)."""
    out = []
    for inst in fs.instances:
        if not inst.flags & 1:
            continue
        m = fs.meshes[inst.mesh_index]
        M = np.array(list(inst.model), dtype=np.float64).reshape(4, 4).T
        p = m.vertices["position"][m.indices.astype(np.int64)].astype(np.float64)
        w = p @ M[:3, :3].T + M[:3, 3]
        out.append(w)
    return np.concatenate(out)


def make_rays(fs, n, seed, lo, hi):
    rng = np.random.default_rng(seed)
    tris = world_triangles(fs)
    k = n // 2
    # random rays
    o1 = rng.uniform(lo, hi, (k, 3))
    d1 = rng.normal(size=(k, 3))
    # rays aimed at triangle interiors, edges and vertices (watertightness, ties)
    pick = tris[rng.integers(0, len(tris), n - k)]
    bc = rng.dirichlet([1, 1, 1], n - k)
    kind = rng.integers(0, 3, n - k)
    bc[kind == 1, 2] = 0.0  # edge v0-v1
    bc[kind == 2] = [1.0, 0.0, 0.0]  # vertex
    bc /= bc.sum(1, keepdims=True)
    target = (pick * bc[:, :, None]).sum(1)
    o2 = rng.uniform(lo, hi, (n - k, 3))
    d2 = target - o2
    o = np.concatenate([o1, o2])
    d = np.concatenate([d1, d2])
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    tmin = np.where(rng.random(n) < 0.5, 0.0, 1e-3)
    rays = np.concatenate([o, tmin[:, None], d, np.full((n, 1), 1e4)], 1).astype(np.float32)
    return rays



HIT_SCENES = {
    "cornell": (lambda: scenes.cornell_box(1)[0], (-0.2, 1.2)),
    "two_balls_mesh_light": (lambda: R.mesh_light()[0], (-3.0, 4.0)),
    "volume_cube": (lambda: R.volume(9)[0], (-3.0, 4.0)),
    "shared_components": (lambda: R.shared_components()[0], (-160.0, 160.0)),
    "displaced_spheres": (lambda: scenes.cornell_medium(3, freq=12, spheres=8)[0], (-0.2, 1.2)),
}


def make_near_rays(fs, n, seed):
    """Rays that start just off a triangle (1e-4 to 1e-2 along its normal, on
    either side) and leave at a random angle: hits at t far below the scene
    size, where the triangle test's absolute rounding dominates t and the
    culling margins must still keep every candidate."""
    rng = np.random.default_rng(seed)
    tris = world_triangles(fs)
    pick = tris[rng.integers(0, len(tris), n)]
    bc = rng.dirichlet([1, 1, 1], n)
    p = (pick * bc[:, :, None]).sum(1)
    nrm = np.cross(pick[:, 1] - pick[:, 0], pick[:, 2] - pick[:, 0])
    nrm /= np.maximum(np.linalg.norm(nrm, axis=1, keepdims=True), 1e-30)
    off = rng.uniform(1e-4, 1e-2, (n, 1)) * rng.choice([-1.0, 1.0], (n, 1))
    o = p + off * nrm
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([o, np.zeros((n, 1)), d, np.full((n, 1), 1e4)], 1).astype(np.float32)


def many_lights_scene(width: int = 64, height: int = 64, samples: int = 16):
    """The Cornell box with 40 small emissive quads: more emissive instances
    than the 32 boxes the prefilter keeps, so the boxes are merged."""
    from vviewer_gb300.scene import MaterialLambert, Transform

    e, info = scenes.cornell_box(2, width, height, samples, 8, 4)
    lamp = e.create_material(MaterialLambert, "lamp")
    lamp.emissive = [3.0, 3.0, 3.0, 1.0]
    quad = next(so.mesh for so in e.scene.objects_flat() if so.name == "light")
    rng = np.random.default_rng(4)
    for k in range(40):
        # the ceiling quad scaled by 0.3 and moved inside the room, facing down
        so = e.scene.add_scene_object(f"lamp{k}", Transform((rng.uniform(0.0, 0.65), rng.uniform(-0.05, 0.6),
                                                             rng.uniform(0.0, 0.65)), (0.3, 0.3, 0.3)))
        so.mesh = quad
        so.material = lamp
    return e, info
