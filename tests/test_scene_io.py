"""Scene files (vviewer's JSON format, core/io/Import.cpp / Export.cpp):
export then import reproduces the camera, materials, lights, object
transforms and geometry; the reference's value notations parse; PNG
textures decode."""
import json

import numpy as np
import pytest

from vviewer_gb300 import scenes
from vviewer_gb300.renderer import write_png
from vviewer_gb300.scene import EnvironmentType, Engine
from vviewer_gb300.scene_io import export_scene, import_scene, read_png


def _world_tris(fs):
    out = []
    for inst in fs.instances:
        if not inst.flags & 1:
            continue
        m = fs.meshes[inst.mesh_index]
        M = np.array(list(inst.model), dtype=np.float64).reshape(4, 4).T
        p = m.vertices["position"][m.indices.astype(np.int64)].astype(np.float64)
        out.append(np.sort((p @ M[:3, :3].T + M[:3, 3]).reshape(-1, 9), axis=0))
    return out


def test_export_import_round_trip(tmp_path):
    e, info = scenes.cornell_medium(3, 64, 48, 4, 8, 4, freq=4, spheres=2)
    s = e.scene
    s.environment_map = scenes.procedural_sky(64, 32, sun_peak=50.0, sun_sigma_deg=5.0)
    s.environment_type = EnvironmentType.SOLID_COLOR_WITH_HDRI_LIGHTING
    s.camera.lens_radius = 0.03
    export_scene(e, tmp_path / "scene.json")
    e2 = import_scene(tmp_path / "scene.json")
    a, b = e.scene.build(), e2.scene.build()
    assert len(a.instances) == len(b.instances)

    def mat_bytes(fs, i):
        m = fs.materials[int(i)]
        bm = bytearray(bytes(m))
        if m.uv_tiling[2] == 3.0:  # volume: the file holds 3 components of sigma_a / sigma_s
            for k in (12, 13, 14, 15, 28, 29, 30, 31):
                bm[k] = 0
        return bm

    # the imported scene also holds the OBJ files' own materials (each model's
    # "<stem>:DefaultMaterial"), so materials are compared by content, not slot
    for x, y in zip(a.instances, b.instances):
        assert np.allclose(list(x.model), list(y.model), atol=1e-6)
        assert mat_bytes(a, x.material_index) == mat_bytes(b, y.material_index) and x.flags == y.flags
        for k in (1, 2):
            vx, vy = list(x.id)[k], list(y.id)[k]
            assert (vx == -1) == (vy == -1)
            if vx != -1:
                assert mat_bytes(a, vx) == mat_bytes(b, vy)
    assert len(b.materials) >= len(a.materials)
    assert len(a.lights) == len(b.lights)
    for x, y in zip(a.lights, b.lights):
        assert np.allclose(list(x.position), list(y.position), atol=1e-5)
    for ta, tb in zip(_world_tris(a), _world_tris(b)):
        assert np.allclose(ta, tb, atol=1e-5)
    sa, sb = e.scene.scene_data(64, 48), e2.scene.scene_data(64, 48)
    assert np.allclose(list(sa.view), list(sb.view), atol=1e-5)
    assert np.allclose(list(sa.projection), list(sb.projection), atol=1e-6)
    assert list(sa.exposure) == list(sb.exposure) and list(sa.background) == list(sb.background)
    env2 = e2.scene.environment_map
    assert env2.shape == (32, 64, 4)
    # RGBE: 8 mantissa bits under a shared exponent (error relative to the largest channel)
    orig = s.environment_map[..., :3]
    assert (np.abs(env2[..., :3] - orig) <= orig.max(-1, keepdims=True) / 128.0).all()


def test_reference_value_notations(tmp_path):
    (tmp_path / "tri.obj").write_text("o tri\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    doc = {
        "camera": {"position": {"x": 0, "y": 0, "z": 3}, "rotation": [0, 0, 0], "fov": 45},
        "models": [{"name": "tri", "filepath": "tri.obj"}],
        "materials": [{"name": "red", "type": "LAMBERT", "albedo": {"value": {"r": 1, "g": 0, "b": 0, "a": 1}}},
                      {"name": "fog", "type": "VOLUME", "scattering": {"value": 0.5}, "absorption": {"value": [0.1]},
                       "g": 0.3}],
        "lights": [{"name": "sun", "type": "DIRECTIONAL", "color": [1, 0.5, 0.25], "intensity": 2.0}],
        "scene": [{"name": "a", "transform": {"position": [1, 2, 3], "rotation": [0, 90, 0], "scale": 2.0},
                   "mesh": {"modelName": "tri", "submesh": "tri"}, "material": {"name": "red"},
                   "volume": {"backFacing": "fog"},
                   "children": [{"name": "b", "light": {"name": "sun"},
                                 "transform": {"rotation": {"x": 0, "y": 0, "z": 0, "w": 1}}}]}],
        "environment": {"environmentType": 0, "backgroundColor": 0.25},
    }
    (tmp_path / "s.json").write_text(json.dumps(doc))
    e = import_scene(tmp_path / "s.json")
    red = e.material("red")
    assert red.albedo == [1.0, 0.0, 0.0, 1.0]
    fog = e.material("fog")
    assert fog.sigma_s[:3] == [0.5] * 3 and fog.sigma_a[:3] == [0.1] * 3 and fog.g == pytest.approx(0.3)
    assert e.light("sun").color == [1.0, 0.5, 0.25, 2.0]
    a = e.scene.roots[0]
    assert a.volume_back is fog and a.children[0].light.name == "sun"
    # Euler (0, 90, 0) degrees: +x maps to -z
    M = a.model_matrix()
    assert np.allclose(M[:3, 0] / 2.0, [0, 0, -1], atol=1e-6)
    assert e.scene.background_color[:3] == [0.25] * 3
    assert e.scene.camera.fov == 45


@pytest.mark.parametrize("mode", ["rgb", "rgba", "grey"])
def test_png_decoder(tmp_path, mode):
    rng = np.random.default_rng(1)
    img = rng.integers(0, 256, (13, 17, 4), dtype=np.uint8)
    if mode == "rgb":
        img[..., 3] = 255
    if mode == "grey":
        img[..., 1] = img[..., 2] = img[..., 0]
        img[..., 3] = 255
    write_png(tmp_path / "t.png", img)
    assert (read_png(tmp_path / "t.png") == img).all()
