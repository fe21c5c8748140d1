"""Host-side logic: C ABI exports and struct layouts, scene flattening in the
reference's order, camera matrices, RGBE and OBJ I/O. No GPU needed."""
import ctypes as C
import re
import subprocess
import textwrap
from pathlib import Path

import numpy as np
import pytest

import reference_scenes as R
from conftest import HAS_GPU, ROOT
from vviewer_gb300 import _native as N
from vviewer_gb300 import assets, scenes
from vviewer_gb300.scene import (EnvironmentType, Engine, LightType, MaterialLambert, MaterialPBRStandard,
                                 MaterialVolume, Transform, look_at, perspective, quat_from_euler, radians)

HEADER = ROOT / "include" / "vvpt.h"


def header_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"VVPT_API\s+[^;]*?\b(vvpt_\w+)\s*\(", text)))


def test_library_exports_every_header_symbol(native_lib):
    syms = header_symbols()
    assert len(syms) >= 12
    out = subprocess.run(["nm", "-D", "--defined-only", str(N.LIB_PATH)], capture_output=True, text=True, check=True)
    exported = set(re.findall(r"\b(vvpt_\w+)\b", out.stdout))
    missing = [s for s in syms if s not in exported]
    assert not missing, f"declared in vvpt.h but not exported: {missing}"
    # the ctypes binding covers exactly the header
    assert sorted(N.declared_symbols()) == syms
    for s in syms:
        assert getattr(native_lib, s) is not None


def test_struct_layouts_match_c_header(tmp_path):
    names = ["vvpt_vertex", "vvpt_mesh_desc", "vvpt_material", "vvpt_instance", "vvpt_light_data",
             "vvpt_light_instance", "vvpt_texture_desc", "vvpt_scene_desc", "vvpt_scene_data", "vvpt_render_info",
             "vvpt_outputs", "vvpt_ray", "vvpt_hit", "vvpt_render_stats", "vvpt_tuning"]
    src = tmp_path / "sizes.c"
    body = "\n".join(f'    printf("{n} %zu\\n", sizeof({n}));' for n in names)
    src.write_text(textwrap.dedent(f"""
        #include <stdio.h>
        #include "vvpt.h"
        int main(void) {{
        {body}
            return 0;
        }}"""))
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    c_sizes = dict(zip(out[0::2], map(int, out[1::2])))
    py = {"vvpt_vertex": N.Vertex, "vvpt_mesh_desc": N.MeshDesc, "vvpt_material": N.Material,
          "vvpt_instance": N.Instance, "vvpt_light_data": N.LightData, "vvpt_light_instance": N.LightInstance,
          "vvpt_texture_desc": N.TextureDesc, "vvpt_scene_desc": N.SceneDesc, "vvpt_scene_data": N.SceneData,
          "vvpt_render_info": N.RenderInfo, "vvpt_outputs": N.Outputs, "vvpt_ray": N.Ray, "vvpt_hit": N.Hit,
          "vvpt_render_stats": N.RenderStats, "vvpt_tuning": N.Tuning}
    for n in names:
        assert C.sizeof(py[n]) == c_sizes[n], n
    # reference GPU struct sizes: Vertex 68 B scalar, MaterialData 128 B,
    # LightData 64 B, LightInstance 64 B (structs.glsl, Instances.hpp)
    assert c_sizes["vvpt_vertex"] == 68
    assert c_sizes["vvpt_material"] == 128
    assert c_sizes["vvpt_light_data"] == 64
    assert c_sizes["vvpt_light_instance"] == 64


@pytest.mark.skipif(HAS_GPU, reason="checks the no-GPU error path")
def test_create_without_gpu_reports_device_error(native_lib):
    h = C.c_void_p()
    assert native_lib.vvpt_create(0, C.byref(h)) == 5  # VVPT_ERR_DEVICE
    assert native_lib.vvpt_create(0, None) == 1  # VVPT_ERR_INVALID_ARG


def test_null_arguments_are_rejected(native_lib):
    assert native_lib.vvpt_destroy(None) == 1
    assert native_lib.vvpt_scene_upload(None, None, None) == 1
    assert native_lib.vvpt_render(None, None, None, None, None) == 1
    assert native_lib.vvpt_progress(None, None) == 1
    assert native_lib.vvpt_set_bvh_builder(None, 2) == 1
    assert native_lib.vvpt_jpeg_decode(None, 0, None, None, None, None, 0) == 1
    assert native_lib.vvpt_version().startswith(b"vvpt")


# ---------------------------------------------------------------- scene flattening

def _two_object_scene():
    e = Engine()
    s = e.scene
    plane = e.add_mesh(scenes.mesh_from_triangles("q", scenes.quad((0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1))))
    box = e.add_mesh(scenes.unit_box())
    lam = e.create_material(MaterialLambert, "lam")
    glass = e.create_material(MaterialPBRStandard, "glass")
    glass.set_transparent(True)
    emit = e.create_material(MaterialPBRStandard, "emit")
    emit.emissive = [1.0, 1.0, 1.0, 5.0]
    vol = e.create_material(MaterialVolume, "vol")
    a = s.add_scene_object("a", Transform((0, 0, 0)))
    a.mesh, a.material = plane, lam
    t = s.add_scene_object("t", Transform((0, 1, 0)))
    t.mesh, t.material, t.volume_back = box, glass, vol
    b = s.add_scene_object("b", Transform((2, 0, 0)))
    b.mesh, b.material = box, lam
    m = s.add_scene_object("m", Transform((0, 3, 0), (2, 2, 2), (radians(90.0), 0.0, 0.0)))
    m.mesh, m.material = plane, emit
    pl = s.add_scene_object("pl", Transform((1, 2, 3)))
    pl.light = e.create_light("p", LightType.POINT_LIGHT)
    dl = s.add_scene_object("dl", Transform((0, 0, 0), (1, 1, 1), (radians(45.0), radians(90.0), 0.0)))
    dl.light = e.create_light("d", LightType.DIRECTIONAL_LIGHT)
    return e, (a, t, b, m, pl, dl)


def test_instance_slot_order_follows_instances_manager():
    # Instances.cpp:145-181: opaque mesh groups, then transparent objects, then lights
    e, (a, t, b, m, pl, dl) = _two_object_scene()
    fs = e.scene.build()
    ids = [int(i.id[0]) for i in fs.instances]
    assert ids == [a.id, m.id, b.id, t.id, pl.id, dl.id]
    flags = [i.flags for i in fs.instances]
    assert flags == [1, 1, 1, 1, 0, 0]
    # the transparent cube carries its back-facing volume in id.b
    assert fs.instances[3].id[2] == e.material("vol").index and fs.instances[3].id[1] == -1.0


def test_light_instances_follow_vulkan_instances_manager():
    e, (a, t, b, m, pl, dl) = _two_object_scene()
    fs = e.scene.build()
    assert fs.num_lights == 3  # point, directional, then mesh light
    p, d, ml = fs.lights
    assert (p.info[3], d.info[3], ml.info[3]) == (0, 1, 2)
    assert list(p.position)[:3] == pytest.approx([1, 2, 3])
    # directional: model matrix applied to +Z (VulkanInstances.cpp:84)
    mm = dl.model_matrix()
    assert list(d.position)[:3] == pytest.approx(list(mm[:3, 2]), abs=1e-6)
    # mesh light rows are the model matrix rows and info.g the InstanceData slot
    rows = np.array([list(ml.position), list(ml.position1), list(ml.position2)])
    assert np.allclose(rows, m.model_matrix()[:3, :], atol=1e-6)
    assert ml.info[1] == 1


def test_transform_and_camera_conventions():
    # identity rotation from zero Euler angles; forward = -Z, up = +Y
    q = quat_from_euler((0, 0, 0))
    assert np.allclose(q, [1, 0, 0, 0])
    t = Transform((1, 2, 3), (2, 2, 2), (0.0, radians(90.0), 0.0))
    m = t.model_matrix()
    assert np.allclose(m[:3, 3], [1, 2, 3])
    assert np.allclose(m[:3, :3] @ [1, 0, 0], [0, 0, -2], atol=1e-6)  # yaw 90: +X -> -Z
    v = look_at((0, 0, 5), (0, 0, 0), (0, 1, 0))
    assert np.allclose(v @ [0, 0, 0, 1], [0, 0, -5, 1], atol=1e-6)
    p = perspective(radians(90.0), 1.0, 0.5, 50.0)
    assert p[0, 0] == pytest.approx(1.0) and p[3, 2] == -1.0
    e, info = scenes.cornell_box(1)
    sd = e.scene.scene_data(256, 256)
    pinv = np.array(list(sd.projection_inverse), dtype=np.float64).reshape(4, 4).T
    # the flipped projection sends pixel row 0 (d.y = -1) to +y in camera space
    top = pinv @ [0.0, -1.0, 1.0, 1.0]
    assert top[1] > 0 and top[2] == pytest.approx(-1.0, abs=1e-6)
    assert list(sd.volumes) == [-1.0, 0.5, 50.0, 0.0]


def test_scene_data_camera_volume_and_background():
    e, info, tol = R.volume(8)
    sd = e.scene.scene_data(256, 256)
    assert sd.volumes[0] == float(e.material("volumematerial2").index)
    assert sd.volumes[2] == 10.0
    assert sd.background[3] == float(int(EnvironmentType.SOLID_COLOR))


def test_material_packing_matches_reference_layout():
    e = Engine()
    v = e.material("defaultVolume")
    pv = v.pack()
    # volume packing, VulkanMaterial.cpp:438-483
    assert list(pv.albedo) == pytest.approx(v.sigma_a) and list(pv.metallic_roughness_ao) == pytest.approx(v.sigma_s)
    assert pv.uv_tiling[2] == 3.0
    d = e.material("defaultMaterial").pack()
    assert list(d.albedo) == pytest.approx([0.8, 0.8, 0.8, 1.0])
    assert list(d.metallic_roughness_ao) == pytest.approx([0.5, 0.5, 1.0, 0.0])
    assert list(d.textures2)[:2] == [1, 2]  # whiteColor emissive, normalmapdefault
    assert e.material("defaultEmissive").is_emissive()
    assert not e.material("defaultMaterial").is_emissive()


# ---------------------------------------------------------------- I/O

@pytest.mark.parametrize("name", ["FurnacePBR", "PointLight", "Volume9", "SharedComponents"])
def test_rgbe_round_trip_on_reference_goldens(name, tmp_path):
    raw = R.golden_rgbe(name)
    rgb = assets.rgbe_decode(raw)
    assert (assets.rgbe_encode(rgb) == raw).all()
    f = tmp_path / "x.hdr"
    assets.write_hdr(f, rgb)
    assert (assets.read_hdr_rgbe(f) == raw).all()


def test_rgbe_edge_values():
    v = np.array([[[0.0, 0.0, 0.0], [1e-40, 0, 0], [1.0, 0.5, 0.25], [65504.0, 1.0, 0.0]]], dtype=np.float32)
    enc = assets.rgbe_encode(v)
    assert (enc[0, 0] == 0).all() and (enc[0, 1] == 0).all()
    dec = assets.rgbe_decode(enc)
    assert np.allclose(dec[0, 2], [1.0, 0.5, 0.25])
    assert dec[0, 3, 0] == pytest.approx(65504.0, rel=1 / 128)


def test_reference_meshes_load_in_assimp_order():
    e = Engine()
    sphere = R._mesh(e, "uvsphere")
    cube = R._mesh(e, "cube")
    plane = R._mesh(e, "plane")
    assert (sphere.name, sphere.num_triangles) == ("defaultobject", 19800)
    assert (cube.name, cube.num_triangles) == ("Cube", 12)
    assert (plane.name, plane.num_triangles) == ("Plane", 2)
    # one vertex per face corner
    assert len(sphere.vertices) == 3 * 19800
    n = sphere.vertices["normal"].astype(np.float64)
    t = sphere.vertices["tangent"].astype(np.float64)
    assert np.allclose(np.linalg.norm(n, axis=1), 1.0, atol=1e-5)
    assert np.allclose(np.linalg.norm(t, axis=1), 1.0, atol=1e-4)
    assert np.abs((n * t).sum(1)).max() < 1e-3


def test_cornell_scene_shape():
    e, info = scenes.cornell_box(1)
    fs = e.scene.build()
    tris = sum(fs.meshes[int(i.mesh_index)].num_triangles for i in fs.instances if i.flags & 1)
    assert tris == 10 + 24 + 2  # walls, two boxes, light quad
    assert fs.num_lights == 1 and fs.lights[0].info[3] == 2
    assert (info.width, info.height, info.samples, info.depth) == (256, 256, 64, 8)


def test_medium_scene_shape():
    e, info = scenes.cornell_medium(1, freq=6, spheres=2)
    fs = e.scene.build()
    # the invisible boundary cube is transparent with the medium behind its faces
    boundary = [i for i in fs.instances if i.id[2] >= 0]
    assert len(boundary) == 1 and boundary[0].flags == 1
    assert (info.width, info.height, info.samples, info.depth) == (1920, 1080, 256, 12)
    full = scenes.icosphere(79)
    assert full[1].shape[0] == 20 * 79 * 79
