"""Model import (vviewer_gb300.model3d): glTF 2.0 files as assimp 5.2.5 hands
them to vengine (AssimpLoadModel.cpp), vengine's node tree
(VulkanModel3D.cpp:49-75) and placement (SceneUtils.cpp:76-130), and scene
files that name glTF models and their EMBEDDED materials."""
import json
import struct
import zlib

import numpy as np
import pytest

from gltf_files import GltfBuilder, png_bytes, quad_arrays, textured_panel_model
from vviewer_gb300 import _native as N
from vviewer_gb300.model3d import add_model3d, decompose, import_model
from vviewer_gb300.renderer import write_png
from vviewer_gb300.scene import TEX_WHITE_COLOR, Engine, Transform, quat_to_mat3
from vviewer_gb300.scene_io import decode_png, import_scene


def _quad_file(tmp_path, container="gltf", tangent=None, name="Quad"):
    b = GltfBuilder()
    pos, nrm, uv, idx = quad_arrays(2.0)
    attrs = {"POSITION": b.accessor(pos), "NORMAL": b.accessor(nrm), "TEXCOORD_0": b.accessor(uv)}
    if tangent is not None:
        attrs["TANGENT"] = b.accessor(np.tile(np.asarray(tangent, dtype=np.float32), (4, 1)))
    m = b.mesh([{"attributes": attrs, "indices": b.accessor(idx)}], name=name)
    b.scene([b.node(name="QuadNode", mesh=m)])
    return b.save(tmp_path / f"quad.{'glb' if container == 'glb' else 'gltf'}", container)


def test_indexed_quad_vertices(tmp_path):
    e = Engine()
    model = import_model(e, _quad_file(tmp_path), name="quad")
    mesh = model.mesh("Quad")
    v = mesh.vertices
    pos, _, uv, idx = quad_arrays(2.0)
    assert (v["position"] == pos).all()
    assert (mesh.indices.ravel() == idx).all() and mesh.indices.shape == (2, 3)
    assert np.allclose(v["normal"], [0, 0, 1])  # normalised
    # assimp flips v on import, FlipUVs flips it back, vengine flips it again
    assert (v["uv"][:, 0] == uv[:, 0]).all() and (v["uv"][:, 1] == 1 - uv[:, 1]).all()
    # CalcTangentSpace on the indexed mesh: dP/du is +x
    assert np.allclose(v["tangent"], [1, 0, 0], atol=1e-6)
    assert (v["color"] == 1).all()
    assert model.meshes() == [mesh] and e.meshes[-1] is mesh


def test_tangent_attribute_gives_tangent_and_signed_bitangent(tmp_path):
    e = Engine()
    mesh = import_model(e, _quad_file(tmp_path, tangent=[2, 0, 0, -1])).mesh("Quad")
    assert np.allclose(mesh.vertices["tangent"], [1, 0, 0])
    # bitangent = normalize(cross(N, T) * w)
    assert np.allclose(mesh.vertices["bitangent"], [0, -1, 0])


def test_containers_give_the_same_model(tmp_path):
    out = []
    for c in ("gltf", "datauri", "glb"):
        d = tmp_path / c
        d.mkdir()
        mesh = import_model(Engine(), _quad_file(d, c)).mesh("Quad")
        out.append((mesh.vertices.tobytes(), mesh.indices.tobytes()))
    assert out[0] == out[1] == out[2]


def test_model_is_imported_once_per_name(tmp_path):
    e = Engine()
    p = _quad_file(tmp_path)
    a = import_model(e, p, name="q")
    n = len(e.meshes)
    assert import_model(e, p, name="q") is a and len(e.meshes) == n


def test_strips_fans_and_accessor_layouts(tmp_path):
    b = GltfBuilder()
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0], [0, 2, 0]], dtype=np.float32)
    nrm = np.tile(np.array([0, 0, 1], dtype=np.float32), (5, 1))
    # interleaved POSITION + NORMAL (stride 24) and normalised uint16 texture coordinates
    inter = np.concatenate([pos, nrm], axis=1).astype(np.float32)
    view = b.view(inter.tobytes(), stride=24)
    pa = b.accessor(pos, view=view, offset=0)
    na = b.accessor(nrm, view=view, offset=12)
    uv16 = np.array([[0, 0], [65535, 0], [0, 32768], [65535, 32768], [0, 65535]], dtype=np.uint16)
    ta = b.accessor(uv16, normalized=True)
    ia = b.accessor(np.arange(5, dtype=np.uint8))
    attrs = {"POSITION": pa, "NORMAL": na, "TEXCOORD_0": ta}
    m = b.mesh([{"attributes": attrs, "indices": ia, "mode": 5},
                {"attributes": attrs, "indices": ia, "mode": 6},
                {"attributes": attrs, "indices": ia, "mode": 1}], name="Shapes")
    b.scene([b.node(mesh=m)])
    model = import_model(Engine(), b.save(tmp_path / "s.gltf"))
    strip, fan = model.mesh("Shapes-0"), model.mesh("Shapes-1")
    assert model.mesh("Shapes-2") is None  # lines are dropped
    assert strip.indices.tolist() == [[0, 1, 2], [2, 1, 3], [2, 3, 4]]
    assert fan.indices.tolist() == [[0, 1, 2], [0, 2, 3], [0, 3, 4]]
    assert (strip.vertices["position"] == pos).all()
    assert np.allclose(strip.vertices["uv"][:, 0], uv16[:, 0] / 65535.0)
    assert np.allclose(strip.vertices["uv"][:, 1], 1 - uv16[:, 1] / 65535.0)


def test_sparse_accessor_and_missing_normals(tmp_path):
    b = GltfBuilder()
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], dtype=np.float32)
    pa = b.accessor(pos)
    acc = b.doc["accessors"][pa]
    acc["sparse"] = {"count": 1,
                     "indices": {"bufferView": b.view(np.array([2], dtype=np.uint32).tobytes()), "componentType": 5125},
                     "values": {"bufferView": b.view(np.array([0, 3, 0], dtype=np.float32).tobytes())}}
    m = b.mesh([{"attributes": {"POSITION": pa}}], name="Tri")
    b.scene([b.node(mesh=m)])
    mesh = import_model(Engine(), b.save(tmp_path / "t.gltf")).mesh("Tri")
    assert mesh.vertices["position"].tolist() == [[0, 0, 0], [1, 0, 0], [0, 3, 0]]
    assert np.allclose(mesh.vertices["normal"], [0, 0, 1])  # flat face normal


def test_node_tree_is_flattened_and_placed_as_the_reference_does(tmp_path):
    b = GltfBuilder()
    pos, nrm, uv, idx = quad_arrays(1.0)
    m = b.mesh([{"attributes": {"POSITION": b.accessor(pos), "NORMAL": b.accessor(nrm)},
                 "indices": b.accessor(idx)}], name="Quad")
    s45 = float(np.sin(np.pi / 4))
    leaf = b.node(name="Leaf", mesh=m, translation=[0, 0, 5])
    mid_m = np.eye(4, dtype=np.float32)
    mid_m[:3, 3] = [10, 0, 0]
    mid = b.node(name="Mid", children=[leaf], matrix=mid_m.T.ravel().tolist())
    top = b.node(name="Top", children=[mid], translation=[1, 2, 3], rotation=[0, s45, 0, s45], scale=[2, 2, 2])
    b.scene([top])
    e = Engine()
    model = import_model(e, b.save(tmp_path / "h.gltf"), name="hier")
    assert model.root.name == "Top"
    assert [c.name for c in model.root.children] == ["Mid", "Leaf"]
    assert all(not c.children for c in model.root.children)
    add_model3d(e.scene, None, model)
    objs = e.scene.objects_flat()
    assert [o.name for o in objs] == ["Top", "hier"]
    holder, obj = objs
    # a primitive without a material gets the importer's default material,
    # named after the file (not the model)
    assert obj.parent is holder and obj.mesh is model.mesh("Quad") and obj.material is e.material("h:DefaultMaterial")
    top_m = np.eye(4)
    top_m[:3, :3] = quat_to_mat3((s45, 0, s45, 0)) * 2
    top_m[:3, 3] = [1, 2, 3]
    leaf_m = np.eye(4)
    leaf_m[:3, 3] = [0, 0, 5]
    # the intermediate node's transform is dropped (VulkanModel3D::importNode, sic)
    assert np.allclose(obj.model_matrix(), top_m @ leaf_m, atol=1e-5)
    # root transform and material overrides
    e.create_material(type(e.material("defaultMaterial")), "floorMat")
    add_model3d(e.scene, None, model, Transform((0, 1, 0)), "floorMat")
    holder2, obj2 = e.scene.objects_flat()[2:]
    assert np.allclose(holder2.model_matrix()[:3, 3], [0, 1, 0]) and obj2.material is e.material("floorMat")


def test_several_roots_get_a_root_node_and_share_meshes(tmp_path):
    b = GltfBuilder()
    pos, nrm, uv, idx = quad_arrays(1.0)
    m = b.mesh([{"attributes": {"POSITION": b.accessor(pos), "NORMAL": b.accessor(nrm)},
                 "indices": b.accessor(idx)}])
    n0 = b.node(mesh=m, translation=[1, 0, 0])
    n1 = b.node(mesh=m, translation=[2, 0, 0])
    b.scene([n0, n1])
    e = Engine()
    before = len(e.meshes)
    model = import_model(e, b.save(tmp_path / "r.gltf"), name="two")
    assert len(e.meshes) == before + 1  # one mesh per primitive, shared by both nodes
    assert model.root.name == "ROOT" and [c.name for c in model.root.children] == ["nodes[0]", "nodes[1]"]
    assert model.mesh("meshes[0]") is not None
    add_model3d(e.scene, None, model)
    objs = e.scene.objects_flat()
    assert [o.name for o in objs] == ["ROOT", "two", "two"]
    assert objs[1].mesh is objs[2].mesh
    assert np.allclose([o.model_matrix()[0, 3] for o in objs[1:]], [1, 2])


def test_decompose_matches_the_composed_transform():
    rng = np.random.default_rng(5)
    for _ in range(20):
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        t = Transform(rng.normal(size=3), rng.uniform(0.2, 3, size=3) * rng.choice([-1, 1]), q)
        m = t.model_matrix().astype(np.float64)
        d = decompose(m)
        assert np.allclose(d.model_matrix(), m, atol=1e-5)
        assert np.linalg.det(quat_to_mat3(d.rotation)) > 0


def test_materials_and_textures(tmp_path):
    b = GltfBuilder()
    rng = np.random.default_rng(2)
    img4 = rng.integers(0, 256, (6, 5, 4), dtype=np.uint8)
    img3 = rng.integers(0, 256, (4, 7, 3), dtype=np.uint8)
    t4 = b.image(png_bytes(img4, tmp_path))
    t3 = b.image(png_bytes(img3, tmp_path))
    write_png(tmp_path / "ext.png", img3)
    t_ext = b.image(b"", uri="ext.png")
    t_jpg = b.image(b"\xff\xd8\xff\xe0" + bytes(32))
    painted = b.material(name="Painted", pbrMetallicRoughness={
        "baseColorFactor": [0.5, 0.6, 0.7, 1.0], "metallicFactor": 0.25, "roughnessFactor": 0.75,
        "baseColorTexture": {"index": t4}, "metallicRoughnessTexture": {"index": t3}},
        occlusionTexture={"index": t3}, normalTexture={"index": t3}, emissiveTexture={"index": t_ext})
    glow = b.material(name="Glow", emissiveFactor=[1.0, 0.5, 0.25],
                      pbrMetallicRoughness={"baseColorTexture": {"index": t_ext}},
                      extensions={"KHR_materials_emissive_strength": {"emissiveStrength": 4.0}})
    unnamed = b.material(pbrMetallicRoughness={"baseColorTexture": {"index": t_jpg}})
    pos, nrm, uv, idx = quad_arrays(1.0)
    attrs = {"POSITION": b.accessor(pos), "NORMAL": b.accessor(nrm), "TEXCOORD_0": b.accessor(uv)}
    ia = b.accessor(idx)
    m = b.mesh([{"attributes": attrs, "indices": ia, "material": painted},
                {"attributes": attrs, "indices": ia, "material": glow},
                {"attributes": attrs, "indices": ia, "material": unnamed},
                {"attributes": attrs, "indices": ia}], name="Mixed")
    b.scene([b.node(mesh=m)])
    e = Engine()
    with pytest.warns(UserWarning, match="JPEG"):
        model = import_model(e, b.save(tmp_path / "mats.gltf"), name="mats")
    assert [x.name for x in model.materials] == ["mats:Painted", "mats:Glow", "mats:materials[2]",
                                                 "mats:DefaultMaterial"]
    p = e.material("mats:Painted")
    assert p.albedo == [0.5, 0.6, 0.7, 1.0] and p.metallic == 0.25 and p.roughness == 0.75 and p.ao == 1.0
    assert p.transparent  # four channels in the base colour image
    fmt, img = e.textures[p.albedo_texture]
    assert fmt == N.TEXTURE_RGBA8_SRGB and (img == img4).all()
    for tex, src, ch in ((p.alpha_texture, img4, 3), (p.roughness_texture, img3, 1),
                         (p.metallic_texture, img3, 2), (p.ao_texture, img3, 0)):
        fmt, img = e.textures[tex]
        assert fmt == N.TEXTURE_RGBA8_LINEAR
        assert (img[..., :3] == src[..., ch:ch + 1]).all() and (img[..., 3] == 255).all()
    fmt, img = e.textures[p.normal_texture]
    assert fmt == N.TEXTURE_RGBA8_LINEAR and (img[..., :3] == img3).all()
    # an emissive texture with a black factor makes the colour white, strength 1
    assert p.emissive == [1.0, 1.0, 1.0, 1.0] and (e.textures[p.emissive_texture][1][..., :3] == img3).all()
    g = e.material("mats:Glow")
    assert g.emissive == [1.0, 0.5, 0.25, 4.0] and not g.transparent  # three-channel base colour
    assert g.metallic == 1.0 and g.roughness == 1.0  # glTF defaults
    u = e.material("mats:materials[2]")
    assert u.albedo_texture == TEX_WHITE_COLOR  # the JPEG was not decoded
    d = e.material("mats:DefaultMaterial")
    assert d.albedo == [1.0, 1.0, 1.0, 1.0] and d.metallic == 1.0 and d.roughness == 1.0
    add_model3d(e.scene, None, model)
    assert [o.material.name for o in e.scene.objects_flat()] == ["mats:Painted", "mats:Glow", "mats:materials[2]",
                                                                "mats:DefaultMaterial"]


def test_scene_file_with_gltf_model_and_embedded_material(tmp_path):
    textured_panel_model(tmp_path, "glb")
    doc = {"camera": {"position": [0, 0, 3], "target": [0, 0, 0], "up": [0, 1, 0]},
           "models": [{"name": "panel", "filepath": "panel.glb"}],
           "materials": [{"name": "panel:Panel", "type": "EMBEDDED"}],
           "scene": [{"name": "board", "mesh": {"modelName": "panel", "submesh": "Panel"},
                      "material": {"name": "panel:Panel"},
                      "transform": {"position": [0, 0, -1]}}]}
    (tmp_path / "s.json").write_text(json.dumps(doc))
    e = import_scene(tmp_path / "s.json")
    so = e.scene.objects_flat()[0]
    assert so.mesh.name == "Panel" and so.material.name == "panel:Panel" and so.material.transparent
    fs = e.scene.build()
    assert any(i.mesh_index == so.mesh.index for i in fs.instances)


def test_bad_files_are_reported(tmp_path):
    (tmp_path / "v1.gltf").write_text(json.dumps({"asset": {"version": "1.0"}}))
    with pytest.raises(ValueError, match="version"):
        import_model(Engine(), tmp_path / "v1.gltf")
    with pytest.raises(ValueError, match="not supported"):
        import_model(Engine(), tmp_path / "model.fbx")
    b = GltfBuilder()
    pos, nrm, uv, _ = quad_arrays(1.0)
    m = b.mesh([{"attributes": {"POSITION": b.accessor(pos)},
                 "indices": b.accessor(np.array([0, 1, 9], dtype=np.uint16))}], name="Bad")
    b.scene([b.node(mesh=m)])
    with pytest.raises(ValueError, match="out of range"):
        import_model(Engine(), b.save(tmp_path / "bad.gltf"))
    b = GltfBuilder()
    a = b.accessor(pos)
    b.doc["accessors"][a]["count"] = 99  # runs past its buffer view
    b.scene([b.node(mesh=b.mesh([{"attributes": {"POSITION": a}}]))])
    with pytest.raises(ValueError, match="past"):
        import_model(Engine(), b.save(tmp_path / "short.gltf"))


def test_panel_model_renders_in_the_oracle(tmp_path):
    """End to end on the CPU: the textured glTF model placed in the Cornell
    room renders finite and lit, and the transparent panel's cut-outs show."""
    from oracle import oracle
    from vviewer_gb300 import scenes

    e, info = scenes.cornell_box(1, 32, 32, 8, 6, 4)
    model = import_model(e, textured_panel_model(tmp_path, "gltf"), name="panel")
    add_model3d(e.scene, None, model, Transform((0.5, 0.45, 0.45), (0.5, 0.5, 0.5)))
    fs = e.scene.build()
    img = oracle.render(fs, e.scene.scene_data(info.width, info.height), info)["radiance"][..., :3]
    assert np.isfinite(img).all() and img.mean() > 0.01


# ---------------------------------------------------------------- PNG filters

def _encode_filtered(img: np.ndarray, ft: int) -> bytes:
    """An RGBA PNG with every row written under filter type `ft`."""
    h, w, _ = img.shape
    bpp = 4
    rows = img.reshape(h, w * 4).astype(np.int64)
    raw = bytearray()
    prev = np.zeros(w * 4, dtype=np.int64)
    for y in range(h):
        cur = rows[y]
        out = np.zeros_like(cur)
        for i in range(w * 4):
            a = cur[i - bpp] if i >= bpp else 0
            bb = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            if ft == 1:
                p = a
            elif ft == 2:
                p = bb
            elif ft == 3:
                p = (a + bb) >> 1
            else:
                pa, pb, pc = abs(bb - c), abs(a - c), abs(a + bb - 2 * c)
                p = a if (pa <= pb and pa <= pc) else (bb if pb <= pc else c)
            out[i] = (cur[i] - p) & 0xFF
        raw += bytes([ft]) + bytes(out.astype(np.uint8))
        prev = cur

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0))
            + chunk(b"IDAT", zlib.compress(bytes(raw))) + chunk(b"IEND", b""))


@pytest.mark.parametrize("ft", [1, 2, 3, 4])
def test_png_row_filters(ft):
    img = np.random.default_rng(ft).integers(0, 256, (9, 11, 4), dtype=np.uint8)
    dec, channels = decode_png(_encode_filtered(img, ft))
    assert channels == 4 and (dec == img).all()


def _grey_png(path, img):
    """8-bit greyscale PNG (colour type 0)."""
    h, w = img.shape
    raw = b"".join(b"\x00" + img[y].astype(np.uint8).tobytes() for y in range(h))

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    path.write_bytes(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 0, 0, 0, 0)) +
                     chunk(b"IDAT", zlib.compress(raw)) + chunk(b"IEND", b""))


def _obj_with_mtl(tmp_path):
    """Two objects; 'Box' has faces before any usemtl, then under 'red', then
    under 'textured'; 'Panel' uses 'bumpy' and an undefined material."""
    rgba = np.zeros((4, 4, 4), dtype=np.uint8)
    rgba[..., 0] = 200
    rgba[..., 3] = np.arange(16, dtype=np.uint8).reshape(4, 4) * 16
    write_png(tmp_path / "albedo.png", rgba)
    write_png(tmp_path / "normal.png", np.full((2, 2, 3), 128, dtype=np.uint8))
    _grey_png(tmp_path / "height.png", np.full((2, 2), 77, dtype=np.uint8))
    (tmp_path / "mats.mtl").write_text(
        "# two-material library\n"
        "newmtl red\nKd 0.8 0.1 0.1\nKs 0.2 0.2 0.2\nNs 25\n"
        "newmtl textured\nKd 0 0 0\nKs 0 0 0\nNs 100\nmap_Kd albedo.png\n"
        "newmtl bumpy\nKd 0.5 0.5 0.5\nKs 0.5 0.25 0\nNs 50\nmap_Bump -bm 1.0 normal.png\n"
        "newmtl flat\nKd 0 0 0\nKs 0.3 0.2 0.1\nNs 10\nbump height.png\n")
    (tmp_path / "model.obj").write_text(
        "mtllib mats.mtl\n"
        "v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvt 0 0\nvt 1 0\nvt 1 1\nvt 0 1\nvn 0 0 1\n"
        "o Box\nf 1/1/1 2/2/1 3/3/1\nusemtl red\nf 1/1/1 3/3/1 4/4/1\nusemtl textured\nf 1/1/1 2/2/1 3/3/1 4/4/1\n"
        "o Panel\nusemtl bumpy\nf 1/1/1 2/2/1 3/3/1\nusemtl missing\nf 1/1/1 3/3/1 4/4/1\nusemtl flat\nf 2/2/1 3/3/1 4/4/1\n")
    return tmp_path / "model.obj"


def test_obj_mtl_materials_follow_the_reference(tmp_path):
    """assimpLoadMaterialsOBJ (AssimpLoadModel.cpp:252-363) over assimp's OBJ
    import: materials "<stem>:<name>" with the importer's default first,
    PBR values derived from Kd / Ks / Ns, textures from map_Kd and map_Bump,
    and one mesh per run of faces under one material."""
    e = Engine()
    model = import_model(e, _obj_with_mtl(tmp_path), name="m")
    names = [m.name for m in model.materials]
    assert names == ["model:DefaultMaterial", "model:red", "model:textured", "model:bumpy", "model:flat"]
    mats = {m.name.split(":")[1]: m for m in model.materials}
    f = np.float32
    d = mats["DefaultMaterial"]
    assert d.albedo == [0.6, 0.6, 0.6, 1.0] and d.metallic == 0.0 and d.roughness == 1.0
    r = mats["red"]
    assert np.allclose(r.albedo, [0.8, 0.1, 0.1, 1.0])
    assert r.metallic == float(f(1) - f(0.8) / (f(0.8) + f(0.2))) and r.roughness == float(f(1) - f(25) / f(100))
    assert r.albedo_texture == TEX_WHITE_COLOR
    t = mats["textured"]
    # a black Kd with a diffuse texture becomes white; four channels: alpha
    # texture and a transparent material
    assert t.albedo == [1.0, 1.0, 1.0, 1.0] and t.albedo_texture != TEX_WHITE_COLOR
    assert t.roughness == 0.0 and t.metallic == 0.0
    built = t.pack()
    assert built.metallic_roughness_ao[3] == 1.0  # transparent
    alpha = e.textures[built.textures2[3]][1]
    assert np.array_equal(alpha[..., 0], (np.arange(16).reshape(4, 4) * 16).astype(np.uint8))
    b = mats["bumpy"]
    assert b.normal_texture != mats["red"].normal_texture  # map_Bump with options before the file
    fl = mats["flat"]
    # black Kd, non-black Ks: albedo takes Ks; a one-channel map_Bump is not a normal map
    assert np.allclose(fl.albedo[:3], [0.3, 0.2, 0.1]) and fl.normal_texture == mats["red"].normal_texture
    assert fl.metallic == 1.0
    # meshes per run of faces under one material, nodes per object
    assert [n.name for n in model.root.children] == ["Box", "Panel"]
    box, panel = model.root.children
    assert [m.name for m in box.meshes] == ["Box", "Box-1", "Box-2"]
    assert [m.name.split(":")[1] for m in box.materials] == ["DefaultMaterial", "red", "textured"]
    assert [m.indices.shape[0] for m in box.meshes] == [1, 1, 2]
    assert [m.name.split(":")[1] for m in panel.materials] == ["bumpy", "DefaultMaterial", "flat"]
    # placed as the reference places a model: its meshes with their materials
    add_model3d(e.scene, None, model)
    fs = e.scene.build()
    used = sorted({int(i.material_index) for i in fs.instances})
    assert len(used) == 5


def test_obj_without_materials_keeps_one_mesh(tmp_path):
    p = tmp_path / "tri.obj"
    p.write_text("o Tri\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    model = import_model(Engine(), p, import_materials=False)
    assert list(model.meshes_by_name) == ["Tri"] and model.materials == []
    assert model.root.children[0].materials == [None]
