"""Model import (glTF 2.0, OBJ) and placement of a model's nodes in a scene.

Restates the reference's model path:
  * src/lib/vengine/core/io/AssimpLoadModel.cpp:51-143 (assimpLoadMesh),
    :145-172 (node transform and tree), :174-250 (texture data), :364-535
    (assimpLoadMaterialsGLTF), :557-613 (assimpLoadModel, assimp flags
    Triangulate | FlipUVs | CalcTangentSpace; materials named
    "<file stem>:<material name>");
  * src/lib/vengine/vulkan/resources/VulkanModel3D.cpp:49-75 (importNode) and
    src/lib/vengine/vulkan/resources/VulkanMaterials.cpp:154-238
    (createImportedMaterials), src/lib/vengine/vulkan/VulkanEngine.cpp:157-186
    (importModel: a model name already imported returns that model);
  * src/lib/vengine/core/SceneUtils.cpp:76-130 (addModel3D).

The glTF reader restates what assimp 5.2.5's glTF 2.0 importer (a third-party
dependency, not in the reference tree) hands to vengine:
  * one assimp mesh per primitive, named after the glTF mesh ("<name>-<p>"
    when the mesh has several primitives); triangle strips and fans are
    turned into triangles in assimp's order; points and lines are dropped
    (the renderer takes triangles only);
  * texture v flipped on import, flipped back by aiProcess_FlipUVs and
    flipped again by vengine: the vertex keeps 1 - v of the file;
  * a TANGENT attribute gives tangent = xyz and bitangent = cross(N, xyz) * w,
    both normalised by vengine; without one, CalcTangentSpace computes them
    on the indexed mesh (assets.calc_tangent_space with the face list);
  * node transforms from `matrix` or T * R * S, decomposed by
    glm::decompose into position, rotation and scale; one root node, or a
    "ROOT" node over several;
  * one material per glTF material plus a default material (base colour 1,
    metallic 1, roughness 1) at the end for primitives without one;
    occlusionTexture arrives as the lightmap slot (vengine's ao texture).

Where a detail is not observable through the reference's renderer or is a
file-level corner case, this module picks plainly: unnamed meshes and nodes
are called "meshes[i]" and "nodes[i]", unnamed materials "materials[i]", the
default material "DefaultMaterial". One Mesh is kept per glTF primitive and
shared by every node that uses it (the reference uploads a copy per node; the
rendered image is the same). Primitives without normals get flat face normals
(glTF's rule; assimp leaves them zero). Images are PNG or sequential JPEG
(embedded, data URI or file); an image that cannot be decoded (a progressive
JPEG, for one) leaves its slot untextured with a warning, as the reference
does when stb_image fails.
"""
from __future__ import annotations

import base64
import json
import struct
import urllib.parse
import warnings
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import _native as N
from .assets import calc_tangent_space
from .scene import VERTEX_DTYPE, Engine, Material, MaterialPBRStandard, Mesh, Scene, SceneObject, Transform

f32 = np.float32

_COMPONENT = {5120: np.int8, 5121: np.uint8, 5122: np.int16, 5123: np.uint16, 5125: np.uint32, 5126: np.float32}
_NCOMP = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4}
_NORM_DIV = {5120: 127.0, 5121: 255.0, 5122: 32767.0, 5123: 65535.0}
_MODE_TRIANGLES, _MODE_STRIP, _MODE_FAN = 4, 5, 6


@dataclass
class ModelNode:
    """Model3D::Model3DNode: a node's local transform, meshes and their materials."""
    name: str
    transform: Transform
    meshes: list = field(default_factory=list)
    materials: list = field(default_factory=list)  # Material or None, one per mesh
    children: list = field(default_factory=list)


@dataclass
class Model3D:
    """An imported model: its node tree (as vengine keeps it) and meshes by name."""
    name: str
    root: ModelNode
    meshes_by_name: dict = field(default_factory=dict)
    materials: list = field(default_factory=list)

    def mesh(self, name: str) -> Mesh | None:
        """Model3D::mesh: the mesh of that name, or None."""
        return self.meshes_by_name.get(name)

    def meshes(self) -> list:
        return list(self.meshes_by_name.values())


# ---------------------------------------------------------------- transforms

def decompose(m: np.ndarray) -> Transform:
    """glm::decompose of a 4x4 affine matrix (row-major here): translation,
    per-axis scale with shear removed by Gram-Schmidt over the columns, a
    negative determinant folded into the scale, and the rotation quaternion
    of the orthonormalised columns."""
    from .scene_io import quat_from_mat3

    m = np.asarray(m, dtype=np.float64)
    if m[3, 3] == 0:
        raise ValueError("node transform: m[3][3] is zero")
    m = m / m[3, 3]
    cols = [m[:3, i].copy() for i in range(3)]
    sx = np.linalg.norm(cols[0])
    cols[0] /= sx
    cols[1] -= cols[0] * (cols[0] @ cols[1])
    sy = np.linalg.norm(cols[1])
    cols[1] /= sy
    cols[2] -= cols[0] * (cols[0] @ cols[2])
    cols[2] -= cols[1] * (cols[1] @ cols[2])
    sz = np.linalg.norm(cols[2])
    cols[2] /= sz
    scale = np.array([sx, sy, sz])
    if cols[0] @ np.cross(cols[1], cols[2]) < 0:
        scale = -scale
        cols = [-c for c in cols]
    rot = quat_from_mat3(np.stack(cols, axis=1))
    return Transform(m[:3, 3].astype(f32), scale.astype(f32), rot)


def _copy_transform(t: Transform) -> Transform:
    return Transform(t.position.copy(), t.scale.copy(), t.rotation.copy())


def _quat_wxyz_to_mat3(q) -> np.ndarray:
    w, x, y, z = (float(v) for v in q)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def _node_matrix(node: dict) -> np.ndarray:
    """A node's local matrix (row-major) in float32, as assimp builds it."""
    if "matrix" in node:
        m = np.asarray(node["matrix"], dtype=f32).reshape(4, 4).T  # glTF stores columns
        return m.astype(np.float64)
    m = np.eye(4)
    if "translation" in node:
        m[:3, 3] = np.asarray(node["translation"], dtype=f32)
    if "rotation" in node:
        x, y, z, w = (float(v) for v in node["rotation"])
        m[:3, :3] = m[:3, :3] @ _quat_wxyz_to_mat3((w, x, y, z))
    if "scale" in node:
        m[:3, :3] = m[:3, :3] * np.asarray(node["scale"], dtype=f32)[None, :]
    return m.astype(f32).astype(np.float64)


# ---------------------------------------------------------------- glTF container

class _GltfFile:
    """The JSON document and binary buffers of a .gltf or .glb file."""

    def __init__(self, path: Path):
        self.path = path
        self.folder = path.parent
        data = path.read_bytes()
        bin_chunk = None
        if data[:4] == b"glTF":
            if len(data) < 12:
                raise ValueError(f"{path}: truncated GLB header")
            _, version, length = struct.unpack_from("<III", data, 0)
            if version != 2:
                raise ValueError(f"{path}: GLB version {version} is not supported")
            length = min(length, len(data))
            pos, doc = 12, None
            while pos + 8 <= length:
                clen, ctype = struct.unpack_from("<II", data, pos)
                body = data[pos + 8:pos + 8 + clen]
                if len(body) != clen:
                    raise ValueError(f"{path}: truncated GLB chunk")
                if ctype == 0x4E4F534A and doc is None:  # "JSON"
                    doc = json.loads(body.decode("utf-8"))
                elif ctype == 0x004E4942 and bin_chunk is None:  # "BIN\0"
                    bin_chunk = body
                pos += 8 + clen
            if doc is None:
                raise ValueError(f"{path}: GLB without a JSON chunk")
        else:
            doc = json.loads(data.decode("utf-8"))
        version = str(doc.get("asset", {}).get("version", ""))
        if not version.startswith("2"):
            raise ValueError(f"{path}: glTF version {version!r} is not supported (2.x only)")
        self.doc = doc
        self.buffers = []
        for i, b in enumerate(doc.get("buffers", [])):
            uri = b.get("uri")
            if uri is None:
                if bin_chunk is None:
                    raise ValueError(f"{path}: buffer {i} has no uri and the file has no BIN chunk")
                raw = bin_chunk
            else:
                raw = self._read_uri(uri)
            if len(raw) < int(b["byteLength"]):
                raise ValueError(f"{path}: buffer {i} holds {len(raw)} bytes, byteLength {b['byteLength']}")
            self.buffers.append(raw)

    def _read_uri(self, uri: str) -> bytes:
        if uri.startswith("data:"):
            head, _, payload = uri.partition(",")
            if not head.endswith(";base64"):
                raise ValueError(f"{self.path}: data URI without base64 encoding")
            return base64.b64decode(payload)
        return (self.folder / urllib.parse.unquote(uri)).read_bytes()

    def buffer_view(self, i: int) -> bytes:
        bv = self.doc["bufferViews"][i]
        buf = self.buffers[bv["buffer"]]
        off = int(bv.get("byteOffset", 0))
        n = int(bv["byteLength"])
        if off + n > len(buf):
            raise ValueError(f"{self.path}: bufferView {i} runs past its buffer")
        return buf[off:off + n]

    def _typed(self, view: int, offset: int, comp: int, nc: int, count: int, stride: int = 0) -> np.ndarray:
        dt = np.dtype(_COMPONENT[comp]).newbyteorder("<")
        elem = dt.itemsize * nc
        stride = stride or elem
        raw = self.buffer_view(view)
        if count and offset + stride * (count - 1) + elem > len(raw):
            raise ValueError(f"{self.path}: accessor data runs past bufferView {view}")
        if count == 0:
            return np.zeros((0, nc), dtype=dt)
        return np.ndarray((count, nc), dtype=dt, buffer=raw, offset=offset, strides=(stride, dt.itemsize)).copy()

    def accessor(self, i: int) -> np.ndarray:
        """Accessor i as a (count, components) array: floats for float or
        normalised data, integers otherwise; sparse substitutions applied."""
        a = self.doc["accessors"][i]
        comp = int(a["componentType"])
        if comp not in _COMPONENT:
            raise ValueError(f"{self.path}: accessor {i}: component type {comp}")
        if a["type"] not in _NCOMP:
            raise ValueError(f"{self.path}: accessor {i}: type {a['type']} is not a vertex attribute type")
        nc = _NCOMP[a["type"]]
        count = int(a["count"])
        if "bufferView" in a:
            bv = self.doc["bufferViews"][a["bufferView"]]
            arr = self._typed(a["bufferView"], int(a.get("byteOffset", 0)), comp, nc, count,
                              int(bv.get("byteStride", 0)))
        else:
            arr = np.zeros((count, nc), dtype=_COMPONENT[comp])
        sp = a.get("sparse")
        if sp:
            n = int(sp["count"])
            ix = sp["indices"]
            idx = self._typed(ix["bufferView"], int(ix.get("byteOffset", 0)), int(ix["componentType"]), 1, n)
            vals = self._typed(sp["values"]["bufferView"], int(sp["values"].get("byteOffset", 0)), comp, nc, n)
            idx = idx.ravel().astype(np.int64)
            if n and (idx.max() >= count):
                raise ValueError(f"{self.path}: accessor {i}: sparse index out of range")
            arr[idx] = vals
        if comp != 5126 and a.get("normalized", False):
            arr = np.maximum(arr.astype(np.float64) / _NORM_DIV[comp], -1.0).astype(f32)
        return arr


# ---------------------------------------------------------------- PNG images

def _decode_image(data: bytes, what: str):
    """(H x W x 4 uint8, channels in the file as stb_image counts them) of a
    PNG or sequential JPEG, or None with a warning when the image cannot be
    decoded (the slot stays untextured, as when stb_image fails)."""
    from .jpeg import decode_jpeg
    from .scene_io import decode_png

    if data[:2] == b"\xff\xd8":
        try:
            return decode_jpeg(data, what)
        except ValueError as e:
            warnings.warn(f"{what}: JPEG not decoded ({e}); the slot stays untextured")
            return None
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        warnings.warn(f"{what}: unknown image format; the slot stays untextured")
        return None
    return decode_png(data, what)


def _channel_texture(rgba: np.ndarray, channel: int) -> np.ndarray:
    """A one-channel image (assimpCreateImage with a channel) as RGBA8 with the
    channel in red, green and blue: the shaders read `.r`."""
    out = np.empty_like(rgba)
    out[..., 0] = out[..., 1] = out[..., 2] = rgba[..., channel]
    out[..., 3] = 255
    return out


# ---------------------------------------------------------------- glTF meshes

def _faces(indices: np.ndarray, mode: int) -> np.ndarray:
    """Triangles (F x 3) of a primitive's index list in assimp's order."""
    n = indices.size
    if mode == _MODE_TRIANGLES:
        return indices[:n - n % 3].reshape(-1, 3)
    if n < 3:
        return np.zeros((0, 3), dtype=np.int64)
    i = np.arange(n - 2)
    if mode == _MODE_STRIP:
        odd = (i + 1) % 2 == 0  # triangles 1, 3, ...: (i + 1, i, i + 2)
        a = np.where(odd, indices[i + 1], indices[i])
        b = np.where(odd, indices[i], indices[i + 1])
        return np.stack([a, b, indices[i + 2]], axis=1)
    # fan: (0, i + 1, i + 2)
    return np.stack([np.full(n - 2, indices[0]), indices[i + 1], indices[i + 2]], axis=1)


def _primitive_mesh(g: _GltfFile, name: str, prim: dict) -> Mesh | None:
    """assimpLoadMesh over what assimp makes of one glTF primitive."""
    attrs = prim.get("attributes", {})
    mode = int(prim.get("mode", _MODE_TRIANGLES))
    if mode not in (_MODE_TRIANGLES, _MODE_STRIP, _MODE_FAN) or "POSITION" not in attrs:
        return None
    pos = g.accessor(attrs["POSITION"]).astype(f32)[:, :3]
    nv = pos.shape[0]

    def attr(key, ncomp):
        if key not in attrs:
            return None
        a = g.accessor(attrs[key])
        if a.shape[0] != nv:  # assimp skips a stream whose size does not match
            return None
        return a.astype(f32)[:, :ncomp]

    nrm = attr("NORMAL", 3)
    uv = attr("TEXCOORD_0", 2)
    tan = attr("TANGENT", 4)
    idx = (g.accessor(prim["indices"]).ravel().astype(np.int64) if "indices" in prim
           else np.arange(nv, dtype=np.int64))
    if idx.size and (idx.min() < 0 or idx.max() >= nv):
        raise ValueError(f"{g.path}: mesh {name}: index out of range")
    faces = _faces(idx, mode)
    if faces.shape[0] == 0:
        return None
    if nrm is None:
        # flat face normals over one vertex per face corner
        corners = faces.ravel()
        pos = pos[corners]
        uv = uv[corners] if uv is not None else None
        tan = None
        p = pos.reshape(-1, 3, 3).astype(np.float64)
        fn = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
        fn /= np.maximum(np.linalg.norm(fn, axis=1, keepdims=True), 1e-30)
        nrm = np.repeat(fn, 3, axis=0).astype(f32)
        faces = np.arange(corners.size, dtype=np.int64).reshape(-1, 3)
        nv = pos.shape[0]
    raw_nrm = nrm
    lens = np.sqrt((nrm.astype(np.float64) ** 2).sum(axis=1))
    nrm = (nrm / np.where(lens > 0, lens, 1.0)[:, None]).astype(f32)
    uv_out = np.zeros((nv, 2), dtype=f32)
    if uv is not None:
        uv_out[:, 0] = uv[:, 0]
        uv_out[:, 1] = f32(1.0) - uv[:, 1]
    if tan is not None:
        t3 = tan[:, :3]
        bt = (np.cross(raw_nrm, t3) * tan[:, 3:4]).astype(f32)

        def _norm(a):
            ln = np.sqrt((a.astype(np.float64) ** 2).sum(axis=1))
            return (a / np.where(ln > 0, ln, 1.0)[:, None]).astype(f32)

        tangent, bitangent = _norm(t3), _norm(bt)
    else:
        tangent, bitangent = calc_tangent_space(pos, uv_out, nrm, faces=faces)
    verts = np.zeros(nv, dtype=VERTEX_DTYPE)
    verts["position"] = pos
    verts["uv"] = uv_out
    verts["normal"] = nrm
    verts["color"] = 1.0
    verts["tangent"] = tangent
    verts["bitangent"] = bitangent
    return Mesh(name=name, vertices=verts, indices=faces.astype(np.uint32))


# ---------------------------------------------------------------- glTF materials

def _gltf_materials(engine: Engine, g: _GltfFile, stem: str) -> list[Material]:
    """assimpLoadMaterialsGLTF + createImportedMaterials: one PBR material per
    glTF material and the importer's default material last."""
    doc = g.doc
    images: dict[int, object] = {}
    textures: dict[tuple, int] = {}

    def image(tex_index: int):
        src = doc["textures"][tex_index].get("source")
        if src is None:
            return None
        if src not in images:
            im = doc["images"][src]
            what = f"{g.path.name}: image {im.get('name', src)}"
            if "bufferView" in im:
                data = g.buffer_view(im["bufferView"])
            elif "uri" in im:
                try:
                    data = g._read_uri(im["uri"])
                except OSError as e:
                    warnings.warn(f"{what}: {e}; the slot stays untextured")
                    data = None
            else:
                data = None
            images[src] = _decode_image(data, what) if data is not None else None
        return images[src]

    def texture(ref: dict | None, fmt: int, channel: int = -1, need_channels: int = 0):
        """Engine texture index of a material's texture reference (or None)."""
        if not ref or "index" not in ref:
            return None
        dec = image(int(ref["index"]))
        if dec is None:
            return None
        rgba, channels = dec
        if need_channels and channels != need_channels:
            return None
        key = (int(ref["index"]), fmt, channel)
        if key not in textures:
            textures[key] = engine.add_texture(fmt, rgba if channel < 0 else _channel_texture(rgba, channel))
        return textures[key]

    out = []
    mats = list(enumerate(doc.get("materials", []))) + [(None, {"name": "DefaultMaterial"})]
    for i, m in mats:
        name = m.get("name") or f"materials[{i}]"
        mat = engine.create_material(MaterialPBRStandard, f"{stem}:{name}")
        pbr = m.get("pbrMetallicRoughness", {})
        mat.albedo = [float(v) for v in pbr.get("baseColorFactor", [1.0, 1.0, 1.0, 1.0])]
        mat.roughness = float(pbr.get("roughnessFactor", 1.0))
        mat.metallic = float(pbr.get("metallicFactor", 1.0))
        mat.ao = 1.0
        t = texture(pbr.get("baseColorTexture"), N.TEXTURE_RGBA8_SRGB)
        if t is not None:
            mat.albedo_texture = t
        t = texture(pbr.get("baseColorTexture"), N.TEXTURE_RGBA8_LINEAR, 3, need_channels=4)
        if t is not None:  # a four-channel base colour image: transparent (AssimpLoadModel.cpp:408-421)
            mat.alpha_texture = t
            mat.set_transparent(True)
        mr = pbr.get("metallicRoughnessTexture")
        t = texture(mr, N.TEXTURE_RGBA8_LINEAR, 1)
        if t is not None:
            mat.roughness_texture = t
        t = texture(mr, N.TEXTURE_RGBA8_LINEAR, 2)
        if t is not None:
            mat.metallic_texture = t
        t = texture(m.get("occlusionTexture"), N.TEXTURE_RGBA8_LINEAR, 0)
        if t is not None:
            mat.ao_texture = t
        color = [float(v) for v in m.get("emissiveFactor", [0.0, 0.0, 0.0])]
        strength = float(m.get("extensions", {}).get("KHR_materials_emissive_strength", {})
                         .get("emissiveStrength", 1.0))
        t = texture(m.get("emissiveTexture"), N.TEXTURE_RGBA8_SRGB)
        if t is not None:
            mat.emissive_texture = t
            if max(color) == 0.0 and min(color) == 0.0:
                color = [1.0, 1.0, 1.0]
            if strength == 0.0:
                strength = 1.0
        mat.emissive = [*color, strength]
        t = texture(m.get("normalTexture"), N.TEXTURE_RGBA8_LINEAR)
        if t is not None:
            mat.normal_texture = t
        out.append(mat)
    return out


# ---------------------------------------------------------------- import

def _flatten(root: ModelNode) -> ModelNode:
    """VulkanModel3D::importNode appends every child, at any depth, to the
    root's list (it recurses into `m_nodeTree.add()`, sic): the model tree is
    the root over all other nodes in depth-first pre-order, each keeping
    only its own local transform."""
    flat: list[ModelNode] = []

    def visit(n: ModelNode):
        for c in n.children:
            flat.append(ModelNode(c.name, c.transform, c.meshes, c.materials, []))
            visit(c)

    visit(root)
    return ModelNode(root.name, root.transform, root.meshes, root.materials, flat)


def _load_gltf(engine: Engine, path: Path, name: str, import_materials: bool) -> Model3D:
    g = _GltfFile(path)
    doc = g.doc
    stem = path.stem
    materials = _gltf_materials(engine, g, stem) if import_materials else []
    default_index = len(doc.get("materials", []))
    prim_meshes: dict[tuple, Mesh | None] = {}
    by_name: dict[str, Mesh] = {}

    def mesh_prims(mi: int):
        gm = doc["meshes"][mi]
        base = gm.get("name") or f"meshes[{mi}]"
        prims = gm.get("primitives", [])
        out = []
        for p, prim in enumerate(prims):
            key = (mi, p)
            if key not in prim_meshes:
                nm = base if len(prims) == 1 else f"{base}-{p}"
                mesh = _primitive_mesh(g, nm, prim)
                if mesh is not None:
                    engine.add_mesh(mesh)
                    by_name[nm] = mesh
                prim_meshes[key] = mesh
            mesh = prim_meshes[key]
            if mesh is not None:
                mat_i = int(prim.get("material", default_index))
                out.append((mesh, materials[mat_i] if materials else None))
        return out

    nodes = doc.get("nodes", [])

    def build(ni: int, depth: int) -> ModelNode:
        if depth > len(nodes):
            raise ValueError(f"{path}: node hierarchy has a cycle")
        nd = nodes[ni]
        node = ModelNode(nd.get("name") or f"nodes[{ni}]", decompose(_node_matrix(nd)))
        if "mesh" in nd:
            for mesh, mat in mesh_prims(int(nd["mesh"])):
                node.meshes.append(mesh)
                node.materials.append(mat)
        node.children = [build(int(c), depth + 1) for c in nd.get("children", [])]
        return node

    scenes = doc.get("scenes", [])
    roots = scenes[int(doc.get("scene", 0))].get("nodes", []) if scenes else []
    if len(roots) == 1:
        root = build(int(roots[0]), 0)
    else:
        root = ModelNode("ROOT", Transform())
        root.children = [build(int(r), 1) for r in roots]
    return Model3D(name, _flatten(root), by_name, materials)


# ---------------------------------------------------------------- OBJ with .mtl materials

def _obj_groups(text: str):
    """Parses an OBJ file into (V, VT, VN, mtllib files, groups). A group is a
    run of faces of one object ('o') under one material ('usemtl'): the
    importer (assimp 5.2.5's OBJ loader) starts a new mesh at each change of
    either. Each group: (object name, material name or None, faces as corner
    lists of 1-based (v, vt, vn) indices)."""
    v, vt, vn = [], [], []
    libs, groups = [], []
    obj, mtl = "defaultobject", None
    for line in text.splitlines():
        parts = line.split()
        if not parts or parts[0].startswith("#"):
            continue
        tag = parts[0]
        if tag == "v":
            v.append([float(x) for x in parts[1:4]])
        elif tag == "vt":
            vt.append([float(x) for x in parts[1:3]])
        elif tag == "vn":
            vn.append([float(x) for x in parts[1:4]])
        elif tag == "o" and len(parts) > 1:
            obj = parts[1]
        elif tag == "usemtl" and len(parts) > 1:
            mtl = " ".join(parts[1:])
        elif tag == "mtllib" and len(parts) > 1:
            libs.append(" ".join(parts[1:]))
        elif tag == "f":
            corners = []
            for c in parts[1:]:
                idx = c.split("/")
                corners.append((int(idx[0]), int(idx[1]) if len(idx) > 1 and idx[1] else 0,
                                int(idx[2]) if len(idx) > 2 and idx[2] else 0))
            if not groups or groups[-1][0] != obj or groups[-1][1] != mtl:
                groups.append((obj, mtl, []))
            groups[-1][2].append(corners)
    return (np.array(v, dtype=f32).reshape(-1, 3), np.array(vt, dtype=f32).reshape(-1, 2),
            np.array(vn, dtype=f32).reshape(-1, 3), libs, groups)


def _mtl_materials(text: str) -> list[dict]:
    """.mtl entries as assimp's OBJ material importer reads them: Kd (default
    0.6 grey), Ks (default black), Ns (default 0), map_Kd, and map_Bump /
    bump as the height texture (texture options before the file name are
    skipped: the file is the last token)."""
    out = []
    cur = None
    for line in text.splitlines():
        parts = line.split()
        if not parts or parts[0].startswith("#"):
            continue
        tag = parts[0]
        if tag == "newmtl":
            cur = {"name": " ".join(parts[1:]), "Kd": [0.6, 0.6, 0.6], "Ks": [0.0, 0.0, 0.0], "Ns": 0.0}
            out.append(cur)
        elif cur is None:
            continue
        elif tag in ("Kd", "Ks") and len(parts) > 1:
            vals = [float(x) for x in parts[1:4]]
            cur[tag] = vals if len(vals) == 3 else [vals[0]] * 3
        elif tag == "Ns" and len(parts) > 1:
            cur["Ns"] = float(parts[1])
        elif tag == "map_Kd" and len(parts) > 1:
            cur["map_Kd"] = parts[-1]
        elif tag in ("map_Bump", "map_bump", "bump") and len(parts) > 1:
            cur["map_Bump"] = parts[-1]
    return out


def _obj_material(engine: Engine, folder: Path, stem: str, m: dict, cache: dict) -> Material:
    """assimpLoadMaterialsOBJ (AssimpLoadModel.cpp:252-363) for one .mtl entry:
    a PBR material "<file stem>:<name>" with albedo Kd; a map_Kd image gives
    the albedo texture (sRGB; a black Kd becomes white) and, with four
    channels, an alpha texture from its alpha channel and a transparent
    material; metallic = 1 - max(Kd) / (max(Kd) + max(Ks)); roughness =
    1 - Ns / 100; a black Kd with a non-black Ks takes Ks as albedo; a
    map_Bump image that is not one-channel is the normal map (linear)."""
    mat = engine.create_material(MaterialPBRStandard, f"{stem}:{m['name']}")
    albedo = [float(c) for c in m["Kd"]] + [1.0]

    def image(file: str):
        if file not in cache:
            fp = folder / file
            try:
                data = fp.read_bytes()
            except OSError as e:
                warnings.warn(f"{fp}: {e}; the slot stays untextured")
                data = None
            cache[file] = _decode_image(data, str(fp)) if data is not None else None
        return cache[file]

    if "map_Kd" in m:
        dec = image(m["map_Kd"])
        if dec is not None:
            rgba, channels = dec
            mat.albedo_texture = engine.add_texture(N.TEXTURE_RGBA8_SRGB, rgba)
            if max(albedo[:3]) == 0.0 and min(albedo[:3]) == 0.0:
                albedo[:3] = [1.0, 1.0, 1.0]
            if channels == 4:
                mat.alpha_texture = engine.add_texture(N.TEXTURE_RGBA8_LINEAR, _channel_texture(rgba, 3))
                if albedo[3] == 0.0:
                    albedo[3] = 1.0
                mat.set_transparent(True)
    ks = [float(c) for c in m["Ks"]]
    diffuse_amount = f32(max(albedo[:3]))
    specular_amount = f32(max(ks))
    with np.errstate(invalid="ignore", divide="ignore"):
        mat.metallic = float(f32(1.0) - diffuse_amount / (diffuse_amount + specular_amount))
    mat.roughness = float(f32(1.0) - f32(m["Ns"]) / f32(100.0))
    if max(albedo[:3]) == 0.0 and min(albedo[:3]) == 0.0 and specular_amount != 0.0:
        albedo[:3] = ks
    mat.albedo = albedo
    mat.ao = 1.0
    if "map_Bump" in m:
        dec = image(m["map_Bump"])
        if dec is not None and dec[1] != 1:
            mat.normal_texture = engine.add_texture(N.TEXTURE_RGBA8_LINEAR, dec[0])
    return mat


def _load_obj_model(engine: Engine, path: Path, name: str, import_materials: bool = True) -> Model3D:
    """An OBJ model as assimp hands it to vengine: a root node named after the
    file over one node per object, whose meshes are the object's runs of
    faces under one material. The first mesh of an object takes the object's
    name, later ones "<object>-<k>" (k = 1, 2, ...). With import_materials the
    materials come from the .mtl files the OBJ names (mtllib), in the
    importer's order: its default material "DefaultMaterial" (grey 0.6) first,
    then the files' entries; faces before any usemtl, or naming a material no
    file defines, use the default one."""
    from .assets import mesh_from_obj_arrays

    V, VT, VN, libs, groups = _obj_groups(path.read_text())
    stem = path.stem
    by_name: dict = {}
    mats: dict = {}
    materials: list = []
    if import_materials:
        entries = [{"name": "DefaultMaterial", "Kd": [0.6, 0.6, 0.6], "Ks": [0.0, 0.0, 0.0], "Ns": 0.0}]
        for lib in libs:
            fp = path.parent / lib
            try:
                entries += _mtl_materials(fp.read_text())
            except OSError as e:
                warnings.warn(f"{fp}: {e}; its materials are not loaded")
        cache: dict = {}
        for m in entries:
            if m["name"] not in mats:
                mats[m["name"]] = _obj_material(engine, path.parent, stem, m, cache)
                materials.append(mats[m["name"]])
    nodes: dict = {}
    counts: dict = {}
    for obj, mtl, faces in groups:
        tris = [(f[0], f[k], f[k + 1]) for f in faces for k in range(1, len(f) - 1)]
        corners = np.zeros((len(tris), 3, 3), dtype=np.int64)
        for t, tri in enumerate(tris):
            for c in range(3):
                vi, ti, ni = tri[c]
                corners[t, c] = (_obj_index(vi, len(V)) + 1, (_obj_index(ti, len(VT)) + 1) if ti else 0,
                                 (_obj_index(ni, len(VN)) + 1) if ni else 0)
        k = counts.get(obj, 0)
        counts[obj] = k + 1
        mesh_name = obj if k == 0 else f"{obj}-{k}"
        mesh = engine.add_mesh(mesh_from_obj_arrays(mesh_name, V, VT, VN, corners.reshape(-1, 3)))
        by_name[mesh_name] = mesh
        if obj not in nodes:
            nodes[obj] = ModelNode(obj, Transform(), [], [])
        nodes[obj].meshes.append(mesh)
        nodes[obj].materials.append(mats.get(mtl, mats.get("DefaultMaterial")) if import_materials else None)
    return Model3D(name, ModelNode(path.name, Transform(), [], [], list(nodes.values())), by_name, materials)


def _obj_index(i: int, n: int) -> int:
    return i - 1 if i > 0 else n + i


def import_model(engine: Engine, path: str | Path, name: str | None = None,
                 import_materials: bool = True) -> Model3D:
    """VulkanEngine::importModel: loads a .gltf, .glb or .obj file into the
    engine (meshes, and for glTF its materials and textures) once per model
    name; returns the model."""
    path = Path(path)
    name = name if name is not None else str(path)
    models = engine.models
    if name in models:
        return models[name]
    ext = path.suffix.lower()
    if ext in (".gltf", ".glb"):
        model = _load_gltf(engine, path, name, import_materials)
    elif ext == ".obj":
        model = _load_obj_model(engine, path, name, import_materials)
    else:
        raise ValueError(f"{path}: model format {ext or '(none)'} is not supported (glTF, GLB, OBJ)")
    models[name] = model
    return model


def add_model3d(scene: Scene, parent: SceneObject | None, model: Model3D,
                override_root_transform: Transform | None = None,
                override_material: str | None = None) -> None:
    """addModel3D: one scene object per mesh of a node (named after the model,
    placed under the node's parent with the node's transform); a node with
    children adds an object of its own name, with its transform, that holds
    them. The root's transform can be overridden, and so can every mesh's
    material; meshes without one get "defaultMaterial"."""
    engine = scene.engine
    default_mat = engine._materials_by_name.get("defaultMaterial")
    override = engine.material(override_material) if override_material is not None else None

    def add(node: ModelNode, parent: SceneObject | None, is_root: bool):
        t = override_root_transform if (is_root and override_root_transform is not None) else node.transform
        for mesh, mat in zip(node.meshes, node.materials):
            so = scene.add_scene_object(model.name, _copy_transform(t), parent)
            so.mesh = mesh
            so.material = override or mat or default_mat
        if node.children:
            holder = scene.add_scene_object(node.name, _copy_transform(t), parent)
            for c in node.children:
                add(c, holder, False)

    add(model.root, parent, True)
