"""Writes small glTF 2.0 files for the model import tests: a builder over one
binary buffer, saved as .gltf with a .bin file, as .gltf with a base64 data
URI, or as a .glb container. Also the textured model used by the render
parity tests."""
from __future__ import annotations

import base64
import json
import struct
from pathlib import Path

import numpy as np

from vviewer_gb300.renderer import write_png

_COMP = {np.dtype(np.int8): 5120, np.dtype(np.uint8): 5121, np.dtype(np.int16): 5122,
         np.dtype(np.uint16): 5123, np.dtype(np.uint32): 5125, np.dtype(np.float32): 5126}
_TYPE = {1: "SCALAR", 2: "VEC2", 3: "VEC3", 4: "VEC4"}


def png_bytes(rgba: np.ndarray, tmp: Path) -> bytes:
    p = tmp / "_img.png"
    write_png(p, rgba)
    data = p.read_bytes()
    p.unlink()
    return data


class GltfBuilder:
    def __init__(self):
        self.bin = bytearray()
        self.doc = {"asset": {"version": "2.0"}, "buffers": [], "bufferViews": [], "accessors": [],
                    "meshes": [], "nodes": [], "scenes": [], "materials": [], "images": [], "textures": []}

    def view(self, data: bytes, stride: int | None = None) -> int:
        while len(self.bin) % 4:
            self.bin.append(0)
        bv = {"buffer": 0, "byteOffset": len(self.bin), "byteLength": len(data)}
        if stride:
            bv["byteStride"] = stride
        self.bin += data
        self.doc["bufferViews"].append(bv)
        return len(self.doc["bufferViews"]) - 1

    def accessor(self, arr, normalized: bool = False, view: int | None = None, offset: int = 0,
                 count: int | None = None, ncomp: int | None = None, dtype=None) -> int:
        arr = np.asarray(arr)
        if arr.ndim == 1:
            arr = arr[:, None]
        if view is None:
            view = self.view(np.ascontiguousarray(arr).tobytes())
        a = {"bufferView": view, "byteOffset": offset, "componentType": _COMP[np.dtype(dtype or arr.dtype)],
             "count": int(count if count is not None else arr.shape[0]),
             "type": _TYPE[ncomp or arr.shape[1]]}
        if normalized:
            a["normalized"] = True
        if arr.dtype == np.float32 and arr.size and (ncomp or arr.shape[1]) == arr.shape[1]:
            a["min"] = arr.min(0).tolist()
            a["max"] = arr.max(0).tolist()
        self.doc["accessors"].append(a)
        return len(self.doc["accessors"]) - 1

    def mesh(self, primitives: list[dict], name: str | None = None) -> int:
        m = {"primitives": primitives}
        if name is not None:
            m["name"] = name
        self.doc["meshes"].append(m)
        return len(self.doc["meshes"]) - 1

    def node(self, **kw) -> int:
        self.doc["nodes"].append(kw)
        return len(self.doc["nodes"]) - 1

    def scene(self, roots: list[int]) -> None:
        self.doc["scenes"].append({"nodes": roots})
        self.doc["scene"] = len(self.doc["scenes"]) - 1

    def image(self, data: bytes, uri: str | None = None) -> int:
        im = {"uri": uri} if uri else {"bufferView": self.view(data), "mimeType": "image/png"}
        self.doc["images"].append(im)
        self.doc["textures"].append({"source": len(self.doc["images"]) - 1})
        return len(self.doc["textures"]) - 1

    def material(self, **kw) -> int:
        self.doc["materials"].append(kw)
        return len(self.doc["materials"]) - 1

    def save(self, path: Path, container: str = "gltf") -> Path:
        doc = json.loads(json.dumps(self.doc))
        for k in ("materials", "images", "textures"):
            if not doc[k]:
                del doc[k]
        data = bytes(self.bin)
        if container == "glb":
            doc["buffers"] = [{"byteLength": len(data)}]
            js = json.dumps(doc).encode()
            js += b" " * (-len(js) % 4)
            bn = data + b"\0" * (-len(data) % 4)
            body = struct.pack("<II", len(js), 0x4E4F534A) + js + struct.pack("<II", len(bn), 0x004E4942) + bn
            path.write_bytes(b"glTF" + struct.pack("<II", 2, 12 + len(body)) + body)
            return path
        if container == "datauri":
            doc["buffers"] = [{"byteLength": len(data),
                               "uri": "data:application/octet-stream;base64," + base64.b64encode(data).decode()}]
        else:
            binp = path.with_suffix(".bin")
            binp.write_bytes(data)
            doc["buffers"] = [{"byteLength": len(data), "uri": binp.name}]
        path.write_text(json.dumps(doc))
        return path


def quad_arrays(size: float = 1.0, z: float = 0.0):
    """A quad in the xy plane facing +z: positions, normals (length 2, to be
    normalised), glTF texture coordinates (origin at the top left), indices."""
    s = size
    pos = np.array([[0, 0, z], [s, 0, z], [s, s, z], [0, s, z]], dtype=np.float32)
    nrm = np.tile(np.array([0, 0, 2], dtype=np.float32), (4, 1))
    uv = np.array([[0, 1], [1, 1], [1, 0], [0, 0]], dtype=np.float32)
    idx = np.array([0, 1, 2, 0, 2, 3], dtype=np.uint16)
    return pos, nrm, uv, idx


def textured_panel_model(folder: Path, container: str = "glb", seed: int = 3) -> Path:
    """A glTF model for render tests: a panel with an RGBA base colour
    texture (alpha cut-outs, so transparent), a metallic-roughness texture,
    an occlusion texture and a normal map; a warm emissive quad above it.
    The panel's mesh sits two levels down the node tree, the light at the
    top level."""
    rng = np.random.default_rng(seed)
    b = GltfBuilder()
    pos, nrm, uv, idx = quad_arrays(1.0)
    p_acc = b.accessor(pos)
    n_acc = b.accessor(nrm)
    t_acc = b.accessor(uv)
    i_acc = b.accessor(idx)
    rgba = np.zeros((16, 16, 4), dtype=np.uint8)
    rgba[..., :3] = rng.integers(40, 255, (16, 16, 3), dtype=np.uint8)
    rgba[..., 3] = np.where((np.arange(16)[:, None] // 4 + np.arange(16)[None, :] // 4) % 2 == 0, 255, 0)
    mr = np.zeros((8, 8, 3), dtype=np.uint8)
    mr[..., 0] = 200  # occlusion
    mr[..., 1] = rng.integers(30, 220, (8, 8), dtype=np.uint8)  # roughness
    mr[..., 2] = rng.integers(0, 255, (8, 8), dtype=np.uint8)  # metallic
    nm = np.zeros((8, 8, 3), dtype=np.uint8)
    nm[..., 0] = rng.integers(100, 156, (8, 8), dtype=np.uint8)
    nm[..., 1] = rng.integers(100, 156, (8, 8), dtype=np.uint8)
    nm[..., 2] = 240
    t_rgba = b.image(png_bytes(rgba, folder))
    t_mr = b.image(png_bytes(mr, folder))
    t_nm = b.image(png_bytes(nm, folder))
    panel = b.material(name="Panel", pbrMetallicRoughness={
        "baseColorFactor": [0.9, 0.8, 0.7, 1.0], "baseColorTexture": {"index": t_rgba},
        "metallicRoughnessTexture": {"index": t_mr}, "metallicFactor": 0.6, "roughnessFactor": 0.8},
        occlusionTexture={"index": t_mr}, normalTexture={"index": t_nm})
    glow = b.material(name="Glow", emissiveFactor=[1.0, 0.8, 0.5],
                      extensions={"KHR_materials_emissive_strength": {"emissiveStrength": 6.0}})
    m_panel = b.mesh([{"attributes": {"POSITION": p_acc, "NORMAL": n_acc, "TEXCOORD_0": t_acc},
                       "indices": i_acc, "material": panel}], name="Panel")
    lpos = np.array([[0, 0, 0], [0.3, 0, 0], [0.3, 0, 0.3], [0, 0, 0.3]], dtype=np.float32)
    lnrm = np.tile(np.array([0, -1, 0], dtype=np.float32), (4, 1))
    m_light = b.mesh([{"attributes": {"POSITION": b.accessor(lpos), "NORMAL": b.accessor(lnrm)},
                       "indices": b.accessor(np.array([0, 1, 2, 0, 2, 3], dtype=np.uint16)), "material": glow}],
                     name="Glow")
    leaf = b.node(name="PanelMesh", mesh=m_panel, translation=[-0.5, -0.5, 0.0])
    mid = b.node(name="PanelPivot", children=[leaf], rotation=[0.0, 0.38268343, 0.0, 0.92387953])
    lamp = b.node(name="Lamp", mesh=m_light, translation=[-0.15, 0.45, -0.15])
    top = b.node(name="Top", children=[mid, lamp])
    b.scene([top])
    return b.save(folder / f"panel.{'glb' if container == 'glb' else 'gltf'}", container)
