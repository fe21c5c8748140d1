"""vviewer scene files (JSON): import into an Engine and export from one.

Follows the reference's format and loading steps:
  * parsing: src/lib/vengine/core/io/Import.cpp:26-566 (vec2/3/4 given as
    {x,y,z[,w]} or {r,g,b[,a]} objects, arrays of 1..4 floats or one float;
    rotations as Euler degrees (vec3) or a quaternion (x, y, z, w); camera by
    target + up or by rotation; materials LAMBERT / PBR_STANDARD / VOLUME,
    EMBEDDED ones named "<model file stem>:<name>" coming with their model;
    lights POINT / DIRECTIONAL; scene objects with transform, mesh, material,
    light, volume and children);
  * applying: src/bin/vviewer/UI/MainWindow.cpp:598-672 (camera through
    Transform::setRotation(forward, up), src/lib/vengine/math/Transform.cpp:90-100;
    models, materials, lights, objects; environment map and type);
  * export: src/lib/vengine/core/io/Export.cpp (the same fields).
Models are glTF 2.0 (.gltf, .glb) or Wavefront OBJ files, imported by
model3d.import_model with the materials a glTF file carries;
textures are 8-bit PNG (albedo and emissive sRGB, the rest linear); the
environment is a Radiance .hdr image used as the equirectangular map.
"""
from __future__ import annotations

import json
import math
import struct
import zlib
from pathlib import Path

import numpy as np

from . import _native as N
from .assets import read_hdr
from .scene import (EnvironmentType, Engine, LightType, MaterialLambert, MaterialPBRStandard, MaterialVolume,
                    Transform, quat_from_euler, quat_to_mat3)

f32 = np.float32

# ---------------------------------------------------------------- PNG (8/16-bit, non-interlaced)


def read_png(path: str | Path) -> np.ndarray:
    """H x W x 4 uint8 RGBA from a PNG file (grey, grey+alpha, RGB, RGBA,
    palette; bit depth 8 or 16; no interlacing)."""
    return decode_png(Path(path).read_bytes(), str(path))[0]


def decode_png(data: bytes, path: str = "PNG") -> tuple[np.ndarray, int]:
    """(H x W x 4 uint8 RGBA, channels in the file) of PNG data. The channel
    count is stb_image's: 1 grey, 2 grey+alpha, 3 RGB, 4 RGBA, and 3 or 4 for
    a palette image (4 with a transparency chunk)."""
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError(f"{path}: not a PNG file")
    pos, idat, plte, trns = 8, [], None, None
    w = h = depth = ctype = interlace = None
    while pos < len(data):
        n, tag = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        pos += 12 + n
        if tag == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
        elif tag == b"PLTE":
            plte = np.frombuffer(body, dtype=np.uint8).reshape(-1, 3)
        elif tag == b"tRNS":
            trns = np.frombuffer(body, dtype=np.uint8)
        elif tag == b"IDAT":
            idat.append(body)
        elif tag == b"IEND":
            break
    if interlace:
        raise ValueError(f"{path}: interlaced PNG is not supported")
    channels = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    bpp = max(1, channels * depth // 8)
    stride = (w * channels * depth + 7) // 8
    raw = zlib.decompress(b"".join(idat))
    out = np.zeros((h, stride), dtype=np.uint8)
    prev = np.zeros(stride, dtype=np.int64)
    for y in range(h):
        ft = raw[y * (stride + 1)]
        line = np.frombuffer(raw, dtype=np.uint8, count=stride, offset=y * (stride + 1) + 1).astype(np.int64)
        if ft == 0:
            cur = line
        elif ft == 2:  # Up
            cur = (line + prev) & 0xFF
        elif ft == 1 and stride % bpp == 0:  # Sub: a running sum per byte lane
            cur = np.cumsum(line.reshape(-1, bpp), axis=0).ravel() & 0xFF
        else:  # Average, Paeth: sequential along the row
            ln, pv = line.tolist(), prev.tolist()
            cl = [0] * stride
            for i in range(stride):
                a = cl[i - bpp] if i >= bpp else 0
                b = pv[i]
                if ft == 1:
                    p = a
                elif ft == 3:
                    p = (a + b) >> 1
                else:  # Paeth
                    c = pv[i - bpp] if i >= bpp else 0
                    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                    p = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cl[i] = (ln[i] + p) & 0xFF
            cur = np.asarray(cl, dtype=np.int64)
        out[y] = cur
        prev = cur
    if depth == 16:
        px = out.reshape(h, w, channels, 2)[..., 0]  # high byte
    elif depth == 8:
        px = out.reshape(h, w, channels)
    else:
        bits = np.unpackbits(out, axis=1)[:, :w * depth].reshape(h, w, depth)
        px = (bits * (1 << np.arange(depth - 1, -1, -1))).sum(-1).astype(np.uint8)[..., None]
        if ctype == 0:
            px = (px.astype(np.uint32) * 255 // ((1 << depth) - 1)).astype(np.uint8)
    rgba = np.full((h, w, 4), 255, dtype=np.uint8)
    if ctype == 3:
        idx = px[..., 0]
        rgba[..., :3] = plte[idx]
        if trns is not None:
            alpha = np.full(256, 255, dtype=np.uint8)
            alpha[:len(trns)] = trns
            rgba[..., 3] = alpha[idx]
    elif channels in (1, 2):
        rgba[..., :3] = px[..., :1]
        if channels == 2:
            rgba[..., 3] = px[..., 1]
    else:
        rgba[..., :channels] = px
    file_channels = (4 if trns is not None else 3) if ctype == 3 else channels
    return rgba, file_channels


# ---------------------------------------------------------------- value parsing (Import.cpp:41-213)

def _vec(o: dict, name: str, n: int, default):
    if name not in o:
        return list(default)
    v = o[name]
    if isinstance(v, dict):
        keys = ("x", "y", "z", "w")[:n]
        alt = ("r", "g", "b", "a")[:n]
        out = []
        for k, a in zip(keys, alt):
            if k in v:
                out.append(float(v[k]))
            elif a in v:
                out.append(float(v[a]))
            else:
                raise ValueError(f"field {name} is malformed")
        return out
    if isinstance(v, list):
        if len(v) == 1:
            return [float(v[0])] * n
        if len(v) == n:
            return [float(x) for x in v]
        raise ValueError(f"field {name} is malformed")
    if isinstance(v, (int, float)):
        return [float(v)] * n
    raise ValueError(f"field {name} is malformed")


def _rotation(o: dict, name: str, default):
    """Euler angles in degrees (vec3) or a quaternion (x, y, z, w); returns (w, x, y, z)."""
    if name not in o:
        return np.asarray(default, dtype=f32)
    try:
        e = _vec(o, name, 3, (0, 0, 0))
        return quat_from_euler([math.radians(x) for x in e])
    except ValueError:
        x, y, z, w = _vec(o, name, 4, (0, 0, 0, 1))
        return np.array([w, x, y, z], dtype=f32)


def quat_from_mat3(m) -> np.ndarray:
    """glm::quat_cast of a rotation matrix m (rows), (w, x, y, z): the largest
    of the four squared components picks the formula."""
    m = np.asarray(m, dtype=np.float64)
    # glm indexes m[col][row]; here m is row-major: element (row r, col c) = m[r][c]
    fx = m[0, 0] - m[1, 1] - m[2, 2]
    fy = m[1, 1] - m[0, 0] - m[2, 2]
    fz = m[2, 2] - m[0, 0] - m[1, 1]
    fw = m[0, 0] + m[1, 1] + m[2, 2]
    big, k = max((fw, 0), (fx, 1), (fy, 2), (fz, 3))
    v = math.sqrt(big + 1.0) * 0.5
    mult = 0.25 / v
    if k == 0:
        q = (v, (m[2, 1] - m[1, 2]) * mult, (m[0, 2] - m[2, 0]) * mult, (m[1, 0] - m[0, 1]) * mult)
    elif k == 1:
        q = ((m[2, 1] - m[1, 2]) * mult, v, (m[1, 0] + m[0, 1]) * mult, (m[0, 2] + m[2, 0]) * mult)
    elif k == 2:
        q = ((m[0, 2] - m[2, 0]) * mult, (m[1, 0] + m[0, 1]) * mult, v, (m[2, 1] + m[1, 2]) * mult)
    else:
        q = ((m[1, 0] - m[0, 1]) * mult, (m[0, 2] + m[2, 0]) * mult, (m[2, 1] + m[1, 2]) * mult, v)
    return np.asarray(q, dtype=f32)


def rotation_from_forward_up(forward, up) -> np.ndarray:
    """Transform::setRotation(forward, up): columns X = up x Z, Y = Z x X,
    Z = -forward."""
    z = -np.asarray(forward, dtype=np.float64)
    z /= np.linalg.norm(z)
    y = np.asarray(up, dtype=np.float64)
    y /= np.linalg.norm(y)
    x = np.cross(y, z)
    x /= np.linalg.norm(x)
    y = np.cross(z, x)
    y /= np.linalg.norm(y)
    return quat_from_mat3(np.stack([x, y, z], axis=1))


# ---------------------------------------------------------------- import

_MATERIALS = {"LAMBERT": MaterialLambert, "PBR_STANDARD": MaterialPBRStandard, "VOLUME": MaterialVolume}


def _texture(engine: Engine, o: dict, folder: Path, srgb: bool, cache: dict):
    if "texture" not in o:
        return None
    t = o["texture"]
    if t.get("type", "STANDALONE") != "STANDALONE" or "filepath" not in t:
        raise ValueError(f"texture {t.get('name')}: only standalone texture files are supported")
    path = folder / t["filepath"]
    key = (str(path), srgb)
    if key not in cache:
        cache[key] = engine.add_texture(N.TEXTURE_RGBA8_SRGB if srgb else N.TEXTURE_RGBA8_LINEAR, read_png(path))
    return cache[key]


def import_scene(path: str | Path, engine: Engine | None = None) -> Engine:
    """Reads a vviewer scene file into `engine` (a new Engine by default)."""
    path = Path(path)
    folder = path.parent
    doc = json.loads(path.read_text())
    engine = engine or Engine()
    scene = engine.scene
    tex_cache: dict = {}

    # camera (MainWindow.cpp:606-619)
    c = doc["camera"]
    cam = scene.camera
    pos = np.asarray(_vec(c, "position", 3, (0, 0, 0)), dtype=f32)
    if "target" in c:
        target = np.asarray(_vec(c, "target", 3, (0, 0, -1)), dtype=f32)
        up = _vec(c, "up", 3, (0, 1, 0))
    elif "rotation" in c:
        q = _rotation(c, "rotation", (1, 0, 0, 0))
        r = quat_to_mat3(q)
        target = pos + r @ np.array([0, 0, -1], dtype=f32)
        up = r @ np.array([0, 1, 0], dtype=f32)
    else:
        raise ValueError("camera: missing target or rotation")
    cam.transform = Transform(pos, (1, 1, 1), rotation_from_forward_up(target - pos, up))
    cam.fov = float(c.get("fov", cam.fov))
    cam.znear = float(c.get("znear", cam.znear))
    cam.zfar = float(c.get("zfar", cam.zfar))
    cam.lens_radius = float(c.get("lensRadius", cam.lens_radius))
    cam.focal_distance = float(c.get("focalDistance", cam.focal_distance))
    camera_volume = c.get("volume", "")

    # models, with their embedded materials (MainWindow.cpp:638-642)
    from .model3d import import_model

    models = {}
    for m in doc.get("models", []):
        models[m["name"]] = import_model(engine, folder / m["filepath"], name=m["name"])

    # materials (Import.cpp:370-432); EMBEDDED ones came with their model
    for m in doc.get("materials", []):
        if m["type"] == "EMBEDDED":
            continue
        cls = _MATERIALS.get(m["type"])
        if cls is None:
            raise ValueError(f"material {m['name']}: {m['type']} materials are not supported")
        mat = engine.create_material(cls, m["name"])
        if cls is MaterialVolume:
            if "scattering" in m:
                mat.sigma_s = _vec(m["scattering"], "value", 3, mat.sigma_s[:3]) + [mat.sigma_s[3]]
            if "absorption" in m:
                mat.sigma_a = _vec(m["absorption"], "value", 3, mat.sigma_a[:3]) + [mat.sigma_a[3]]
            if "g" in m:
                mat.g = float(m["g"])
            continue
        if cls is MaterialPBRStandard:
            if "roughness" in m:
                t = _texture(engine, m["roughness"], folder, False, tex_cache)
                if t is not None:
                    mat.roughness_texture = t
                mat.roughness = float(m["roughness"].get("value", mat.roughness))
            if "metallic" in m:
                t = _texture(engine, m["metallic"], folder, False, tex_cache)
                if t is not None:
                    mat.metallic_texture = t
                mat.metallic = float(m["metallic"].get("value", mat.metallic))
        if "albedo" in m:
            t = _texture(engine, m["albedo"], folder, True, tex_cache)
            if t is not None:
                mat.albedo_texture = t
            mat.albedo = _vec(m["albedo"], "value", 4, mat.albedo)
        if "ao" in m:
            t = _texture(engine, m["ao"], folder, False, tex_cache)
            if t is not None:
                mat.ao_texture = t
            mat.ao = float(m["ao"].get("value", mat.ao))
        if "emissive" in m:
            t = _texture(engine, m["emissive"], folder, True, tex_cache)
            if t is not None:
                mat.emissive_texture = t
            mat.emissive = _vec(m["emissive"], "value", 4, mat.emissive)
        if "normal" in m:
            t = _texture(engine, m["normal"], folder, False, tex_cache)
            if t is not None:
                mat.normal_texture = t
        if "alpha" in m:
            t = _texture(engine, m["alpha"], folder, False, tex_cache)
            if t is not None:
                mat.alpha_texture = t
        if "transparent" in m:
            mat.set_transparent(bool(m["transparent"]))
        if "scale" in m:
            mat.u_tiling, mat.v_tiling = _vec(m, "scale", 2, (mat.u_tiling, mat.v_tiling))

    # lights (Import.cpp:434-452)
    for lt in doc.get("lights", []):
        type_ = {"POINT": LightType.POINT_LIGHT, "DIRECTIONAL": LightType.DIRECTIONAL_LIGHT}.get(
            lt.get("type", "POINT"))
        if type_ is None:
            raise ValueError(f"light {lt['name']}: {lt['type']} lights are not supported")
        color = _vec(lt, "color", 3, (1, 1, 1))
        engine.create_light(lt["name"], type_, (*color, float(lt.get("intensity", 1.0))))

    # scene objects (Import.cpp:330-365; MainWindow addImportedSceneObject)
    def add(o: dict, parent):
        tr = o.get("transform", {})
        t = Transform(_vec(tr, "position", 3, (0, 0, 0)), _vec(tr, "scale", 3, (1, 1, 1)),
                      _rotation(tr, "rotation", (1, 0, 0, 0)))
        so = scene.add_scene_object(o["name"], t, parent)
        so.active = bool(o.get("active", True))
        if "mesh" in o:
            model = o["mesh"]["modelName"]
            if model not in models:
                raise ValueError(f"object {o['name']}: unknown model {model}")
            sub = o["mesh"].get("submesh")
            candidates = models[model].meshes()
            mesh = models[model].mesh(sub) if sub is not None else None
            if mesh is None and len(candidates) == 1:
                # a one-mesh model whose mesh name differs (assimp's naming of
                # unnamed OBJ objects, for one): its only mesh
                mesh = candidates[0]
            if mesh is None:
                raise ValueError(f"object {o['name']}: model {model} has no mesh {sub!r}")
            so.mesh = mesh
        if "material" in o:
            so.material = engine.material(o["material"]["name"])
        if "light" in o:
            so.light = engine.light(o["light"]["name"])
            so.cast_shadows = bool(o["light"].get("shadows", True))
        if "volume" in o:
            v = o["volume"]
            if "frontFacing" in v:
                so.volume_front = engine.material(v["frontFacing"])
            if "backFacing" in v:
                so.volume_back = engine.material(v["backFacing"])
        for ch in o.get("children", []):
            add(ch, so)

    for o in doc.get("scene", []):
        add(o, None)

    # environment (Import.cpp:454-465, MainWindow.cpp:646-663)
    env = doc.get("environment", {})
    if env.get("path"):
        img = read_hdr(folder / env["path"])
        rgba = np.ones((*img.shape[:2], 4), dtype=f32)
        rgba[..., :3] = img[..., :3]
        scene.environment_map = rgba
    if "environmentType" in env:
        scene.environment_type = EnvironmentType(int(env["environmentType"]))
    if "backgroundColor" in env:
        scene.background_color = _vec(env, "backgroundColor", 3, scene.background_color[:3])
    if camera_volume:
        cam.volume = engine.material(camera_volume)
    return engine


# ---------------------------------------------------------------- export

def _write_obj(path: Path, mesh) -> None:
    v = mesh.vertices
    lines = [f"o {mesh.name}"]
    lines += [f"v {p[0]:.9g} {p[1]:.9g} {p[2]:.9g}" for p in v["position"]]
    lines += [f"vt {t[0]:.9g} {t[1]:.9g}" for t in v["uv"]]
    lines += [f"vn {n[0]:.9g} {n[1]:.9g} {n[2]:.9g}" for n in v["normal"]]
    for a, b, c in np.asarray(mesh.indices, dtype=np.int64).reshape(-1, 3) + 1:
        lines.append(f"f {a}/{a}/{a} {b}/{b}/{b} {c}/{c}/{c}")
    path.write_text("\n".join(lines) + "\n")


def export_scene(engine: Engine, path: str | Path) -> None:
    """Writes the engine's scene as a vviewer scene file; meshes go to OBJ
    files beside it (materials' texture images are not exported: their
    values are)."""
    path = Path(path)
    folder = path.parent
    scene = engine.scene
    cam = scene.camera
    pos = cam.transform.position
    doc = {"camera": {"position": [float(x) for x in pos],
                      "target": [float(x) for x in pos + cam.transform.forward()],
                      "up": [float(x) for x in cam.transform.up()],
                      "fov": cam.fov, "znear": cam.znear, "zfar": cam.zfar, "lensRadius": cam.lens_radius,
                      "focalDistance": cam.focal_distance}}
    if cam.volume is not None:
        doc["camera"]["volume"] = cam.volume.name
    used_meshes = {}
    for so in scene.objects_flat():
        if so.mesh is not None:
            used_meshes[so.mesh.name + f"_{so.mesh.index}"] = so.mesh
    models = []
    for name, mesh in used_meshes.items():
        _write_obj(folder / f"{name}.obj", mesh)
        models.append({"name": name, "filepath": f"{name}.obj"})
    doc["models"] = models
    mats = []
    for m in engine.materials:
        if isinstance(m, MaterialVolume):
            mats.append({"name": m.name, "type": "VOLUME", "scattering": {"value": m.sigma_s[:3]},
                         "absorption": {"value": m.sigma_a[:3]}, "g": m.g})
            continue
        d = {"name": m.name, "type": "LAMBERT" if isinstance(m, MaterialLambert) else "PBR_STANDARD",
             "albedo": {"value": list(m.albedo)}, "ao": {"value": m.ao}, "emissive": {"value": list(m.emissive)},
             "transparent": m.transparent, "scale": [m.u_tiling, m.v_tiling]}
        if isinstance(m, MaterialPBRStandard):
            d["roughness"] = {"value": m.roughness}
            d["metallic"] = {"value": m.metallic}
        mats.append(d)
    doc["materials"] = mats
    doc["lights"] = [{"name": lt.name, "type": "POINT" if lt.type == LightType.POINT_LIGHT else "DIRECTIONAL",
                      "color": lt.color[:3], "intensity": lt.color[3]} for lt in engine.lights]

    def obj(so):
        t = so.local_transform
        w, x, y, z = (float(v) for v in t.rotation)
        d = {"name": so.name, "active": so.active,
             "transform": {"position": [float(v) for v in t.position], "scale": [float(v) for v in t.scale],
                           "rotation": [x, y, z, w]}}
        if so.mesh is not None:
            d["mesh"] = {"modelName": so.mesh.name + f"_{so.mesh.index}", "submesh": so.mesh.name}
        if so.material is not None:
            d["material"] = {"name": so.material.name}
        if so.light is not None:
            d["light"] = {"name": so.light.name, "shadows": so.cast_shadows}
        vol = {}
        if so.volume_front is not None:
            vol["frontFacing"] = so.volume_front.name
        if so.volume_back is not None:
            vol["backFacing"] = so.volume_back.name
        if vol:
            d["volume"] = vol
        if so.children:
            d["children"] = [obj(c) for c in so.children]
        return d

    doc["scene"] = [obj(so) for so in scene.roots]
    env = {"environmentType": int(scene.environment_type), "backgroundColor": list(scene.background_color[:3])}
    if scene.environment_map is not None:
        from .assets import write_hdr
        write_hdr(folder / "environment.hdr", scene.environment_map[..., :3])
        env["path"] = "environment.hdr"
    doc["environment"] = env
    path.write_text(json.dumps(doc, indent=2))
