"""Mesh and image I/O for the path tracer's host side.

OBJ: the reference imports models with assimp 5.2.5 using
aiProcess_Triangulate | aiProcess_FlipUVs | aiProcess_CalcTangentSpace and then
flips v once more (src/lib/vengine/core/io/AssimpLoadModel.cpp:55-130, 543).
assimp's OBJ importer emits one vertex per face corner; the two v flips cancel.
Tangents follow assimp's published CalcTangentSpace method: a per-face tangent
from the UV gradients, projected per corner onto the plane of that corner's
normal, then averaged over corners that share a position when both their
normals and tangents are within the 45 degree smoothing angle. Only the
tangent reaches the shading frame (fixFrame overwrites the bitangent), and it
is invariant under the v flip.

RGBE: Greg Ward's shared-exponent format as written by stb_image_write
(header "#?RADIANCE", FORMAT=32-bit_rle_rgbe, "-Y H +X W", new-style RLE
scanlines) and decoded as stb_image does (c * 2^(e - 136)).
"""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np

from .scene import VERTEX_DTYPE, Mesh

f32 = np.float32


# ---------------------------------------------------------------- OBJ

def _parse_obj(text: str):
    v, vt, vn = [], [], []
    faces = []  # list of corner lists (vi, ti, ni)
    name = "defaultobject"
    for line in text.splitlines():
        if not line or line[0] == "#":
            continue
        parts = line.split()
        tag = parts[0]
        if tag == "v":
            v.append([float(x) for x in parts[1:4]])
        elif tag == "vt":
            vt.append([float(x) for x in parts[1:3]])
        elif tag == "vn":
            vn.append([float(x) for x in parts[1:4]])
        elif tag == "o":
            name = parts[1] if len(parts) > 1 else name
        elif tag == "f":
            corners = []
            for c in parts[1:]:
                idx = c.split("/")
                vi = int(idx[0])
                ti = int(idx[1]) if len(idx) > 1 and idx[1] else 0
                ni = int(idx[2]) if len(idx) > 2 and idx[2] else 0
                corners.append((vi, ti, ni))
            faces.append(corners)
    return name, np.array(v, dtype=f32).reshape(-1, 3), np.array(vt, dtype=f32).reshape(-1, 2), \
        np.array(vn, dtype=f32).reshape(-1, 3), faces


def _fix(i: int, n: int) -> int:
    return i - 1 if i > 0 else n + i


def obj_arrays(path: str | Path) -> dict:
    """Parsed OBJ as arrays: v, vt, vn and triangulated corner indices
    (T x 3 x 3, 1-based position/uv/normal indices, 0 = absent)."""
    name, V, VT, VN, faces = _parse_obj(Path(path).read_text())
    tris = []
    for f in faces:
        # fan triangulation (aiProcess_Triangulate on convex polygons)
        for k in range(1, len(f) - 1):
            tris.append((f[0], f[k], f[k + 1]))
    corners = np.zeros((len(tris), 3, 3), dtype=np.int64)
    for t, tri in enumerate(tris):
        for c in range(3):
            vi, ti, ni = tri[c]
            corners[t, c] = (_fix(vi, len(V)) + 1, (_fix(ti, len(VT)) + 1) if ti else 0,
                             (_fix(ni, len(VN)) + 1) if ni else 0)
    return {"name": name, "v": V, "vt": VT, "vn": VN, "f": corners.astype(np.int32)}


def mesh_from_obj_arrays(name: str, V: np.ndarray, VT: np.ndarray, VN: np.ndarray, F: np.ndarray) -> Mesh:
    """Builds a Mesh with one vertex per face corner, in face order (assimp's OBJ importer)."""
    F = np.asarray(F, dtype=np.int64).reshape(-1, 3)
    n = F.shape[0]
    pos = np.asarray(V, dtype=f32)[F[:, 0] - 1]
    uv = np.zeros((n, 2), dtype=f32)
    if len(VT):
        ok = F[:, 1] > 0
        uv[ok] = np.asarray(VT, dtype=f32)[F[ok, 1] - 1]
    nrm = np.zeros((n, 3), dtype=f32)
    if len(VN) and (F[:, 2] > 0).all():
        nrm = np.asarray(VN, dtype=f32)[F[:, 2] - 1]
    else:
        p = pos.reshape(-1, 3, 3).astype(np.float64)
        fn = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
        fn /= np.maximum(np.linalg.norm(fn, axis=1, keepdims=True), 1e-30)
        nrm = np.repeat(fn, 3, axis=0).astype(f32)
    # AssimpLoadModel.cpp:72: normals normalised
    lens = np.sqrt((nrm.astype(np.float64) ** 2).sum(axis=1))
    nrm = (nrm / np.where(lens > 0, lens, 1.0)[:, None]).astype(f32)
    tangent, bitangent = calc_tangent_space(pos, uv, nrm)
    verts = np.zeros(n, dtype=VERTEX_DTYPE)
    verts["position"] = pos
    verts["uv"] = uv  # FlipUVs then 1 - v again: net original v
    verts["normal"] = nrm
    verts["color"] = 1.0
    verts["tangent"] = tangent
    verts["bitangent"] = bitangent
    return Mesh(name=name, vertices=verts, indices=np.arange(n, dtype=np.uint32).reshape(-1, 3))


def load_obj(path: str | Path) -> Mesh:
    """Loads a single-object OBJ as one Mesh in assimp's vertex order."""
    a = obj_arrays(path)
    return mesh_from_obj_arrays(a["name"], a["v"], a["vt"], a["vn"], a["f"].reshape(-1, 3))


def calc_tangent_space(pos: np.ndarray, uv: np.ndarray, nrm: np.ndarray, max_angle_deg: float = 45.0,
                       faces: np.ndarray | None = None):
    """Per-vertex tangents/bitangents, restating assimp 5.2.5's
    CalcTangentSpace step in float32:

    1. per face, with v = p1 - p0, w = p2 - p0 and UV deltas (sx, sy), (tx, ty):
       tangent = (w*sy - v*ty) * dirCorrection, bitangent = (v*tx - w*sx) * dirCorrection,
       dirCorrection = -1 when tx*sy - ty*sx < 0; degenerate UVs use (0,1),(1,0);
    2. per face corner, both projected onto the plane of that vertex's normal
       and normalised, and stored at the vertex; faces are visited in order,
       so a vertex shared by several faces (indexed meshes) keeps the last
       face's value;
    3. smoothing, visiting vertices in index order: a vertex not yet assigned
       gathers every unassigned vertex within the position epsilon
       (1e-4 x bounding-box diagonal) whose normal has a dot product >= 0.9999
       and whose tangent and bitangent are within the smoothing angle of its
       own. The seed vertex is part of the neighbour search as well, so it
       enters the sum twice. The normalised sums replace all gathered values.

    `faces` (F x 3 vertex indices) describes an indexed mesh (glTF); without
    it the vertices are face corners grouped in threes (assimp's OBJ output).
    Vertices no face uses keep zero vectors.
    """
    from scipy.spatial import cKDTree

    n = pos.shape[0]
    faces = (np.arange(n, dtype=np.int64) if faces is None else np.asarray(faces, dtype=np.int64)).reshape(-1, 3)
    p = pos.astype(f32)[faces]
    t = uv.astype(f32)[faces]
    v = p[:, 1] - p[:, 0]
    w = p[:, 2] - p[:, 0]
    sx = t[:, 1, 0] - t[:, 0, 0]
    sy = t[:, 1, 1] - t[:, 0, 1]
    tx = t[:, 2, 0] - t[:, 0, 0]
    ty = t[:, 2, 1] - t[:, 0, 1]
    dir_corr = np.where(tx * sy - ty * sx < 0, f32(-1), f32(1)).astype(f32)
    degen = sx * ty == sy * tx
    sx = np.where(degen, 0, sx).astype(f32)
    sy = np.where(degen, 1, sy).astype(f32)
    tx = np.where(degen, 1, tx).astype(f32)
    ty = np.where(degen, 0, ty).astype(f32)
    tan = np.repeat(((w * sy[:, None] - v * ty[:, None]) * dir_corr[:, None]).astype(f32), 3, axis=0)
    bit = np.repeat(((-w * sx[:, None] + v * tx[:, None]) * dir_corr[:, None]).astype(f32), 3, axis=0)
    corner_vertex = faces.ravel()
    nn = nrm.astype(f32)
    nc = nn[corner_vertex]
    ct = (tan - nc * (tan * nc).sum(1, keepdims=True)).astype(f32)
    cb = (bit - nc * (bit * nc).sum(1, keepdims=True)).astype(f32)

    def _normalize_safe(a):
        ln = np.sqrt((a * a).sum(1, keepdims=True))
        return np.where(ln > 0, a / np.where(ln > 0, ln, 1), a).astype(f32)

    ct = _normalize_safe(ct)
    cb = _normalize_safe(cb)
    # non-finite frames: rebuild from the normal
    bad = ~(np.isfinite(ct).all(1) & np.isfinite(cb).all(1)) | ~(np.abs(ct).sum(1) > 0)
    for i in np.nonzero(bad)[0]:
        a = np.array([1.0, 0.0, 0.0]) if abs(nc[i, 0]) < 0.9 else np.array([0.0, 1.0, 0.0])
        tt = np.cross(nc[i], a)
        ct[i] = tt / np.linalg.norm(tt)
        cb[i] = np.cross(nc[i], ct[i])
    # the last face corner of each vertex wins
    last = np.full(n, -1, dtype=np.int64)
    np.maximum.at(last, corner_vertex, np.arange(corner_vertex.size, dtype=np.int64))
    used = last >= 0
    lt = np.zeros((n, 3), dtype=f32)
    lb = np.zeros((n, 3), dtype=f32)
    lt[used] = ct[last[used]]
    lb[used] = cb[last[used]]

    eps = float(np.linalg.norm(pos.max(0) - pos.min(0))) * 1e-4
    neighbours = cKDTree(pos.astype(np.float64)).query_ball_point(pos.astype(np.float64), r=max(eps, 1e-12))
    limit = f32(math.cos(math.radians(max_angle_deg)))
    T = lt.copy()
    B = lb.copy()
    done = ~used
    for a in range(n):
        if done[a]:
            continue
        found = np.sort(np.asarray(neighbours[a], dtype=np.int64))
        found = found[~done[found]]
        if found.size <= 1:
            continue  # only itself: the normalised value stays
        keep = ((nn[found] @ nn[a]) >= f32(0.9999)) & ((T[found] @ lt[a]) >= limit) & ((B[found] @ lb[a]) >= limit)
        group = np.concatenate([[a], found[keep]])
        done[found[keep]] = True
        st = T[group].sum(0, dtype=f32)
        sb = B[group].sum(0, dtype=f32)
        st = (st / np.sqrt(st @ st)).astype(f32)
        sb = (sb / np.sqrt(sb @ sb)).astype(f32)
        T[group] = st
        B[group] = sb
    return T.astype(f32), B.astype(f32)


# ---------------------------------------------------------------- RGBE (Radiance .hdr)

def rgbe_encode(rgb: np.ndarray) -> np.ndarray:
    """float RGB (H x W x 3) -> RGBE bytes (H x W x 4), stb_image_write's rule."""
    rgb = np.asarray(rgb, dtype=np.float32)
    m = rgb.max(axis=-1)
    out = np.zeros(rgb.shape[:-1] + (4,), dtype=np.uint8)
    ok = m >= 1e-32
    mant, ex = np.frexp(m[ok].astype(np.float32))
    scale = (mant.astype(np.float32) * np.float32(256.0) / m[ok]).astype(np.float32)
    vals = (rgb[ok] * scale[:, None]).astype(np.float32)
    out[ok, :3] = vals.astype(np.uint8)
    out[ok, 3] = (ex + 128).astype(np.uint8)
    return out


def rgbe_decode(rgbe: np.ndarray) -> np.ndarray:
    """RGBE bytes -> float32 RGB, stb_image's rule (no half-step offset)."""
    rgbe = np.asarray(rgbe, dtype=np.uint8)
    e = rgbe[..., 3].astype(np.int32)
    f = np.where(e != 0, np.ldexp(np.float32(1.0), e - 136), 0.0).astype(np.float32)
    return (rgbe[..., :3].astype(np.float32) * f[..., None]).astype(np.float32)


def read_hdr_rgbe(path: str | Path) -> np.ndarray:
    """Reads a Radiance file written with new-style RLE; returns H x W x 4 RGBE bytes."""
    data = Path(path).read_bytes()
    pos = 0
    lines = []
    while True:
        end = data.index(b"\n", pos)
        line = data[pos:end].decode("latin-1")
        pos = end + 1
        if line.startswith("-Y") or line.startswith("+Y"):
            lines.append(line)
            break
        lines.append(line)
    if not lines[0].startswith("#?RADIANCE") and not lines[0].startswith("#?RGBE"):
        raise ValueError("not a Radiance file")
    parts = lines[-1].split()
    H, W = int(parts[1]), int(parts[3])
    out = np.zeros((H, W, 4), dtype=np.uint8)
    buf = np.frombuffer(data, dtype=np.uint8)
    for y in range(H):
        if (W >= 8 and W < 32768 and int(buf[pos]) == 2 and int(buf[pos + 1]) == 2
                and (int(buf[pos + 2]) << 8 | int(buf[pos + 3])) == W):
            pos += 4
            for c in range(4):
                x = 0
                while x < W:
                    count = int(buf[pos])
                    pos += 1
                    if count > 128:
                        count -= 128
                        out[y, x:x + count, c] = buf[pos]
                        pos += 1
                    else:
                        out[y, x:x + count, c] = buf[pos:pos + count]
                        pos += count
                    x += count
        else:
            out[y] = buf[pos:pos + 4 * W].reshape(W, 4)
            pos += 4 * W
    return out


def read_hdr(path: str | Path) -> np.ndarray:
    return rgbe_decode(read_hdr_rgbe(path))


def _rle_channel(row: np.ndarray) -> bytes:
    """stb_image_write's run-length encoding of one scanline channel."""
    out = bytearray()
    n = len(row)
    x = 0
    while x < n:
        r = x
        while r + 2 < n:
            if row[r] == row[r + 1] and row[r] == row[r + 2]:
                break
            r += 1
        if r + 2 >= n:
            r = n
        # literals x..r
        while x < r:
            len_ = min(r - x, 128)
            out.append(len_)
            out.extend(bytes(row[x:x + len_]))
            x += len_
        if r + 2 < n:
            run_end = r
            while run_end < n and row[run_end] == row[r]:
                run_end += 1
            while x < run_end:
                len_ = min(run_end - x, 127)
                out.append(len_ + 128)
                out.append(int(row[r]))
                x += len_
    return bytes(out)


def write_hdr(path: str | Path, image: np.ndarray) -> None:
    """Writes RGB(A) float data as an RLE Radiance file (alpha ignored)."""
    img = np.asarray(image, dtype=np.float32)
    H, W = img.shape[:2]
    rgbe = rgbe_encode(img[..., :3])
    head = f"#?RADIANCE\n# Written by stb_image_write\nFORMAT=32-bit_rle_rgbe\n\n-Y {H} +X {W}\n".encode()
    body = bytearray()
    for y in range(H):
        if 8 <= W < 32768:
            body.extend(bytes([2, 2, (W >> 8) & 0xFF, W & 0xFF]))
            for c in range(4):
                body.extend(_rle_channel(rgbe[y, :, c]))
        else:
            body.extend(rgbe[y].tobytes())
    Path(path).write_bytes(head + bytes(body))


def srgb_encode(linear: np.ndarray) -> np.ndarray:
    """linearToSRGB(clamp(x, 0, 1)) in float32 arithmetic, as
    ImageUtils.cpp:12-21 evaluates it (float constants, powf)."""
    x = np.clip(np.asarray(linear, dtype=np.float32), np.float32(0.0), np.float32(1.0))
    lin = x * np.float32(12.92)
    pw = np.float32(1.055) * np.power(x, np.float32(1.0) / np.float32(2.4)) - np.float32(0.055)
    return np.where(x <= np.float32(0.0031308), lin, pw).astype(np.float32)
