"""Seeded procedural scenes for the benchmark workloads.

cornell_box      256 x 256, 64 spp, depth 8: room [0,1]^3 open at z = 1, red/green
                 side walls, two seeded boxes, a 0.25 x 0.25 ceiling light of
                 radiance (17, 12, 4), pinhole camera at (0.5, 0.5, 2.2), fov 40.
cornell_medium   the same room filled with a homogeneous isotropic medium
                 (sigma_a 0.05, sigma_s 0.2) plus ~1M triangles as 8 noise-displaced
                 geodesic spheres with metallic/roughness materials; 1920 x 1080,
                 256 spp, depth 12.

The medium fills the room the way the reference models media: an invisible
transparent boundary cube (alpha 0) whose back-facing volume is the medium
(src/lib/vengine/core/Instances.cpp:90-97, shaders/pt/rayPrimaryPBRStandard.rchit.glsl:74-89).
"""
from __future__ import annotations

import math

import numpy as np

from .assets import calc_tangent_space
from .renderer import RenderInfo
from .scene import (VERTEX_DTYPE, EnvironmentType, Engine, MaterialLambert, MaterialPBRStandard, MaterialVolume,
                    Mesh, Transform, radians)

f32 = np.float32


def mesh_from_triangles(name: str, pos: np.ndarray, uv: np.ndarray | None = None,
                        nrm: np.ndarray | None = None) -> Mesh:
    """Mesh from per-corner arrays (3 corners per triangle)."""
    pos = np.asarray(pos, dtype=f32).reshape(-1, 3)
    n = pos.shape[0]
    if uv is None:
        uv = np.zeros((n, 2), dtype=f32)
    if nrm is None:
        nrm = np.zeros((n, 3), dtype=f32)
        p = pos.reshape(-1, 3, 3).astype(np.float64)
        fn = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
        fn /= np.maximum(np.linalg.norm(fn, axis=1, keepdims=True), 1e-30)
        nrm = np.repeat(fn, 3, axis=0).astype(f32)
    t, b = calc_tangent_space(pos, np.asarray(uv, dtype=f32), np.asarray(nrm, dtype=f32))
    v = np.zeros(n, dtype=VERTEX_DTYPE)
    v["position"] = pos
    v["uv"] = uv
    v["normal"] = nrm
    v["color"] = 1.0
    v["tangent"] = t
    v["bitangent"] = b
    return Mesh(name, v, np.arange(n, dtype=np.uint32).reshape(-1, 3))


def indexed_mesh(name: str, pos: np.ndarray, tris: np.ndarray, uv: np.ndarray, nrm: np.ndarray) -> Mesh:
    """Mesh with shared vertices; tangents from per-face UV gradients averaged per vertex."""
    pos = np.asarray(pos, dtype=f32)
    tris = np.asarray(tris, dtype=np.uint32)
    uv = np.asarray(uv, dtype=f32)
    nrm = np.asarray(nrm, dtype=f32)
    p = pos[tris].astype(np.float64)
    t = uv[tris].astype(np.float64)
    e1, e2 = p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]
    d1, d2 = t[:, 1] - t[:, 0], t[:, 2] - t[:, 0]
    r = d1[:, 0] * d2[:, 1] - d2[:, 0] * d1[:, 1]
    sgn = np.where(r < 0, -1.0, 1.0)
    tan_f = (e1 * d2[:, 1:2] - e2 * d1[:, 1:2]) * sgn[:, None]
    tan_v = np.zeros_like(pos, dtype=np.float64)
    for c in range(3):
        np.add.at(tan_v, tris[:, c], tan_f)
    nn = nrm.astype(np.float64)
    tan_v -= nn * (tan_v * nn).sum(1, keepdims=True)
    ln = np.linalg.norm(tan_v, axis=1, keepdims=True)
    fallback = np.cross(nn, np.where(np.abs(nn[:, :1]) < 0.9, [[1.0, 0, 0]], [[0, 1.0, 0]]))
    tan_v = np.where(ln > 1e-12, tan_v / np.maximum(ln, 1e-30), fallback / np.maximum(
        np.linalg.norm(fallback, axis=1, keepdims=True), 1e-30))
    v = np.zeros(len(pos), dtype=VERTEX_DTYPE)
    v["position"] = pos
    v["uv"] = uv
    v["normal"] = nrm
    v["color"] = 1.0
    v["tangent"] = tan_v.astype(f32)
    v["bitangent"] = np.cross(nn, tan_v).astype(f32)
    return Mesh(name, v, tris)


def quad(p0, p1, p2, p3) -> np.ndarray:
    """Two triangles (p0, p1, p2), (p0, p2, p3)."""
    return np.array([p0, p1, p2, p0, p2, p3], dtype=f32)


QUAD_UV = np.array([[0, 0], [1, 0], [1, 1], [0, 0], [1, 1], [0, 1]], dtype=f32)


def unit_box() -> Mesh:
    """Axis-aligned box [-0.5, 0.5]^3 with outward faces (12 triangles)."""
    h = 0.5
    faces = [
        quad((-h, -h, h), (h, -h, h), (h, h, h), (-h, h, h)),      # +z
        quad((h, -h, -h), (-h, -h, -h), (-h, h, -h), (h, h, -h)),  # -z
        quad((h, -h, h), (h, -h, -h), (h, h, -h), (h, h, h)),      # +x
        quad((-h, -h, -h), (-h, -h, h), (-h, h, h), (-h, h, -h)),  # -x
        quad((-h, h, h), (h, h, h), (h, h, -h), (-h, h, -h)),      # +y
        quad((-h, -h, -h), (h, -h, -h), (h, -h, h), (-h, -h, h)),  # -y
    ]
    return mesh_from_triangles("box", np.concatenate(faces), np.tile(QUAD_UV, (6, 1)))


def _cornell_room(engine: Engine, seed: int):
    scene = engine.scene
    white = engine.create_material(MaterialLambert, "cornell_white")
    white.albedo = [0.725, 0.725, 0.725, 1.0]
    red = engine.create_material(MaterialLambert, "cornell_left")
    red.albedo = [0.63, 0.065, 0.05, 1.0]
    green = engine.create_material(MaterialLambert, "cornell_right")
    green.albedo = [0.14, 0.45, 0.091, 1.0]
    light_mat = engine.create_material(MaterialLambert, "cornell_light")
    light_mat.albedo = [0.78, 0.78, 0.78, 1.0]
    light_mat.emissive = [17.0, 12.0, 4.0, 1.0]

    # walls facing into the room
    floor = quad((0, 0, 1), (1, 0, 1), (1, 0, 0), (0, 0, 0))
    ceiling = quad((0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1))
    back = quad((0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0))
    white_mesh = engine.add_mesh(mesh_from_triangles("walls", np.concatenate([floor, ceiling, back]),
                                                     np.tile(QUAD_UV, (3, 1))))
    left_mesh = engine.add_mesh(mesh_from_triangles("left", quad((0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1)), QUAD_UV))
    right_mesh = engine.add_mesh(mesh_from_triangles("right", quad((1, 0, 1), (1, 1, 1), (1, 1, 0), (1, 0, 0)), QUAD_UV))
    s = 0.125
    lq = quad((0.5 - s, 0.999, 0.5 - s), (0.5 + s, 0.999, 0.5 - s), (0.5 + s, 0.999, 0.5 + s), (0.5 - s, 0.999, 0.5 + s))
    light_mesh = engine.add_mesh(mesh_from_triangles("light", lq, QUAD_UV))
    box = engine.add_mesh(unit_box())

    for name, mesh, mat in (("walls", white_mesh, white), ("left", left_mesh, red), ("right", right_mesh, green),
                            ("light", light_mesh, light_mat)):
        so = scene.add_scene_object(name, Transform())
        so.mesh = mesh
        so.material = mat

    rng = np.random.Generator(np.random.PCG64(seed))
    # a tall box at the back left, a short box at the front right
    specs = [((0.33, 0.6, 0.35), (0.26, 0.4, 0.3), (0.55, 0.7)), ((0.68, 0.3, 0.62), (0.24, 0.34, 0.26), (0.25, 0.35))]
    for k, (center, size_rng, h_rng) in enumerate(specs):
        w = float(rng.uniform(size_rng[0], size_rng[1]))
        h = float(rng.uniform(h_rng[0], h_rng[1]))
        ang = float(rng.uniform(-30.0, 30.0))
        so = scene.add_scene_object(f"box{k}", Transform((center[0], h / 2, center[2]), (w, h, w),
                                                         (0.0, radians(ang), 0.0)))
        so.mesh = box
        so.material = white

    cam = scene.camera
    cam.transform = Transform((0.5, 0.5, 2.2))
    cam.fov = 40.0
    cam.lens_radius = 0.0
    scene.environment_type = EnvironmentType.SOLID_COLOR
    scene.background_color = [0.0, 0.0, 0.0]
    return scene


def cornell_box(seed: int = 1, width: int = 256, height: int = 256, samples: int = 64, depth: int = 8,
                batch_size: int = 4) -> tuple[Engine, RenderInfo]:
    engine = Engine()
    _cornell_room(engine, seed)
    info = RenderInfo(samples=samples, depth=depth, batch_size=batch_size, width=width, height=height,
                      filename="cornell", write_files=False)
    return engine, info


# ---------------------------------------------------------------- geodesic spheres + Perlin displacement

def icosphere(freq: int) -> tuple[np.ndarray, np.ndarray]:
    """Geodesic sphere of frequency `freq` (20 * freq^2 triangles), unit radius."""
    t = (1.0 + 5 ** 0.5) / 2.0
    V = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    F = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]])
    n = freq
    ii, jj = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    mask = ii + jj <= n
    ii, jj = ii[mask], jj[mask]
    local = {(a, b): k for k, (a, b) in enumerate(zip(ii.tolist(), jj.tolist()))}
    tri_local = []
    for a in range(n):
        for b in range(n - a):
            tri_local.append((local[(a, b)], local[(a + 1, b)], local[(a, b + 1)]))
            if a + b < n - 1:
                tri_local.append((local[(a + 1, b)], local[(a + 1, b + 1)], local[(a, b + 1)]))
    tri_local = np.array(tri_local, dtype=np.int64)
    pts, tris = [], []
    base = 0
    for f in F:
        A, B, Cc = V[f[0]], V[f[1]], V[f[2]]
        w1 = ii[:, None] / n
        w2 = jj[:, None] / n
        P = A * (1 - w1 - w2) + B * w1 + Cc * w2
        pts.append(P)
        tris.append(tri_local + base)
        base += len(P)
    P = np.concatenate(pts)
    T = np.concatenate(tris)
    P /= np.linalg.norm(P, axis=1, keepdims=True)
    # weld shared edge vertices
    key = np.round(P * 1e9).astype(np.int64)
    _, first, inv = np.unique(key, axis=0, return_index=True, return_inverse=True)
    return P[first], inv.reshape(-1)[T].astype(np.uint32)


def perlin3(p: np.ndarray, perm: np.ndarray) -> np.ndarray:
    """Ken Perlin's improved noise (2002) at points p (N x 3), value in ~[-1, 1]."""
    P = np.floor(p).astype(np.int64)
    f = p - P
    X, Y, Z = (P[:, 0] & 255), (P[:, 1] & 255), (P[:, 2] & 255)
    u = f * f * f * (f * (f * 6 - 15) + 10)

    def grad(h, x, y, z):
        h = h & 15
        uu = np.where(h < 8, x, y)
        vv = np.where(h < 4, y, np.where((h == 12) | (h == 14), x, z))
        return np.where(h & 1, -uu, uu) + np.where(h & 2, -vv, vv)

    pp = np.concatenate([perm, perm])
    A = pp[X] + Y
    AA, AB = pp[A] + Z, pp[A + 1] + Z
    B = pp[X + 1] + Y
    BA, BB = pp[B] + Z, pp[B + 1] + Z
    x, y, z = f[:, 0], f[:, 1], f[:, 2]

    def lerp(t, a, b):
        return a + t * (b - a)

    return lerp(u[:, 2],
                lerp(u[:, 1], lerp(u[:, 0], grad(pp[AA], x, y, z), grad(pp[BA], x - 1, y, z)),
                     lerp(u[:, 0], grad(pp[AB], x, y - 1, z), grad(pp[BB], x - 1, y - 1, z))),
                lerp(u[:, 1], lerp(u[:, 0], grad(pp[AA + 1], x, y, z - 1), grad(pp[BA + 1], x - 1, y, z - 1)),
                     lerp(u[:, 0], grad(pp[AB + 1], x, y - 1, z - 1), grad(pp[BB + 1], x - 1, y - 1, z - 1))))


def displaced_sphere(freq: int, radius: float, amplitude: float, noise_scale: float, rng) -> Mesh:
    P, T = icosphere(freq)
    perm = rng.permutation(256).astype(np.int64)
    off = rng.uniform(0, 100, size=3)
    d = perlin3(P * noise_scale + off, perm)
    pos = P * (radius + amplitude * d)[:, None]
    # area-weighted vertex normals of the displaced surface
    tri = pos[T.astype(np.int64)]
    fn = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    nrm = np.zeros_like(pos)
    for c in range(3):
        np.add.at(nrm, T[:, c].astype(np.int64), fn)
    nrm /= np.maximum(np.linalg.norm(nrm, axis=1, keepdims=True), 1e-30)
    uv = np.stack([0.5 + np.arctan2(P[:, 2], P[:, 0]) / (2 * math.pi), np.arccos(np.clip(P[:, 1], -1, 1)) / math.pi], 1)
    return indexed_mesh("displaced_sphere", pos, T, uv, nrm)


def random_scene(seed: int, min_tris: int = 10_000, max_tris: int = 2_000_000, max_lights: int = 4) -> Engine:
    """One scene of the batched/serving workloads: the Cornell room with
    10k-2M triangles of displaced spheres (log-uniform count), a Lambert /
    metallic-roughness mix, 0-4 extra mesh lights (the ceiling light stays) and
    a homogeneous medium of density U[0, 0.3] (none below 0.01)."""
    engine = Engine()
    scene = _cornell_room(engine, seed)
    rng = np.random.Generator(np.random.PCG64(seed + 7919))
    target = float(np.exp(rng.uniform(np.log(min_tris), np.log(max_tris))))
    n_spheres = int(rng.integers(1, 9))
    freq = max(2, int(math.ceil(math.sqrt(target / (20.0 * n_spheres)))))
    centers = []
    for k in range(n_spheres):
        r = float(rng.uniform(0.06, 0.12))
        for _ in range(200):
            c = rng.uniform([0.15, 0.1, 0.15], [0.85, 0.85, 0.85])
            if all(np.linalg.norm(c - c2) > r + r2 + 0.02 for c2, r2 in centers):
                break
        centers.append((c, r))
        mesh = engine.add_mesh(displaced_sphere(freq, 1.0, 0.04 / r, 4.0, rng))
        if rng.random() < 0.5:
            mat = engine.create_material(MaterialLambert, f"sphere_mat{k}")
            mat.albedo = [*rng.uniform(0.1, 0.9, size=3).tolist(), 1.0]
        else:
            mat = engine.create_material(MaterialPBRStandard, f"sphere_mat{k}")
            mat.albedo = [*rng.uniform(0.1, 0.9, size=3).tolist(), 1.0]
            mat.roughness = float(rng.uniform(0.05, 1.0))
            mat.metallic = float(rng.random() < 0.3)
        so = scene.add_scene_object(f"sphere{k}", Transform(tuple(c), (r, r, r)))
        so.mesh = mesh
        so.material = mat
    n_lights = int(rng.integers(0, max_lights + 1))
    lq = mesh_from_triangles("light_quad", quad((-0.5, 0, -0.5), (0.5, 0, -0.5), (0.5, 0, 0.5), (-0.5, 0, 0.5)), QUAD_UV)
    lmesh = engine.add_mesh(lq) if n_lights else None
    for k in range(n_lights):
        m = engine.create_material(MaterialLambert, f"extra_light{k}")
        m.albedo = [0.8, 0.8, 0.8, 1.0]
        m.emissive = [*rng.uniform(0.5, 1.0, size=3).tolist(), float(rng.uniform(2.0, 10.0))]
        s = float(rng.uniform(0.08, 0.2))
        # on the back wall, facing the room (+z)
        p = (float(rng.uniform(0.2, 0.8)), float(rng.uniform(0.3, 0.8)), 0.002)
        so = scene.add_scene_object(f"extra_light{k}", Transform(p, (s, s, s), (radians(90.0), 0.0, 0.0)))
        so.mesh = lmesh
        so.material = m
    density = float(rng.uniform(0.0, 0.3))
    if density >= 0.01:
        medium = engine.create_material(MaterialVolume, "room_medium")
        medium.sigma_a = [0.2 * density] * 3 + [0.0]
        medium.sigma_s = [0.8 * density] * 3 + [0.0]
        medium.g = 0.0
        boundary_mat = engine.create_material(MaterialPBRStandard, "medium_boundary")
        boundary_mat.albedo = [1.0, 1.0, 1.0, 0.0]
        boundary_mat.set_transparent(True)
        b = scene.add_scene_object("medium_boundary", Transform((0.5, 0.5, 0.5), (1.002, 1.002, 1.002)))
        b.mesh = engine.add_mesh(unit_box())
        b.material = boundary_mat
        b.volume_back = medium
    scene.background_color = [0.05, 0.05, 0.05]
    return engine


RESOLUTIONS = [(256, 256), (512, 512), (1024, 1024), (1920, 1080)]
SPPS = [16, 64, 256]


def job_mix(seed: int, n_jobs: int, n_scenes: int, distinct: bool = False) -> list[tuple[int, RenderInfo]]:
    """(scene index, render info) per job: scene drawn from a pool of n_scenes
    (or, with distinct, job j renders scene j), resolution from {256^2, 512^2,
    1024^2, 1920x1080}, spp from {16, 64, 256}."""
    rng = np.random.Generator(np.random.PCG64(seed))
    jobs = []
    for j in range(n_jobs):
        w, h = RESOLUTIONS[int(rng.integers(0, len(RESOLUTIONS)))]
        spp = SPPS[int(rng.integers(0, len(SPPS)))]
        k = int(rng.integers(0, n_scenes))
        jobs.append((j if distinct else k,
                     RenderInfo(samples=spp, depth=8, batch_size=4, width=w, height=h, filename=f"job{j}",
                                write_files=False)))
    return jobs


def env_directions(width: int, height: int) -> np.ndarray:
    """World direction of every texel centre of an equirect environment image
    under the lookup mapping (u = atan2(z, x) * 0.1591 + 0.75 wrapped,
    w = asin(y) * 0.3183 + 0.5): H x W x 3."""
    u = (np.arange(width) + 0.5) / width
    w = (np.arange(height) + 0.5) / height
    x = np.mod(u - 0.25, 1.0)
    lon = (x - 0.5) / 0.1591
    lat = np.clip((w - 0.5) / 0.3183, -math.pi / 2, math.pi / 2)
    lat, lon = np.meshgrid(lat, lon, indexing="ij")
    return np.stack([np.cos(lat) * np.cos(lon), np.sin(lat), np.cos(lat) * np.sin(lon)], -1)


def procedural_sky(width: int = 4096, height: int = 2048, sun_dir=(0.4, 0.55, -0.35), sun_peak: float = 5.0e4,
                   sun_sigma_deg: float = 0.8, zenith=(0.25, 0.45, 0.9), horizon=(0.9, 0.85, 0.8),
                   ground=(0.25, 0.22, 0.2)) -> np.ndarray:
    """RGBA32F equirect sky: a vertical gradient (ground below the horizon,
    horizon to zenith above) plus a Gaussian sun of angular sigma
    `sun_sigma_deg` and peak radiance `sun_peak` (warm white)."""
    d = env_directions(width, height)
    y = d[..., 1:2]
    t = np.clip(y, 0.0, 1.0) ** 0.5
    sky = np.where(y >= 0.0, np.asarray(horizon) * (1 - t) + np.asarray(zenith) * t, np.asarray(ground))
    sd = np.asarray(sun_dir, dtype=np.float64)
    sd = sd / np.linalg.norm(sd)
    ang = np.arccos(np.clip(d @ sd, -1.0, 1.0))
    sig = math.radians(sun_sigma_deg)
    sun = sun_peak * np.exp(-0.5 * (ang / sig) ** 2)[..., None] * np.asarray([1.0, 0.95, 0.85])
    rgb = sky + sun
    return np.concatenate([rgb, np.ones_like(rgb[..., :1])], -1).astype(np.float32)


def sky_scene(seed: int = 1, width: int = 96, height: int = 64, samples: int = 16, depth: int = 8,
              batch_size: int = 4, sky_w: int = 512, sky_h: int = 256, sun_peak: float = 5.0e3,
              sun_sigma_deg: float = 2.0) -> tuple[Engine, RenderInfo]:
    """Displaced spheres on a ground quad under a procedural sky with a small
    bright sun (background mode 1): the case environment importance sampling
    is for."""
    engine = Engine()
    scene = engine.scene
    rng = np.random.Generator(np.random.PCG64(seed))
    ground = engine.create_material(MaterialLambert, "ground")
    ground.albedo = [0.6, 0.6, 0.6, 1.0]
    gq = mesh_from_triangles("ground", quad((-4, 0, -4), (4, 0, -4), (4, 0, 4), (-4, 0, 4)), QUAD_UV)
    so = scene.add_scene_object("ground", Transform((0, 0, 0)))
    so.mesh = engine.add_mesh(gq)
    so.material = ground
    for k in range(3):
        mesh = engine.add_mesh(displaced_sphere(6, 1.0, 0.05, 3.0, rng))
        if k == 1:
            mat = engine.create_material(MaterialPBRStandard, f"ball{k}")
            mat.albedo = [0.8, 0.6, 0.3, 1.0]
            mat.roughness = 0.3
            mat.metallic = 1.0
        else:
            mat = engine.create_material(MaterialLambert, f"ball{k}")
            mat.albedo = [*rng.uniform(0.2, 0.9, size=3).tolist(), 1.0]
        b = scene.add_scene_object(f"ball{k}", Transform((-1.2 + 1.2 * k, 0.5, 0.0), (0.5, 0.5, 0.5)))
        b.mesh = mesh
        b.material = mat
    scene.camera.transform = Transform((0.0, 1.2, 4.0), (1, 1, 1), (math.radians(-12.0), 0.0, 0.0))
    scene.environment_map = procedural_sky(sky_w, sky_h, sun_peak=sun_peak, sun_sigma_deg=sun_sigma_deg)
    scene.environment_type = EnvironmentType.HDRI
    scene.environment_intensity = 1.0
    info = RenderInfo(samples=samples, depth=depth, batch_size=batch_size, width=width, height=height,
                      filename="sky", write_files=False)
    return engine, info


def instanced_sky_scene(seed: int = 1, width: int = 3840, height: int = 2160, samples: int = 16, depth: int = 8,
                        batch_size: int = 4, n_meshes: int = 8, n_instances: int = 512, freq: int = 45,
                        n_lights: int = 32, sky_w: int = 4096, sky_h: int = 2048) -> tuple[Engine, RenderInfo]:
    """Open scene under a procedural sky: `n_instances` random rigid placements
    (rotation about a random axis, translation) of `n_meshes` seeded
    displaced spheres of 20 * freq^2 triangles (8 x 40,500 = 324,000 unique,
    512 instances = 20,736,000 instanced triangles), a ground quad, `n_lights`
    emissive quads as mesh lights, a thin lens of radius 0.02, and a
    4096 x 2048 sky (gradient plus a Gaussian sun of peak 5e4)."""
    engine = Engine()
    scene = engine.scene
    rng = np.random.Generator(np.random.PCG64(seed))
    ground = engine.create_material(MaterialLambert, "ground")
    ground.albedo = [0.45, 0.42, 0.38, 1.0]
    gq = mesh_from_triangles("ground", quad((-40, 0, -40), (40, 0, -40), (40, 0, 40), (-40, 0, 40)), QUAD_UV)
    so = scene.add_scene_object("ground", Transform((0, 0, 0)))
    so.mesh = engine.add_mesh(gq)
    so.material = ground
    meshes, radii = [], []
    for k in range(n_meshes):
        r = float(rng.uniform(0.5, 1.2))
        meshes.append(engine.add_mesh(displaced_sphere(freq, r, 0.08 * r, 2.5, rng)))
        radii.append(r)
    mats = []
    for k in range(8):
        if k % 2 == 0:
            m = engine.create_material(MaterialLambert, f"diffuse{k}")
        else:
            m = engine.create_material(MaterialPBRStandard, f"pbr{k}")
            m.roughness = float(rng.uniform(0.05, 0.8))
            m.metallic = float(rng.random() < 0.4)
        m.albedo = [*rng.uniform(0.15, 0.9, size=3).tolist(), 1.0]
        mats.append(m)
    for i in range(n_instances):
        k = int(rng.integers(0, n_meshes))
        axis = rng.normal(size=3)
        axis /= np.linalg.norm(axis)
        ang = float(rng.uniform(0, 2 * math.pi))
        q = (math.cos(ang / 2), *(math.sin(ang / 2) * axis).tolist())
        pos = (float(rng.uniform(-30, 30)), radii[k] * 1.02, float(rng.uniform(-30, 30)))
        o = scene.add_scene_object(f"inst{i}", Transform(pos, (1, 1, 1), q))
        o.mesh = meshes[k]
        o.material = mats[int(rng.integers(0, len(mats)))]
    lq = engine.add_mesh(mesh_from_triangles("light_quad", quad((-0.5, 0, -0.5), (0.5, 0, -0.5), (0.5, 0, 0.5),
                                                                (-0.5, 0, 0.5)), QUAD_UV))
    for k in range(n_lights):
        m = engine.create_material(MaterialLambert, f"lamp{k}")
        m.albedo = [0.8, 0.8, 0.8, 1.0]
        m.emissive = [*rng.uniform(0.6, 1.0, size=3).tolist(), float(rng.uniform(20.0, 80.0))]
        pos = (float(rng.uniform(-25, 25)), float(rng.uniform(2.5, 4.0)), float(rng.uniform(-25, 25)))
        o = scene.add_scene_object(f"lamp{k}", Transform(pos, (0.6, 0.6, 0.6), (math.pi, 0.0, 0.0)))
        o.mesh = lq
        o.material = m
    cam = scene.camera
    cam.transform = Transform((0.0, 6.0, 34.0), (1, 1, 1), (math.radians(-10.0), 0.0, 0.0))
    cam.lens_radius = 0.02
    cam.focal_distance = 30.0
    scene.environment_map = procedural_sky(sky_w, sky_h, sun_peak=5.0e4, sun_sigma_deg=0.5)
    scene.environment_type = EnvironmentType.HDRI
    scene.environment_intensity = 1.0
    info = RenderInfo(samples=samples, depth=depth, batch_size=batch_size, width=width, height=height,
                      filename="instanced_sky", write_files=False)
    return engine, info


SERVING_RESOLUTIONS = [(256, 256), (512, 512)]
SERVING_SPPS = [8, 16, 32]


def serving_requests(seed: int, n_requests: int, n_scenes: int, mean_gap_ms: float = 50.0, preview: bool = False):
    """(arrival ms, scene index, render info) per request: Poisson arrivals
    (exponential gaps, mean `mean_gap_ms`), scenes from the pool of the
    batched workload, resolution and spp drawn as in the batched workload
    ({256^2, 512^2, 1024^2, 1920x1080}, {16, 64, 256}: about 94M paths per
    request, an offered load far above one GPU, so requests queue for
    admission), or with `preview` from {256^2, 512^2} and {8, 16, 32}."""
    rng = np.random.Generator(np.random.PCG64(seed))
    gaps = rng.exponential(mean_gap_ms, n_requests)
    t = np.cumsum(gaps) - gaps[0]
    res, spps = (SERVING_RESOLUTIONS, SERVING_SPPS) if preview else (RESOLUTIONS, SPPS)
    out = []
    for j in range(n_requests):
        w, h = res[int(rng.integers(0, len(res)))]
        spp = spps[int(rng.integers(0, len(spps)))]
        out.append((float(t[j]), int(rng.integers(0, n_scenes)),
                    RenderInfo(samples=spp, depth=8, batch_size=4, width=w, height=h, filename=f"req{j}",
                               write_files=False)))
    return out


def cornell_medium(seed: int = 1, width: int = 1920, height: int = 1080, samples: int = 256, depth: int = 12,
                   batch_size: int = 4, freq: int = 79, spheres: int = 8) -> tuple[Engine, RenderInfo]:
    engine = Engine()
    scene = _cornell_room(engine, seed)
    rng = np.random.Generator(np.random.PCG64(seed + 1000))
    medium = engine.create_material(MaterialVolume, "room_medium")
    medium.sigma_a = [0.05, 0.05, 0.05, 0.0]
    medium.sigma_s = [0.2, 0.2, 0.2, 0.0]
    medium.g = 0.0
    boundary_mat = engine.create_material(MaterialPBRStandard, "medium_boundary")
    boundary_mat.albedo = [1.0, 1.0, 1.0, 0.0]
    boundary_mat.set_transparent(True)
    bmesh = engine.add_mesh(unit_box())
    b = scene.add_scene_object("medium_boundary", Transform((0.5, 0.5, 0.5), (1.002, 1.002, 1.002)))
    b.mesh = bmesh
    b.material = boundary_mat
    b.volume_back = medium

    centers = []
    for k in range(spheres):
        r = float(rng.uniform(0.07, 0.11))
        for _ in range(200):
            c = rng.uniform([0.15, 0.1, 0.15], [0.85, 0.85, 0.85])
            if all(np.linalg.norm(c - c2) > r + r2 + 0.03 for c2, r2 in centers):
                break
        centers.append((c, r))
        mesh = engine.add_mesh(displaced_sphere(freq, 1.0, 0.05 / r, 4.0, rng))
        mat = engine.create_material(MaterialPBRStandard, f"sphere_mat{k}")
        mat.albedo = [*rng.uniform(0.1, 0.9, size=3).tolist(), 1.0]
        mat.roughness = float(rng.uniform(0.05, 1.0))
        mat.metallic = float(rng.random() < 0.3)
        so = scene.add_scene_object(f"sphere{k}", Transform(tuple(c), (r, r, r)))
        so.mesh = mesh
        so.material = mat
    info = RenderInfo(samples=samples, depth=depth, batch_size=batch_size, width=width, height=height,
                      filename="cornell_medium", write_files=False)
    return engine, info
