"""The reference's render-test scenes (src/bin/unittests/RenderTests.cpp) that
can be rebuilt from assets present in the reference tree, with their golden
images and MSE tolerances.

Each builder returns (engine, render_info, tolerance). State the reference's
tests carry from one test to the next (render depth 9, background colour of
the previous test) is applied explicitly.
"""
from __future__ import annotations

from functools import lru_cache
from pathlib import Path

import numpy as np

from vviewer_gb300.assets import mesh_from_obj_arrays, rgbe_decode
from vviewer_gb300.renderer import RenderInfo
from vviewer_gb300.scene import (EnvironmentType, Engine, LightType, MaterialLambert, MaterialPBRStandard,
                                 MaterialVolume, PerspectiveCamera, Transform, radians)

ASSETS = Path(__file__).resolve().parent / "golden" / "reference_assets.npz"


@lru_cache(maxsize=1)
def _assets():
    return dict(np.load(ASSETS))


def golden(name: str) -> np.ndarray:
    """Decoded golden image (H x W x 3 float32)."""
    return rgbe_decode(_assets()[f"golden_{name}"])


def golden_rgbe(name: str) -> np.ndarray:
    return _assets()[f"golden_{name}"]


def _mesh(engine: Engine, model: str):
    a = _assets()
    m = mesh_from_obj_arrays(str(a[f"{model}_name"]), a[f"{model}_v"], a[f"{model}_vt"], a[f"{model}_vn"],
                             a[f"{model}_f"].reshape(-1, 3))
    return engine.add_mesh(m)


def _info(name: str, batch: int = 64, samples: int = 2048) -> RenderInfo:
    # depth is never set by the render tests: RenderInfo's default of 9
    return RenderInfo(samples=samples, depth=9, batch_size=batch, width=256, height=256, filename=name + "_test",
                      write_files=False)


def _camera(pos, euler=(0.0, 0.0, 0.0), fov=60.0) -> PerspectiveCamera:
    c = PerspectiveCamera()
    c.transform.position = np.asarray(pos, dtype=np.float32)
    c.transform.set_rotation(euler)
    c.fov = fov
    return c


def furnace(lambert: bool):
    """RenderTests.cpp:74-154"""
    e = Engine()
    s = e.scene
    cam = _camera((0, 0, 2))
    cam.lens_radius = 0.0
    cam.focal_distance = 0.0
    s.camera = cam
    so = s.add_scene_object("sphere", Transform((0, 0, 0), (1, 1, 1)))
    so.mesh = _mesh(e, "uvsphere")
    if lambert:
        m = e.create_material(MaterialLambert, "lambertmaterial1")
    else:
        m = e.create_material(MaterialPBRStandard, "pbrmaterial1")
    m.albedo = [0.6, 0.6, 0.6, 1.0]
    so.material = m
    s.environment_intensity = 1.0
    s.environment_type = EnvironmentType.SOLID_COLOR
    s.background_color = [1.0, 1.0, 1.0]
    return e, _info("FurnaceLambert" if lambert else "FurnacePBR"), 1e-6


def _volume_scene(second: bool):
    """RenderTests.cpp:309-364 (Volume1) and :441-504 (Volume2)."""
    e = Engine()
    s = e.scene
    if second:
        cam = _camera((0, 1.0, 7))
        cam.zfar = 10.0
    else:
        cam = _camera((0, 0.5, 4))
    s.camera = cam
    sphere = _mesh(e, "uvsphere")  # loaded by the test, unused
    cube = _mesh(e, "cube")
    plane = _mesh(e, "plane")
    e.create_material(MaterialLambert, "lambertmaterial")
    pbr = e.create_material(MaterialPBRStandard, "pbrmaterial")
    pbr.set_transparent(True)
    pbr.albedo = [1.0, 1.0, 1.0, 0.2]
    pbr.metallic = 0.0
    pbr.roughness = 0.0
    vol1 = e.create_material(MaterialVolume, "volumematerial1")
    vol2 = e.create_material(MaterialVolume, "volumematerial2") if second else None
    c = s.add_scene_object("cube1", Transform((0, 0.5, 0), (1, 1, 1)))
    c.mesh = cube
    c.material = pbr
    c.volume_back = vol1
    if second:
        c.volume_front = vol2
    p = s.add_scene_object("plane", Transform((0, -1, 0), (10, 10, 10)))
    p.mesh = plane
    p.material = e.material("defaultMaterial")
    if second:
        vol1.sigma_a = [0.2, 0.4, 0.0, 0.0]
        vol1.sigma_s = [0.8, 0.4, 0.2, 0.0]
        vol2.sigma_a = [0.04, 0.04, 0.04, 0.0]
        vol2.sigma_s = [0.04, 0.04, 0.04, 0.0]
        vol1.g = 0.0
        vol2.g = 0.0
        cam.volume = vol2
    else:
        vol1.sigma_a = [0.2, 0.4, 0.8, 0.0]
        vol1.sigma_s = [0.8, 0.4, 0.2, 0.0]
        vol1.g = 0.0
    s.environment_intensity = 1.0
    s.environment_type = EnvironmentType.SOLID_COLOR
    s.background_color = [0.0, 0.0, 0.0]
    del sphere
    return e, plane


def volume(case: int):
    """Volume3/4/5 (first volume test) and Volume7/8/9 (second): directional
    light, point light, then mesh light."""
    second = case >= 7
    e, plane = _volume_scene(second)
    s = e.scene
    kind = case - (7 if second else 3)
    so = s.add_scene_object("light", Transform((0, 4, 0), (1, 1, 1), (radians(45.0), radians(90.0), 0.0)))
    if kind == 0:
        light = e.create_light("Directional light 1", LightType.DIRECTIONAL_LIGHT)
        light.color[3] = 1.0
        so.light = light
        tol = 8e-6
    elif kind == 1:
        light = e.create_light("Point light 1", LightType.POINT_LIGHT)
        light.color[3] = 15.0
        so.light = light
        tol = 8e-6
    else:
        em = e.create_material(MaterialPBRStandard, "emissivepbrmaterial")
        em.emissive = [0.3, 0.3, 0.7, 15.0]
        so.set_local_transform(Transform((0, 1.5, -3), (1, 1, 1), (radians(90.0), radians(0.0), 0.0)))
        so.mesh = plane
        so.material = em
        tol = 1e-5
    return e, _info(f"Volume{case}"), tol


def _two_balls(e: Engine):
    """PrepareTwoBallsOnPlaneScene, RenderTests.cpp:35-72."""
    s = e.scene
    pbr = e.create_material(MaterialPBRStandard, "pbrmaterial6")
    lam = e.create_material(MaterialLambert, "lambertmaterial6")
    floor = e.create_material(MaterialLambert, "lambertmaterial7")
    pbr.albedo = [0.7, 0.1, 0.1, 1.0]
    pbr.roughness = 0.3
    lam.albedo = [0.1, 0.7, 0.1, 1.0]
    s.camera = _camera((0, 1, 4))
    sphere = _mesh(e, "uvsphere")
    plane = _mesh(e, "plane")
    _mesh(e, "cube")
    a = s.add_scene_object("sphere", Transform((-1, 1, 0), (1, 1, 1)))
    a.mesh, a.material = sphere, pbr
    b = s.add_scene_object("sphere", Transform((1, 1, 0), (1, 1, 1)))
    b.mesh, b.material = sphere, lam
    p = s.add_scene_object("plane", Transform((0, 0, 0), (10, 10, 10)))
    p.mesh, p.material = plane, floor
    s.environment_intensity = 1.0
    s.environment_type = EnvironmentType.SOLID_COLOR
    s.background_color = [0.0, 0.0, 0.0]
    return plane


def point_light():
    """RenderTests.cpp:567-602"""
    e = Engine()
    _two_balls(e)
    light = e.create_light("Point light", LightType.POINT_LIGHT)
    light.color[3] = 10.0
    so = e.scene.add_scene_object("Point light", Transform((0, 4, 0)))
    so.light = light
    return e, _info("PointLight"), 1e-8


def directional_light():
    """RenderTests.cpp:604-641"""
    e = Engine()
    _two_balls(e)
    light = e.create_light("Directional light", LightType.DIRECTIONAL_LIGHT)
    light.color[3] = 1.0
    so = e.scene.add_scene_object("Directional light",
                                  Transform((0, 0, 0), (1, 1, 1), (radians(45.0), radians(90.0), 0.0)))
    so.light = light
    return e, _info("DirectionalLight"), 1e-8


def mesh_light():
    """RenderTests.cpp:643-689"""
    e = Engine()
    plane = _two_balls(e)
    so = e.scene.add_scene_object("Mesh light", Transform((0, 2, 0), (0.4, 0.4, 0.4), (radians(90.0), radians(0.0), 0.0)))
    so.mesh = plane
    em = e.create_material(MaterialPBRStandard, "emissivepbrmaterial3")
    em.emissive = [0.3, 0.3, 0.7, 15.0]
    so.material = em
    cam = e.scene.camera
    cam.transform.position = np.array([0, 3, 5], dtype=np.float32)
    cam.transform.set_rotation((radians(-20.0), 0.0, 0.0))
    return e, _info("MeshLight"), 1e-8


def shared_components():
    """RenderTests.cpp:969-1031. The background colour carries over from the
    Hierarchy test before it: (0, 0, 0)."""
    e = Engine()
    s = e.scene
    s.camera = _camera((0, 20, 50), (radians(-15.0), radians(90.0), 0.0))
    cube = _mesh(e, "cube")
    mat = e.material("defaultMaterial")
    s.add_scene_object("root", Transform())
    for i in range(-150, 150, 3):
        for j in range(-150, 150, 3):
            so = s.add_scene_object(f"cube{i}{j}", Transform((i, 0, j), (1, 1, 1)))
            so.mesh = cube
            so.material = mat
    so = s.add_scene_object("directionalLight", Transform((0, 2, 0), (1, 1, 1), (radians(45.0), radians(90.0), 0.0)))
    so.light = e.light("defaultDirectionalLightSun")
    s.environment_type = EnvironmentType.SOLID_COLOR
    s.environment_intensity = 0.0
    s.background_color = [0.0, 0.0, 0.0]
    return e, _info("SharedComponents", batch=4), 1e-6


BUILDERS = {
    "FurnacePBR": lambda: furnace(False),
    "FurnaceLambert": lambda: furnace(True),
    "PointLight": point_light,
    "DirectionalLight": directional_light,
    "MeshLight": mesh_light,
    "Volume3": lambda: volume(3),
    "Volume4": lambda: volume(4),
    "Volume5": lambda: volume(5),
    "Volume7": lambda: volume(7),
    "Volume8": lambda: volume(8),
    "Volume9": lambda: volume(9),
    "SharedComponents": shared_components,
}


def compare_images(test_rgb: np.ndarray, ref_rgb: np.ndarray) -> float:
    """CompareImages (RenderTests.cpp:7-33): MSE over the three channels."""
    d = test_rgb[..., :3].astype(np.float64) - ref_rgb[..., :3].astype(np.float64)
    return float((d * d).mean())


ORDERS = Path(__file__).resolve().parent / "golden" / "meshlight_orders.npz"
# Scenes whose golden depends on the order in which the hardware reported the
# any-hit candidates of BSDF-direction emitter rays (rayNEE.rahit.glsl:43-131):
# the emissive plane of MeshLight cuts into the glossy sphere, so rays that
# reach the plane can also hit the sphere behind it, and the reference keeps
# whichever candidate its traversal reported first. Data: the oracle's
# full-image renders in the two end orders (tests/golden/make_meshlight_orders.py).
ORDER_DEPENDENT = {"MeshLight"}


@lru_cache(maxsize=1)
def _orders():
    z = np.load(ORDERS)
    return z["pixels"].astype(np.int64), z["nearest"], z["alt"]


def order_dependent_pixels(name: str):
    """(pixel indices, nearest-first values, instance-order values) of the
    pixels whose radiance depends on the emitter rays' candidate order, or
    None for scenes where no pixel does."""
    return _orders() if name in ORDER_DEPENDENT else None


def golden_check_with_orders(name: str, radiance_rgb: np.ndarray, alt_rgb: np.ndarray | None = None):
    """Compares a render (H x W x 3, nearest-first candidate order) with the
    golden. Returns (mse_outside, bracketed, mse_bracket):
      mse_outside: the reference's CompareImages MSE summed over the pixels
        whose value does not depend on the candidate order (normalised by the
        full image, so it is the full-image MSE when no pixel depends on it);
      bracketed: fraction of the order-dependent pixel channels whose golden
        value lies between this render and the instance-order render, within
        one RGBE quantisation step of the golden;
      mse_bracket: how far the golden lies outside that bracket, as a
        full-image MSE.
    alt_rgb (H x W x 3) overrides the stored instance-order values."""
    from vviewer_gb300.assets import rgbe_encode

    h, w = radiance_rgb.shape[:2]
    gold_rgbe = golden_rgbe(name).reshape(-1, 4)
    gold = rgbe_decode(gold_rgbe).astype(np.float64)
    q = rgbe_decode(rgbe_encode(radiance_rgb.reshape(-1, 3).astype(np.float32))).astype(np.float64)
    total = h * w * 3
    dep = order_dependent_pixels(name)
    mask = np.zeros(h * w, dtype=bool)
    if dep is None:
        return float(((q - gold) ** 2).sum() / total), 1.0, 0.0
    pix, _, alt = dep
    if alt_rgb is not None:
        alt = alt_rgb.reshape(-1, 3)[pix]
    mask[pix] = True
    mse_outside = float(((q - gold) ** 2)[~mask].sum() / total)
    qa = rgbe_decode(rgbe_encode(np.asarray(alt, dtype=np.float32))).astype(np.float64)
    lo = np.minimum(q[pix], qa)
    hi = np.maximum(q[pix], qa)
    e = gold_rgbe[pix, 3].astype(np.int32)
    step = np.where(e != 0, np.ldexp(1.0, e - 136), 0.0)[:, None]
    g = gold[pix]
    bracketed = float(((g >= lo - step) & (g <= hi + step)).mean())
    mse_bracket = float(((g - np.clip(g, lo, hi)) ** 2).sum() / total)
    return mse_outside, bracketed, mse_bracket
