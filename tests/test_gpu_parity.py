"""GPU parity: the sm_103a kernels through the C ABI against the CPU oracle
and against the reference's golden images.

Tolerances:
  * closest hit: instance, primitive, t, u, v bit-identical (integer/index
    work and an exactly rounded triangle test);
  * renders vs the oracle (same RTGEMS stream, FP32 path arithmetic): image
    mean within 1e-4 relative, >= 95% of pixels within 1e-3 relative, and the
    remaining pixels within Monte Carlo noise (|z| > 4 on < 0.5%);
  * renders vs the reference goldens: the reference's own MSE tolerance
    (CompareImages, src/bin/unittests/RenderTests.cpp:7-33).
"""
import ctypes as C

import numpy as np
import pytest

import reference_scenes as R
from raygen import HIT_SCENES, make_near_rays, make_rays
from oracle import oracle
from vviewer_gb300 import _native as N
from vviewer_gb300 import scenes
from vviewer_gb300.assets import rgbe_decode, rgbe_encode
from vviewer_gb300.renderer import RenderInfo
from vviewer_gb300.scene import EnvironmentType, Engine, MaterialLambert, Transform

pytestmark = pytest.mark.gpu
N_BVH_AUTO, N_BVH_HOST, N_BVH_GPU = 0, 1, 2


def assert_hits_equal(hg, ho):
    for f in ("instance", "primitive", "t", "u", "v"):
        eq = hg[f] == ho[f]
        assert eq.all(), f"{f}: {np.count_nonzero(~eq)} of {len(eq)} differ, first {np.nonzero(~eq)[0][:5]}"




@pytest.mark.parametrize("name", list(HIT_SCENES))
def test_closest_hit_bit_exact(ctx, name):
    build, (lo, hi) = HIT_SCENES[name]
    fs = build().scene.build()
    g = ctx.upload(fs)
    rays = make_rays(fs, 200_000 if name != "shared_components" else 50_000, 7, lo, hi)
    rays = np.concatenate([rays, make_near_rays(fs, 50_000, 11)])
    hg = g.trace_closest(rays)
    ho = oracle.trace_closest(fs, rays)
    assert (hg["instance"] != 0xFFFFFFFF).mean() > 0.3
    assert_hits_equal(hg, ho)
    g.release()


def test_closest_hit_empty_and_degenerate(ctx):
    e = Engine()
    s = e.scene
    so = s.add_scene_object("light", Transform((0, 1, 0)))
    so.light = e.light("defaultPointLight")
    fs = s.build()
    g = ctx.upload(fs)
    rays = np.array([[0, 0, 0, 0, 0, 0, 1, 10], [0, 0, 0, 0, 1, 0, 0, 10]], dtype=np.float32)
    h = g.trace_closest(rays)
    assert (h["instance"] == 0xFFFFFFFF).all()
    g.release()


def compare_renders(a, b, m2a, batches):
    a = a[..., :3].astype(np.float64)
    b = b[..., :3].astype(np.float64)
    rel_mean = abs(a.mean() - b.mean()) / max(b.mean(), 1e-12)
    close = np.isclose(a, b, rtol=1e-3, atol=1e-7).all(-1)
    var = np.maximum(batches * m2a[..., :3].astype(np.float64) - a * a, 0.0) / max(batches - 1, 1)
    z = np.abs(a - b) / np.sqrt(2.0 * var + 1e-20)
    # pixels that neither agree to float noise nor lie within Monte Carlo noise
    outliers = (~close) & (z > 4).any(-1)
    return rel_mean, close.mean(), outliers.mean()


def render_pair(ctx, engine, info, env_is=False, sampler="rtgems", **kw):
    fs = engine.scene.build()
    sd = engine.scene.scene_data(info.width, info.height)
    g = ctx.upload(fs)
    res = g.render(sd, info, want_m2=True, env_is=env_is, sampler=sampler)
    g.release()
    ref = oracle.render(fs, sd, info, env_is=env_is, sampler=sampler, **kw)
    return res, ref


def test_cornell_render_matches_oracle(ctx):
    e, info = scenes.cornell_box(1, 128, 128, 64, 8, 4)
    res, ref = render_pair(ctx, e, info)
    rel, close, z4 = compare_renders(res.radiance, ref["radiance"], res.radiance_m2, info.samples // info.batch_size)
    assert rel < 1e-4 and close >= 0.95 and z4 < 0.005, (rel, close, z4)
    assert (res.albedo == ref["albedo"]).all(-1).mean() >= 0.99
    assert (res.normal == ref["normal"]).all(-1).mean() >= 0.99
    assert res.stats.paths == 128 * 128 * 64
    assert res.stats.kernel_launches > 0


def test_medium_scene_matches_oracle(ctx):
    """The headline scene at its full geometry: the Cornell room filled with
    the medium and eight displaced spheres at frequency 79 (998,560
    triangles), depth 12, at a small resolution, with the Cornell box's
    bounds."""
    e, info = scenes.cornell_medium(2, 96, 54, 16, 12, 4, freq=79, spheres=8)
    res, ref = render_pair(ctx, e, info)
    rel, close, z4 = compare_renders(res.radiance, ref["radiance"], res.radiance_m2, info.samples // info.batch_size)
    assert rel < 1e-4 and close >= 0.95 and z4 < 0.005, (rel, close, z4)


def _mean_and_se(img, m2, nb):
    # the image is the sum of nb batch contributions; m2 sums their squares
    x = img[..., :3].astype(np.float64)
    var = np.maximum(nb * m2[..., :3].astype(np.float64) - x * x, 0.0) / max(nb - 1, 1)
    return x, np.sqrt(var)


def test_converged_medium_scene_matches_fp64_oracle(ctx):
    """The benchmark spec's converged-image criterion on the headline scene
    (medium, eight displaced spheres of 124,820 triangles each, depth 12),
    through a 12-degree view of spheres and walls at 3 x 2 pixels: the GPU at
    2^26 samples per pixel (batches of 512, so its random streams differ from
    the reference's) against the oracle's FP64-accumulated render at 2^25
    (tests/golden/make_medium_converged.py; minutes of CPU, so a fixture).
    Every pixel channel within 3 Monte Carlo standard errors of the
    difference (4 allowed on one of the 18), and the relative RMSE of the
    GPU image against the FP64 one, sqrt(sum (a - b)^2 / sum b^2), at most
    1e-3."""
    import importlib.util
    from pathlib import Path
    spec = importlib.util.spec_from_file_location(
        "make_medium_converged", Path(__file__).resolve().parent / "golden" / "make_medium_converged.py")
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    ref = np.load(Path(__file__).resolve().parent / "golden" / "medium_converged.npz")
    e, info = gen.scene(1 << 26, 512)
    fs = e.scene.build()
    sd = e.scene.scene_data(info.width, info.height)
    g = ctx.upload(fs)
    res = g.render(sd, info, want_m2=True)
    g.release()
    a, sa = gen.mean_and_se(res.radiance, res.radiance_m2, info.samples // info.batch_size)
    b, sb = ref["mean"], ref["se"]
    z = np.abs(a - b) / np.sqrt(sa ** 2 + sb ** 2 + 1e-30)
    rel_rmse = float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))
    assert (z <= 3.0).sum() >= z.size - 1 and z.max() <= 4.0, np.sort(z.ravel())[-4:]
    assert rel_rmse <= 1e-3, rel_rmse


def test_gltf_model_scene_matches_oracle(ctx, tmp_path):
    """A glTF model (indexed meshes, a node tree, an RGBA base colour texture
    with cut-outs, metallic-roughness, occlusion and normal maps, an emissive
    quad) placed twice in the Cornell room through addModel3D."""
    from gltf_files import textured_panel_model
    from vviewer_gb300.model3d import add_model3d, import_model

    e, info = scenes.cornell_box(3, 96, 72, 32, 8, 4)
    model = import_model(e, textured_panel_model(tmp_path, "glb"), name="panel")
    add_model3d(e.scene, None, model, Transform((0.5, 0.45, 0.45), (0.5, 0.5, 0.5)))
    add_model3d(e.scene, None, model, Transform((0.3, 0.25, 0.7), (0.3, 0.3, 0.3), (0.0, 0.6, 0.0)))
    res, ref = render_pair(ctx, e, info)
    rel, close, z4 = compare_renders(res.radiance, ref["radiance"], res.radiance_m2, info.samples // info.batch_size)
    assert rel < 1e-3 and close >= 0.9 and z4 < 0.01, (rel, close, z4)
    # textured first-hit albedo: bilinear sRGB lookups agree to rounding
    assert np.isclose(res.albedo, ref["albedo"], rtol=1e-5, atol=1e-6).all(-1).mean() >= 0.99


def _scene_file(folder):
    """A vviewer scene file (core/io/Import.cpp's format) and everything it
    names: an OBJ model with an .mtl library (two materials, one with a PNG
    albedo texture), a closed OBJ cube, a glTF model with its EMBEDDED
    materials, LAMBERT / PBR_STANDARD / VOLUME materials, point and
    directional lights, an emissive mesh light, a medium inside a transparent
    boundary, an HDR environment, and a thin-lens camera given by target and
    up."""
    import json

    from gltf_files import textured_panel_model
    from vviewer_gb300.assets import write_hdr
    from vviewer_gb300.renderer import write_png

    a = R._assets()
    V, VT, VN, F = a["cube_v"], a["cube_vt"], a["cube_vn"], a["cube_f"].reshape(-1, 3, 3)
    head = [f"v {x:.6f} {y:.6f} {z:.6f}" for x, y, z in V] + [f"vt {u:.6f} {v:.6f}" for u, v in VT] + \
        [f"vn {x:.6f} {y:.6f} {z:.6f}" for x, y, z in VN]

    def faces(tris):
        return [f"f {' '.join('/'.join(str(int(i)) for i in c) for c in t)}" for t in tris]

    half = F.shape[0] // 2
    (folder / "crate.obj").write_text("\n".join(["mtllib crate.mtl", "o Crate"] + head + ["usemtl paint"] +
                                                 faces(F[:half]) + ["usemtl lacquer"] + faces(F[half:])) + "\n")
    (folder / "box.obj").write_text("\n".join(["o Box"] + head + faces(F)) + "\n")
    stripes = np.zeros((8, 8, 3), dtype=np.uint8)
    stripes[:, ::2] = [220, 180, 60]
    stripes[:, 1::2] = [40, 90, 200]
    write_png(folder / "stripes.png", stripes)
    (folder / "crate.mtl").write_text("newmtl paint\nKd 0.9 0.9 0.9\nKs 0.1 0.1 0.1\nNs 30\nmap_Kd stripes.png\n"
                                      "newmtl lacquer\nKd 0.2 0.5 0.3\nKs 0.6 0.6 0.6\nNs 85\n")
    textured_panel_model(folder, "glb")
    sky = scenes.procedural_sky(64, 32, sun_peak=4.0, sun_sigma_deg=15.0)
    write_hdr(folder / "sky.hdr", sky)
    doc = {
        "camera": {"position": [0.0, 1.1, 3.4], "target": [0.0, 0.5, 0.0], "up": [0, 1, 0], "fov": 55.0,
                   "lensRadius": 0.01, "focalDistance": 3.3},
        "models": [{"name": "crate", "filepath": "crate.obj"}, {"name": "box", "filepath": "box.obj"},
                   {"name": "panel", "filepath": "panel.glb"}],
        "materials": [
            {"name": "floor", "type": "LAMBERT", "albedo": {"value": [0.55, 0.55, 0.5, 1.0]}},
            {"name": "metal", "type": "PBR_STANDARD", "albedo": {"value": [0.9, 0.6, 0.3, 1.0]},
             "metallic": {"value": 1.0}, "roughness": {"value": 0.35}},
            {"name": "fog", "type": "VOLUME", "absorption": {"value": [0.05, 0.06, 0.08]},
             "scattering": {"value": [0.1, 0.1, 0.08]}, "g": 0.3},
            {"name": "shell", "type": "PBR_STANDARD", "albedo": {"value": [1.0, 1.0, 1.0, 0.0]}, "transparent": True},
            {"name": "lamp", "type": "LAMBERT", "albedo": {"value": [1.0, 1.0, 1.0, 1.0]},
             "emissive": {"value": [4.0, 3.0, 2.0, 1.0]}},
            {"name": "crate:paint", "type": "EMBEDDED"}, {"name": "crate:lacquer", "type": "EMBEDDED"},
            {"name": "panel:Panel", "type": "EMBEDDED"}],
        "lights": [{"name": "bulb", "type": "POINT", "color": [1.0, 0.9, 0.8], "intensity": 2.0},
                   {"name": "sun", "type": "DIRECTIONAL", "color": [1.0, 1.0, 0.95], "intensity": 0.6}],
        "scene": [
            {"name": "floor", "mesh": {"modelName": "box"}, "material": {"name": "floor"},
             "transform": {"position": [0, -0.05, 0], "scale": [2.5, 0.05, 2.5]}},
            {"name": "crate", "transform": {"position": [-0.6, 0.3, 0.1], "scale": [0.3, 0.3, 0.3],
                                            "rotation": [0.0, 30.0, 0.0]},
             "children": [{"name": "paint", "mesh": {"modelName": "crate", "submesh": "Crate"},
                           "material": {"name": "crate:paint"}},
                          {"name": "lacquer", "mesh": {"modelName": "crate", "submesh": "Crate-1"},
                           "material": {"name": "crate:lacquer"}}]},
            {"name": "block", "mesh": {"modelName": "box"}, "material": {"name": "metal"},
             "transform": {"position": [0.55, 0.25, -0.2], "scale": [0.25, 0.25, 0.25],
                           "rotation": [0.0, -20.0, 10.0]}},
            {"name": "board", "mesh": {"modelName": "panel", "submesh": "Panel"}, "material": {"name": "panel:Panel"},
             "transform": {"position": [0.0, 0.6, -0.6], "scale": [0.5, 0.5, 0.5]}},
            {"name": "haze", "mesh": {"modelName": "box"}, "material": {"name": "shell"},
             "volume": {"backFacing": "fog"},
             "transform": {"position": [0.0, 0.6, 0.0], "scale": [1.2, 0.6, 1.2]}},
            {"name": "lamp", "mesh": {"modelName": "box"}, "material": {"name": "lamp"},
             "transform": {"position": [0.3, 1.6, 0.5], "scale": [0.15, 0.02, 0.15]}},
            {"name": "bulb", "light": {"name": "bulb"}, "transform": {"position": [-0.8, 1.5, 1.0]}},
            {"name": "sun", "light": {"name": "sun"}, "transform": {"rotation": [-50.0, 30.0, 0.0]}}],
        "environment": {"path": "sky.hdr", "environmentType": 1, "backgroundColor": [0.0, 0.0, 0.0]},
    }
    (folder / "scene.json").write_text(json.dumps(doc))
    return folder / "scene.json"


def test_imported_scene_file_matches_oracle(ctx, tmp_path):
    """A scene file with OBJ (+ .mtl) and glTF models, every material and
    light kind, a medium and an environment map, imported and rendered on
    the GPU against the oracle."""
    from vviewer_gb300.scene_io import import_scene

    e = import_scene(_scene_file(tmp_path))
    fs = e.scene.build()
    assert len(fs.lights) >= 3 and any(m.uv_tiling[2] == 3.0 for m in fs.materials)
    info = RenderInfo(samples=64, depth=8, batch_size=2, width=96, height=64)
    res, ref = render_pair(ctx, e, info)
    # Many scattering events in an anisotropic medium: GPU and CPU float
    # rounding (contracted multiply-adds, libm ulps) make about a quarter of
    # the pixels' paths part ways, as they do between two builds of the
    # oracle itself. So the images are compared as estimates: every pixel
    # within 4 standard errors of the difference (both images' batch
    # variances) unless equal to float noise, and the image means.
    nb = info.samples // info.batch_size
    a, sa = _mean_and_se(res.radiance, res.radiance_m2, nb)
    b, sb = _mean_and_se(ref["radiance"], ref["radiance_m2"], nb)
    z = np.abs(a - b) / np.sqrt(sa ** 2 + sb ** 2 + 1e-20)
    close = np.isclose(a, b, rtol=1e-3, atol=1e-7).all(-1)
    outliers = ((~close) & (z > 4).any(-1)).mean()
    rel = abs(a.mean() - b.mean()) / b.mean()
    assert rel < 3e-3 and outliers < 0.002, (rel, outliers, close.mean())
    # first-surface albedo: camera rays that scatter in the medium first reach
    # their surface along diverged paths, so compare the image means
    aa, ab = res.albedo[..., :3].astype(np.float64), ref["albedo"][..., :3].astype(np.float64)
    assert abs(aa.mean() - ab.mean()) <= 1e-3 * ab.mean(), (aa.mean(), ab.mean())
    assert np.isclose(aa, ab, rtol=1e-5, atol=1e-6).all(-1).mean() >= 0.8


def test_many_emitters_match_oracle(ctx):
    """41 emissive instances: the emitter-ray prefilter merges their boxes
    into 32; every emitter contribution must survive it."""
    from raygen import many_lights_scene

    e, info = many_lights_scene(96, 96, 32)
    res, ref = render_pair(ctx, e, info)
    rel, close, z4 = compare_renders(res.radiance, ref["radiance"], res.radiance_m2, info.samples // info.batch_size)
    assert rel < 1e-4 and close >= 0.95 and z4 < 0.005, (rel, close, z4)


def test_thin_lens_and_non_square_match_oracle(ctx):
    e, info = scenes.cornell_box(4, 80, 48, 16, 8, 4)
    cam = e.scene.camera
    cam.lens_radius = 0.05
    cam.focal_distance = 1.8
    res, ref = render_pair(ctx, e, info)
    rel, close, z4 = compare_renders(res.radiance, ref["radiance"], res.radiance_m2, info.samples // info.batch_size)
    assert rel < 1e-4 and close >= 0.95 and z4 < 0.005, (rel, close, z4)


@pytest.mark.parametrize("mode", [EnvironmentType.HDRI, EnvironmentType.SOLID_COLOR_WITH_HDRI_LIGHTING])
def test_environment_map_matches_oracle(ctx, mode):
    e, info = scenes.cornell_box(5, 64, 64, 16, 8, 4)
    s = e.scene
    # open the room to the sky: remove the back wall's occlusion by moving the camera out
    s.camera.transform = Transform((0.5, 0.5, 3.0))
    h, w = 32, 64
    yy, xx = np.meshgrid(np.linspace(0, 1, h), np.linspace(0, 1, w), indexing="ij")
    env = np.stack([0.2 + xx, 0.3 + yy, 1.0 - 0.5 * yy, np.ones_like(xx)], -1).astype(np.float32)
    s.environment_map = env
    s.environment_type = mode
    s.environment_intensity = 0.7
    s.background_color = [0.1, 0.2, 0.3]
    res, ref = render_pair(ctx, e, info)
    rel, close, z4 = compare_renders(res.radiance, ref["radiance"], res.radiance_m2, info.samples // info.batch_size)
    assert rel < 1e-4 and close >= 0.95 and z4 < 0.005, (rel, close, z4)


@pytest.mark.parametrize("mode", [EnvironmentType.HDRI, EnvironmentType.SOLID_COLOR_WITH_HDRI_LIGHTING])
def test_environment_importance_sampling_matches_oracle(ctx, mode):
    """VVPT_RENDER_ENV_IS (environment as a light, importance sampled by
    luminance) against the oracle's same estimator, under a sky with a
    small bright sun."""
    e, info = scenes.sky_scene(2, 96, 64, 32, 8, 4)
    e.scene.environment_type = mode
    e.scene.background_color = [0.2, 0.3, 0.4]
    res, ref = render_pair(ctx, e, info, env_is=True)
    rel, close, z4 = compare_renders(res.radiance, ref["radiance"], res.radiance_m2, info.samples // info.batch_size)
    assert rel < 1e-4 and close >= 0.95 and z4 < 0.005, (rel, close, z4)


@pytest.mark.parametrize("scene", ["cornell", "medium_thin_lens"])
def test_pmj_sampler_matches_oracle(ctx, scene):
    """The low-discrepancy sampler (VVPT_RENDER_SAMPLER_PMJ) against the
    oracle's restatement of rng_pmj.glsl over the same tables: pixel jitter,
    lens, light and BSDF/phase draws from the (0,2) sequences or the hashed
    permutation plus blue noise, per-sample dimension restart."""
    if scene == "cornell":
        e, info = scenes.cornell_box(1, 96, 64, 32, 8, 4)
    else:
        e, info = scenes.cornell_medium(2, 64, 48, 32, 8, 4, freq=12, spheres=2)
        e.scene.camera.lens_radius = 0.02
        e.scene.camera.focal_distance = 2.0
    res, ref = render_pair(ctx, e, info, sampler="pmj")
    rel, close, z4 = compare_renders(res.radiance, ref["radiance"], res.radiance_m2, info.samples // info.batch_size)
    assert rel < 1e-4 and close >= 0.95 and z4 < 0.005, (rel, close, z4)


def test_converged_render_matches_fp64_oracle(ctx):
    """A converged GPU image (4096 spp) against the oracle's FP64-accumulated
    render at 4x the samples: per pixel within 3 Monte Carlo standard errors
    (the standard errors of both images from their batch sums, at least 99 %
    of the pixels) and the image means within 1e-3 relative."""
    e, info = scenes.cornell_box(1, 32, 32, 4096, 8, 4)
    fs = e.scene.build()
    sd = e.scene.scene_data(info.width, info.height)
    g = ctx.upload(fs)
    res = g.render(sd, info, want_m2=True)
    g.release()
    batches = info.samples // info.batch_size
    info.samples *= 4
    ref = oracle.render(fs, sd, info, fp64=True)
    rb = info.samples // info.batch_size
    a, sa = _mean_and_se(res.radiance, res.radiance_m2, batches)
    b, sb = _mean_and_se(ref["radiance"], ref["radiance_m2"], rb)
    z = np.abs(a - b) / np.sqrt(sa ** 2 + sb ** 2 + 1e-30)
    assert (z <= 3.0).all(-1).mean() >= 0.99, np.sort(z.ravel())[-10:]
    assert abs(a.mean() - b.mean()) <= 1e-3 * b.mean(), (a.mean(), b.mean())


def test_fp64_batch_reduction(ctx):
    """VVPT_RENDER_REDUCE_FP64: the same per-batch sums added in double
    precision. Against the float reduction the images differ by float
    rounding only; against the oracle's FP64 render (double sums throughout)
    they agree like the other renders."""
    e, info = scenes.cornell_box(2, 64, 48, 1024, 8, 4)
    fs = e.scene.build()
    sd = e.scene.scene_data(info.width, info.height)
    g = ctx.upload(fs)
    f32 = g.render(sd, info, want_m2=True)
    f64 = g.render(sd, info, want_m2=True, reduce_fp64=True)
    g.release()
    a, b = f64.radiance[..., :3].astype(np.float64), f32.radiance[..., :3].astype(np.float64)
    assert np.allclose(a, b, rtol=1e-4, atol=1e-7) and not np.array_equal(a, b)
    assert np.array_equal(f64.albedo[..., 3], f32.albedo[..., 3])
    ref = oracle.render(fs, sd, info, fp64=True)
    rel, close, z4 = compare_renders(f64.radiance, ref["radiance"], f64.radiance_m2, info.samples // info.batch_size)
    assert rel < 1e-4 and close >= 0.95 and z4 < 0.005, (rel, close, z4)


def test_instanced_sky_scene_matches_oracle(ctx):
    """512 rigid instances of 8 displaced meshes (20.7M instanced
    triangles), 32 mesh lights, thin lens, procedural sky with the
    environment importance sampled: a small crop-sized render against the
    oracle."""
    e, info = scenes.instanced_sky_scene(1, 64, 36, 16, 8, 4, sky_w=512, sky_h=256)
    res, ref = render_pair(ctx, e, info, env_is=True)
    rel, close, z4 = compare_renders(res.radiance, ref["radiance"], res.radiance_m2, info.samples // info.batch_size)
    assert rel < 1e-3 and close >= 0.9 and z4 < 0.01, (rel, close, z4)


@pytest.mark.parametrize("name", list(R.BUILDERS))
def test_gpu_render_meets_reference_golden(ctx, name):
    """Every pixel, untrimmed, against the reference's MSE tolerance. For
    MeshLight, whose golden depends on the order in which the reference's
    hardware reported any-hit candidates to BSDF-direction emitter rays
    (reference_scenes.ORDER_DEPENDENT), the pixels where that order matters
    are checked against the bracket of the two end orders instead: this
    render (nearest first) and the oracle's instance-order render."""
    e, info, tol = R.BUILDERS[name]()
    fs = e.scene.build()
    sd = e.scene.scene_data(256, 256)
    g = ctx.upload(fs)
    res = g.render(sd, info)
    g.release()
    rgb = res.radiance[..., :3]
    enc = rgbe_encode(rgb)
    mse_outside, bracketed, mse_bracket = R.golden_check_with_orders(name, rgb)
    exact = (enc == R.golden_rgbe(name)).all(-1).mean()
    assert mse_outside + mse_bracket <= tol, f"{name}: mse {mse_outside:.3e} + {mse_bracket:.3e} > {tol:.0e}"
    assert bracketed >= 0.99, f"{name}: {bracketed:.4f} of order-dependent values bracketed"
    assert exact >= 0.9
    dep = R.order_dependent_pixels(name)
    if dep is not None:
        # the order-dependent pixels themselves match the oracle's
        # nearest-first image (same RTGEMS stream)
        pix, near, _ = dep
        ours = rgb.reshape(-1, 3)[pix].astype(np.float64)
        rel = np.abs(ours - near) / np.maximum(np.abs(near), 1e-3)
        assert np.median(rel) < 1e-4 and (rel < 1e-2).mean() > 0.99, (np.median(rel), (rel < 1e-2).mean())


def test_autotune_picks_a_candidate_and_keeps_images(ctx):
    e, info = scenes.cornell_box(7, 96, 64, 16, 8, 4)
    fs = e.scene.build()
    sd = e.scene.scene_data(96, 64)
    g = ctx.upload(fs)
    before = g.render(sd, info)
    try:
        t = g.autotune(sd, info, budget_ms=400.0)
        assert t["blocks_per_sm"] in (0, 2, 3, 4, 6, 8)
        assert t["slots"] in (0, 1 << 19, 1 << 20, 3 << 19, 1 << 21)
        assert t["iterations_per_graph"] in (0, 4, 8, 16)
        after = g.render(sd, info)
        assert (after.radiance == before.radiance).all()
    finally:
        ctx.set_tuning()
        g.release()


def test_render_is_deterministic_across_schedules(ctx):
    e, info = scenes.cornell_box(6, 64, 64, 32, 8, 4)
    fs = e.scene.build()
    sd = e.scene.scene_data(64, 64)
    g = ctx.upload(fs)
    a = g.render(sd, info)
    b = g.render(sd, info)
    ctx.set_tuning(slots=1000, blocks_per_sm=1, threads_per_block=128, iterations_per_graph=2)
    try:
        c = g.render(sd, info)
    finally:
        ctx.set_tuning()
    g.release()
    for k in ("radiance", "albedo", "normal"):
        assert (getattr(a, k) == getattr(b, k)).all()
        assert (getattr(a, k) == getattr(c, k)).all()


def test_render_edge_cases(ctx):
    e, info = scenes.cornell_box(1, 32, 32, 8, 8, 4)
    fs = e.scene.build()
    sd = e.scene.scene_data(32, 32)
    g = ctx.upload(fs)
    info.depth = 0
    assert (g.render(sd, info).radiance == 0).all()
    info.depth, info.samples = 8, 3  # batches = 3 / 4 = 0
    assert (g.render(sd, info).radiance == 0).all()
    info.samples, info.batch_size = 8, 8  # one batch
    r = g.render(sd, info)
    assert np.isfinite(r.radiance).all() and r.radiance[..., :3].sum() > 0
    assert (r.radiance[..., 3] == 1.0).all()
    g.release()


def test_light_only_scene_renders_background(ctx):
    e = Engine()
    s = e.scene
    so = s.add_scene_object("light", Transform((0, 1, 0)))
    so.light = e.light("defaultPointLight")
    s.background_color = [0.25, 0.5, 0.75]
    info = RenderInfo(samples=4, depth=4, batch_size=2, width=16, height=16, write_files=False)
    g = ctx.upload(s.build())
    r = g.render(s.scene_data(16, 16), info)
    g.release()
    assert np.allclose(r.radiance[..., :3], [0.25, 0.5, 0.75], atol=1e-6)
    assert np.allclose(r.albedo[..., :3], [0.25, 0.5, 0.75], atol=1e-6)


def test_device_outputs_equal_host_outputs(ctx):
    torch = pytest.importorskip("torch")
    e, info = scenes.cornell_box(2, 48, 32, 8, 8, 4)
    fs = e.scene.build()
    sd = e.scene.scene_data(48, 32)
    g = ctx.upload(fs)
    host = g.render(sd, info)
    bufs = {k: torch.zeros((32, 48, 4), dtype=torch.float32, device="cuda") for k in ("radiance", "albedo", "normal")}
    g.render(sd, info, outputs={k: v.data_ptr() for k, v in bufs.items()})
    torch.cuda.synchronize()
    g.release()
    for k, v in bufs.items():
        assert (v.cpu().numpy() == getattr(host, k)).all()


def test_invalid_arguments_are_reported(ctx):
    e, info = scenes.cornell_box(1, 16, 16, 4, 4, 4)
    fs = e.scene.build()
    fs.instances[0].material_index = 999
    with pytest.raises(N.VvptError) as ei:
        ctx.upload(fs)
    assert ei.value.status == 1 and "material" in str(ei.value)
    fs = e.scene.build()
    g = ctx.upload(fs)
    sd = e.scene.scene_data(16, 16)
    info.width = 0
    with pytest.raises(N.VvptError):
        g.render(sd, info)
    info.width = 16
    sd.volumes[0] = 999.0
    with pytest.raises(N.VvptError):
        g.render(sd, info)
    g.release()


def test_progress_reaches_one(ctx):
    e, info = scenes.cornell_box(1, 16, 16, 4, 4, 4)
    g = ctx.upload(e.scene.build())
    g.render(e.scene.scene_data(16, 16), info)
    p = C.c_float()
    ctx.lib.vvpt_progress(ctx.handle, C.byref(p))
    assert p.value == 1.0
    g.release()


def test_gpu_bvh_builder_gives_the_same_hits(ctx):
    """Meshes of 65,536 triangles or more are built on the GPU by default;
    the host builder (VVPT_BVH_BUILDER_HOST) and the all-GPU builder
    (VVPT_BVH_BUILDER_GPU: every BLAS, the baked small instances and the
    TLAS) must give identical closest hits (all are exact), and they must
    match the oracle."""
    e, _ = scenes.cornell_medium(4, 64, 64, 4, 8, 4, freq=60, spheres=2)  # 2 x 72,000 triangles
    fs = e.scene.build()
    rays = np.concatenate([make_rays(fs, 100_000, 17, -0.2, 1.2), make_near_rays(fs, 20_000, 18)])
    hits = {}
    try:
        for builder in (N_BVH_AUTO, N_BVH_HOST, N_BVH_GPU):
            ctx.check(ctx.lib.vvpt_set_bvh_builder(ctx.handle, builder))
            g = ctx.upload(fs)
            hits[builder] = g.trace_closest(rays)
            g.release()
    finally:
        ctx.check(ctx.lib.vvpt_set_bvh_builder(ctx.handle, N_BVH_AUTO))
    assert_hits_equal(hits[N_BVH_AUTO], hits[N_BVH_HOST])
    assert_hits_equal(hits[N_BVH_GPU], hits[N_BVH_HOST])
    assert_hits_equal(hits[N_BVH_AUTO], oracle.trace_closest(fs, rays))
    assert ctx.lib.vvpt_set_bvh_builder(ctx.handle, 3) == 1  # VVPT_ERR_INVALID_ARG


@pytest.mark.parametrize("name", ["cornell", "volume_cube", "shared_components"])
def test_all_gpu_builder_hits_and_renders(ctx, name):
    """Every tree built on the GPU, including the TLAS over many instances
    and the baked BLAS of the small instances: closest hits equal to the
    oracle's, and a render equal bit for bit to the default builder's."""
    build, (lo, hi) = HIT_SCENES[name]
    e = build()
    fs = e.scene.build()
    rays = np.concatenate([make_rays(fs, 60_000, 23, lo, hi), make_near_rays(fs, 20_000, 24)])
    info = RenderInfo(samples=8, depth=6, batch_size=4, width=24, height=16, write_files=False)
    sd = e.scene.scene_data(info.width, info.height)
    out = {}
    try:
        for builder in (N_BVH_AUTO, N_BVH_GPU):
            ctx.check(ctx.lib.vvpt_set_bvh_builder(ctx.handle, builder))
            g = ctx.upload(fs)
            out[builder] = (g.trace_closest(rays), g.render(sd, info))
            g.release()
    finally:
        ctx.check(ctx.lib.vvpt_set_bvh_builder(ctx.handle, N_BVH_AUTO))
    assert_hits_equal(out[N_BVH_GPU][0], oracle.trace_closest(fs, rays))
    assert np.array_equal(out[N_BVH_GPU][1].radiance, out[N_BVH_AUTO][1].radiance)
