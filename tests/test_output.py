"""The output step: exposure, sRGB 8-bit PNG, RGBE HDR
and the AOV file set, against the reference's own rules restated here in
float32 arithmetic:
  * applyExposure / tonemap (src/lib/vengine/core/ImageUtils.cpp:34-49):
    v * 2^exposure on the first three channels;
  * writeToDisk (ImageUtils.cpp:51-76): PNG = uint8(255 * linearToSRGB(
    clamp(v, 0, 1))) on every channel (truncation), HDR = RGBE of RGB;
  * storeToDisk (src/lib/vengine/vulkan/renderers/VulkanRendererPathTracing.cpp:958-1027):
    which files, exposure for PNG only, the noisy radiance beside the
    denoised image.
"""
import numpy as np
import pytest

from vviewer_gb300.assets import read_hdr_rgbe, rgbe_decode, rgbe_encode
from vviewer_gb300.renderer import RenderResult, RendererPathTracing, apply_exposure, write_to_disk
from vviewer_gb300.scene import Engine
from vviewer_gb300.scene_io import read_png


def linear_to_srgb_f32(v):
    """ImageUtils.cpp:12-21 for one float, in float32."""
    v = np.float32(v)
    if v <= np.float32(0.0031308):
        return np.float32(v * np.float32(12.92))
    return np.float32(np.float32(1.055) * np.float32(np.power(v, np.float32(1.0) / np.float32(2.4))) -
                      np.float32(0.055))


def image(seed, h=7, w=11):
    rng = np.random.default_rng(seed)
    img = rng.uniform(-0.2, 1.4, size=(h, w, 4)).astype(np.float32)
    img[0, 0, :3] = [0.0, 0.0031308, 0.0031309]
    img[0, 1, :3] = [1.0, 0.5, 1e-5]
    img[..., 3] = rng.uniform(0.0, 1.0, size=(h, w)).astype(np.float32)
    return img


def test_apply_exposure_scales_rgb_only():
    img = image(1)
    for e in (0.0, 1.0, -2.5, 0.75):
        out = apply_exposure(img, e)
        f = np.float32(np.power(np.float32(2.0), np.float32(e)))
        assert np.array_equal(out[..., :3], img[..., :3] * f)
        assert np.array_equal(out[..., 3], img[..., 3])
    assert out is not img


def test_png_is_srgb8_of_every_channel(tmp_path):
    img = image(2)
    write_to_disk(img, str(tmp_path / "x"), "png")
    got = read_png(tmp_path / "x.png")
    assert got.shape == img.shape and got.dtype == np.uint8
    want = np.zeros(img.shape, dtype=np.uint8)
    for idx in np.ndindex(img.shape):
        c = min(max(img[idx], np.float32(0.0)), np.float32(1.0))
        want[idx] = int(np.float32(255.0) * linear_to_srgb_f32(c))
    assert np.array_equal(got, want)


def test_hdr_is_rgbe_of_rgb(tmp_path):
    img = image(3, 9, 40)  # width >= 8: run-length rows
    # radiance is never negative (stb's float-to-byte cast of a negative
    # component is undefined behaviour)
    img[..., :3] = np.abs(img[..., :3]) * 50.0
    write_to_disk(img, str(tmp_path / "y"), "hdr")
    rgbe = read_hdr_rgbe(tmp_path / "y.hdr")
    assert np.array_equal(rgbe, rgbe_encode(img[..., :3]))
    dec = rgbe_decode(rgbe)
    pos = np.clip(img[..., :3], 0.0, None)
    big = pos.max(-1, keepdims=True) > 1e-3
    assert (np.abs(dec - pos) <= pos.max(-1, keepdims=True) * 2.0 ** -7 + 1e-30)[big[..., 0]].all()
    with pytest.raises(ValueError):
        write_to_disk(img, str(tmp_path / "z"), "exr")


def _result(seed):
    return RenderResult(image(seed), image(seed + 1), image(seed + 2), None, None, 1)


class _FakeDenoiser:
    """Records what the output step hands the denoising step."""

    def __init__(self):
        self.calls = []

    def denoise(self, radiance, albedo, normal):
        self.calls.append((radiance.copy(), albedo.copy(), normal.copy()))
        return np.full_like(radiance, 0.25)


@pytest.mark.parametrize("file_type", ["hdr", "png"])
@pytest.mark.parametrize("write_all", [False, True])
def test_store_to_disk_file_set_without_denoising(tmp_path, file_type, write_all):
    r = RendererPathTracing(Engine())
    info = r.render_info()
    info.filename = str(tmp_path / "shot")
    info.file_type = file_type
    info.exposure = 1.5
    info.write_all_files = write_all
    res = _result(10)
    r.store_to_disk(res)
    names = sorted(p.name for p in tmp_path.iterdir())
    want = [f"shot.{file_type}"] + (["shot_albedo.hdr", "shot_normal.hdr"] if write_all else [])
    assert names == sorted(want)
    if file_type == "png":
        # exposure applies to PNG output only
        ref_dir = tmp_path / "ref"
        ref_dir.mkdir()
        write_to_disk(apply_exposure(res.radiance, 1.5), str(ref_dir / "r"), "png")
        assert np.array_equal(read_png(tmp_path / "shot.png"), read_png(ref_dir / "r.png"))
    else:
        assert np.array_equal(read_hdr_rgbe(tmp_path / "shot.hdr"), rgbe_encode(res.radiance[..., :3]))
    if write_all:
        assert np.array_equal(read_hdr_rgbe(tmp_path / "shot_albedo.hdr"), rgbe_encode(res.albedo[..., :3]))
        assert np.array_equal(read_hdr_rgbe(tmp_path / "shot_normal.hdr"), rgbe_encode(res.normal[..., :3]))


@pytest.mark.parametrize("file_type", ["hdr", "png"])
def test_store_to_disk_with_denoising(tmp_path, file_type):
    fake = _FakeDenoiser()
    r = RendererPathTracing(Engine(), denoiser=fake)
    info = r.render_info()
    info.filename = str(tmp_path / "d")
    info.file_type = file_type
    info.exposure = -1.0
    info.denoise = True
    info.write_all_files = True
    res = _result(20)
    r.store_to_disk(res)
    names = sorted(p.name for p in tmp_path.iterdir())
    assert names == sorted([f"d.{file_type}", "d_albedo.hdr", "d_normal.hdr", "d_radiance.hdr"])
    # the noisy radiance is kept beside the denoised image
    assert np.array_equal(read_hdr_rgbe(tmp_path / "d_radiance.hdr"), rgbe_encode(res.radiance[..., :3]))
    assert len(fake.calls) == 1
    rad, alb, nrm = fake.calls[0]
    assert np.array_equal(rad, res.radiance) and np.array_equal(alb, res.albedo) and np.array_equal(nrm, res.normal)
    denoised = np.full_like(res.radiance, 0.25)
    if file_type == "png":
        ref = tmp_path / "ref"
        ref.mkdir()
        write_to_disk(apply_exposure(denoised, -1.0), str(ref / "r"), "png")
        assert np.array_equal(read_png(tmp_path / "d.png"), read_png(ref / "r.png"))
    else:
        assert np.array_equal(read_hdr_rgbe(tmp_path / "d.hdr"), rgbe_encode(denoised[..., :3]))


def test_denoise_without_a_denoiser_is_refused(tmp_path):
    r = RendererPathTracing(Engine())
    info = r.render_info()
    info.filename = str(tmp_path / "n")
    info.denoise = True
    with pytest.raises(ValueError):
        r.store_to_disk(_result(30))
