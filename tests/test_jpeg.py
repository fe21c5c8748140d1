"""JPEG texture decoding (vengine reads model textures through stb_image,
AssimpLoadModel.cpp:assimpLoadTextureData, which decodes JPEG as well as PNG).
The files come from the small baseline encoder in jpeg_files.py, which also
returns the quantised coefficients it wrote. The Python restatement
(jpeg_reference.py) is checked coefficient for coefficient against the
encoder and its reconstruction against a direct evaluation of the T.81 inverse
DCT formula; libvvpt's host decoder (vvpt_jpeg_decode, what model import
uses) is checked against the restatement. No GPU is needed."""
import math

import numpy as np
import pytest

from jpeg_files import ZIGZAG, encode_jpeg
from jpeg_reference import decode_jpeg as decode_jpeg_py
from jpeg_reference import decode_jpeg_coefficients
from vviewer_gb300.jpeg import decode_jpeg


def _image(h, w, seed=1):
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w]
    img = np.stack([128 + 100 * np.sin(xx / 7.0), 128 + 90 * np.cos(yy / 5.0), (xx * 3 + yy * 2) % 256], -1)
    return np.clip(img + rng.normal(0, 3, img.shape), 0, 255).astype(np.uint8)


def _psnr(a, b):
    return 10 * math.log10(255.0 ** 2 / np.mean((a.astype(np.float64) - b) ** 2))


@pytest.mark.parametrize("h,w", [(8, 8), (37, 53), (16, 33), (1, 1)])
@pytest.mark.parametrize("subsample", [False, True, (2, 1), (1, 2)])
def test_coefficients_match_the_encoder(h, w, subsample):
    data, coefs, q = encode_jpeg(_image(h, w), subsample=subsample, return_coefficients=True)
    frame, qt = decode_jpeg_coefficients(data, "t.jpg")
    assert (frame["h"], frame["w"]) == (h, w) and len(frame["comps"]) == 3
    for comp, ref in zip(frame["comps"], coefs):
        assert np.array_equal(comp["coef"], ref)
    assert np.array_equal(qt[0], q)


def test_inverse_dct_follows_the_formula():
    """Grey 4:4:4 file: each sample equals the rounded, clamped, level-shifted
    sum of T.81 A.3.3 over the dequantised coefficients."""
    img = _image(16, 24)[..., 1]
    data, coefs, q = encode_jpeg(img, return_coefficients=True)
    out, channels = decode_jpeg(data, "g.jpg")
    assert channels == 1
    cos = [[math.cos((2 * x + 1) * u * math.pi / 16) for u in range(8)] for x in range(8)]
    c = [1 / math.sqrt(2)] + [1.0] * 7
    for by, bx in ((0, 0), (1, 2), (0, 1)):
        f = np.zeros(64)
        f[ZIGZAG] = coefs[0][by, bx]
        f = f.reshape(8, 8) * q
        for y in range(8):
            for x in range(8):
                s = sum(c[u] * c[v] * f[v, u] * cos[x][u] * cos[y][v] for u in range(8) for v in range(8)) / 4
                ref = min(255, max(0, math.floor(s + 128 + 0.5)))
                assert abs(int(out[by * 8 + y, bx * 8 + x, 0]) - ref) <= (0 if abs(s % 1 - 0.5) > 1e-9 else 1)


@pytest.mark.parametrize("subsample,min_psnr", [(False, 45.0), (True, 37.0), ((2, 1), 39.0), ((1, 2), 39.0)])
def test_round_trip_quality(subsample, min_psnr):
    img = _image(37, 53)
    out, channels = decode_jpeg(encode_jpeg(img, subsample=subsample), "t.jpg")
    assert channels == 3 and out.shape == (37, 53, 4) and (out[..., 3] == 255).all()
    assert _psnr(out[..., :3], img) > min_psnr


def test_flat_colour_is_exact():
    img = np.zeros((20, 30, 3), dtype=np.uint8)
    img[:] = (90, 140, 200)
    out, _ = decode_jpeg(encode_jpeg(img, subsample=False), "flat.jpg")
    assert np.abs(out[..., :3].astype(int) - img).max() <= 1


@pytest.mark.parametrize("interval", [1, 3, 7])
def test_restart_intervals_decode_identically(interval):
    img = _image(40, 72, seed=3)
    for subsample in (False, True):
        plain, _ = decode_jpeg(encode_jpeg(img, subsample=subsample), "a.jpg")
        rst, _ = decode_jpeg(encode_jpeg(img, subsample=subsample, restart=interval), "b.jpg")
        assert np.array_equal(plain, rst)


def test_grey_file_fills_rgb_and_opaque_alpha():
    g = _image(13, 21)[..., 0]
    out, channels = decode_jpeg(encode_jpeg(g), "g.jpg")
    assert channels == 1
    assert (out[..., 0] == out[..., 1]).all() and (out[..., 1] == out[..., 2]).all() and (out[..., 3] == 255).all()
    assert _psnr(out[..., 0], g) > 45.0


def test_unsupported_and_broken_files_raise():
    data = bytearray(encode_jpeg(_image(16, 16)))
    sof = data.index(b"\xff\xc0")
    progressive = bytes(data[:sof + 1]) + b"\xc2" + bytes(data[sof + 2:])
    with pytest.raises(ValueError, match="progressive"):
        decode_jpeg(progressive, "p.jpg")
    with pytest.raises(ValueError, match="not a JPEG"):
        decode_jpeg(b"\x89PNG\r\n\x1a\n", "x.jpg")
    with pytest.raises(ValueError):
        decode_jpeg(bytes(data[:len(data) // 2]), "truncated.jpg")
    twelve = bytes(data[:sof + 4]) + b"\x0c" + bytes(data[sof + 5:])
    with pytest.raises(ValueError, match="12-bit"):
        decode_jpeg(twelve, "12.jpg")


def test_obj_map_kd_jpeg_becomes_the_albedo_texture(tmp_path):
    """A .mtl map_Kd naming a JPEG gives an sRGB albedo texture of the decoded
    texels, three channels: no alpha texture, not transparent."""
    from vviewer_gb300 import _native as N
    from vviewer_gb300.model3d import import_model
    from vviewer_gb300.scene import TEX_WHITE_COLOR, Engine

    img = _image(12, 20, seed=5)
    data = encode_jpeg(img, subsample=True, restart=2)
    (tmp_path / "wood.jpg").write_bytes(data)
    (tmp_path / "grey.jpg").write_bytes(encode_jpeg(img[..., 2]))
    (tmp_path / "prog.jpg").write_bytes(data.replace(b"\xff\xc0", b"\xff\xc2", 1))
    (tmp_path / "m.mtl").write_text("newmtl wood\nKd 0 0 0\nmap_Kd wood.jpg\n"
                                    "newmtl grey\nKd 0.5 0.5 0.5\nmap_Kd grey.jpg\n"
                                    "newmtl prog\nKd 0.25 0.25 0.25\nmap_Kd prog.jpg\n")
    (tmp_path / "m.obj").write_text("mtllib m.mtl\nv 0 0 0\nv 1 0 0\nv 1 1 0\nvt 0 0\nvt 1 0\nvt 1 1\n"
                                    "usemtl wood\nf 1/1 2/2 3/3\nusemtl grey\nf 1/1 3/3 2/2\n"
                                    "usemtl prog\nf 2/2 1/1 3/3\n")
    e = Engine()
    with pytest.warns(UserWarning, match="prog.jpg: JPEG not decoded"):
        model = import_model(e, tmp_path / "m.obj", name="m")
    mats = {m.name.split(":")[1]: m for m in model.materials}
    wood = mats["wood"]
    assert wood.albedo == [1.0, 1.0, 1.0, 1.0] and wood.alpha_texture == mats["DefaultMaterial"].alpha_texture
    fmt, tex = e.textures[wood.albedo_texture]
    assert fmt == N.TEXTURE_RGBA8_SRGB and np.array_equal(tex, decode_jpeg(data)[0])
    assert not wood.pack().metallic_roughness_ao[3]  # three channels: opaque
    fmt, tex = e.textures[mats["grey"].albedo_texture]
    assert (tex[..., 0] == tex[..., 2]).all() and _psnr(tex[..., 0], img[..., 2]) > 45.0
    assert mats["prog"].albedo_texture == TEX_WHITE_COLOR


def test_gltf_embedded_jpeg_is_decoded(tmp_path):
    from gltf_files import GltfBuilder, quad_arrays
    from vviewer_gb300.model3d import import_model
    from vviewer_gb300.scene import Engine

    img = _image(16, 16, seed=7)
    data = encode_jpeg(img, subsample=False)
    b = GltfBuilder()
    t = b.image(data)
    mat = b.material(name="Photo", pbrMetallicRoughness={"baseColorTexture": {"index": t}})
    pos, nrm, uv, idx = quad_arrays(1.0)
    attrs = {"POSITION": b.accessor(pos), "NORMAL": b.accessor(nrm), "TEXCOORD_0": b.accessor(uv)}
    b.scene([b.node(mesh=b.mesh([{"attributes": attrs, "indices": b.accessor(idx), "material": mat}]))])
    e = Engine()
    import_model(e, b.save(tmp_path / "photo.glb"), name="photo")
    p = e.material("photo:Photo")
    assert np.array_equal(e.textures[p.albedo_texture][1], decode_jpeg(data)[0]) and not p.transparent


@pytest.mark.parametrize("subsample", [False, True, (2, 1), (1, 2)])
@pytest.mark.parametrize("h,w,restart", [(37, 53, 0), (64, 48, 3), (9, 130, 1)])
def test_native_decoder_matches_the_restatement(subsample, h, w, restart):
    """libvvpt's decoder against the Python restatement of the same steps:
    the same texels (an IDCT summed in another order may round a .5 tie the
    other way: at most one unit, on few texels)."""
    data = encode_jpeg(_image(h, w, seed=h + w), quality=2.0, subsample=subsample, restart=restart)
    a, ca = decode_jpeg(data, "n.jpg")
    b, cb = decode_jpeg_py(data, "p.jpg")
    assert ca == cb == 3 and a.shape == b.shape == (h, w, 4)
    diff = np.abs(a.astype(int) - b.astype(int))
    assert diff.max() <= 1 and (diff > 0).mean() < 1e-3


def test_native_decoder_survives_corrupt_files():
    """Truncated and byte-flipped files give an error status or an image,
    never a crash or an out-of-range read."""
    rng = np.random.default_rng(0)
    bases = [encode_jpeg(_image(24, 40, seed=2), restart=2, subsample=s) for s in (False, True)]
    bases.append(encode_jpeg(_image(16, 16, seed=3)[..., 0]))
    decoded = failed = 0
    for k in range(3000):
        d = bytearray(bases[k % 3])
        if k % 2:
            d = d[:rng.integers(2, len(d))]
        else:
            for _ in range(rng.integers(1, 6)):
                d[rng.integers(2, len(d))] = rng.integers(0, 256)
        try:
            img, _ = decode_jpeg(bytes(d), "f.jpg")
            assert img.dtype == np.uint8 and img.ndim == 3
            decoded += 1
        except ValueError:
            failed += 1
    assert decoded + failed == 3000 and failed > 0
