"""Learned denoiser on the GPU (vvpt_denoiser_*): its gradients against the
NumPy oracle with the same BF16 rounding points, and what training on
tracer-rendered pairs gains over the noisy render on a held-out scene."""
import numpy as np
import pytest

from oracle import denoiser_oracle as D
from vviewer_gb300 import _native as N
from vviewer_gb300 import scenes
from vviewer_gb300.denoiser import Denoiser

pytestmark = pytest.mark.gpu


def _cuda(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32)).cuda().contiguous()


def test_gradients_match_oracle(ctx):
    """Every parameter's gradient against the oracle's BF16 mode. The whole
    gradient agrees to < 5e-3 relative; single layers at the coarsest levels
    (2 x 3 pixels here) sum few products, where one BF16 rounding that lands
    the other way in the forward pass moves them by a few percent (seen with
    both the tcgen05 and the mma.sync kernels), hence 6e-2 per layer."""
    rng = np.random.default_rng(5)
    n, h, w = 2, 32, 48
    rad = rng.gamma(1.0, 0.5, (n, h, w, 4)).astype(np.float32)
    alb = rng.uniform(0, 1, (n, h, w, 4)).astype(np.float32)
    nrm = rng.uniform(0, 1, (n, h, w, 4)).astype(np.float32)
    tgt = (rad * rng.uniform(0.5, 1.5, rad.shape)).astype(np.float32)
    dn = Denoiser(ctx, seed=7)
    p = dn.params()
    loss_gpu, g_gpu = dn.gradients(_cuda(rad), _cuda(alb), _cuda(nrm), _cuda(tgt))
    loss_ref, g_ref = D.loss_and_grads(p, rad, alb, nrm, tgt)
    assert abs(loss_gpu - loss_ref) <= 1e-3 * loss_ref, (loss_gpu, loss_ref)
    assert np.linalg.norm(g_gpu - g_ref) <= 5e-3 * np.linalg.norm(g_ref)
    off = 0
    for k, (cin, cout, _) in enumerate(D.layers()):
        nw = cout * 9 * cin
        for name, sl in (("weights", slice(off, off + nw)), ("bias", slice(off + nw, off + nw + cout))):
            a, b = g_gpu[sl].astype(np.float64), g_ref[sl]
            if not np.any(b):
                assert not np.any(a), (k, name)
                continue
            rel = np.linalg.norm(a - b) / np.linalg.norm(b)
            assert rel < 6e-2, f"layer {k} {name}: relative error {rel:.3e}"
        off += nw + cout
    dn.close()


def test_shape_checks(ctx):
    dn = Denoiser(ctx, seed=1)
    x = _cuda(np.zeros((1, 20, 32, 4)))
    with pytest.raises(N.VvptError):
        dn.gradients(x, x, x, x)
    dn.close()


def _pairs(ctx, seeds, size, noisy_spp, target_spp):
    """(noisy radiance, albedo, normal, target) tensors [n, size, size, 4]
    rendered by the tracer from seeded Cornell scenes with a medium."""
    import torch
    out = {k: [] for k in ("rad", "alb", "nrm", "tgt")}
    for s in seeds:
        e, info = scenes.cornell_medium(s, size, size, noisy_spp, 8, 4, freq=12, spheres=4)
        g = ctx.upload(e.scene.build())
        sd = e.scene.scene_data(size, size)
        r = g.render(sd, info)
        info.samples = target_spp
        t = g.render(sd, info)
        g.release()
        out["rad"].append(r.radiance)
        out["alb"].append(r.albedo)
        out["nrm"].append(r.normal)
        out["tgt"].append(t.radiance)
    return [torch.from_numpy(np.stack(out[k])).cuda().contiguous() for k in ("rad", "alb", "nrm", "tgt")]


def _rel_rmse(img, ref):
    img = img[..., :3].astype(np.float64)
    ref = ref[..., :3].astype(np.float64)
    return np.sqrt(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))


def test_training_on_tracer_pairs_beats_the_noisy_render(ctx):
    import torch
    rad, alb, nrm, tgt = _pairs(ctx, range(10, 18), 64, 4, 512)
    dn = Denoiser(ctx, seed=3)
    losses = []
    for step in range(400):
        losses.append(dn.train_step(rad, alb, nrm, tgt, lr=2e-3 if step < 300 else 5e-4))
    assert np.mean(losses[-20:]) < 0.6 * np.mean(losses[:5])
    # held-out scene
    hr, ha, hn, ht = _pairs(ctx, [99], 64, 4, 512)
    out = torch.zeros_like(hr[0])
    dn.apply(hr[0], ha[0], hn[0], out)
    torch.cuda.synchronize()
    den = out.cpu().numpy()
    noisy = hr[0].cpu().numpy()
    ref = ht[0].cpu().numpy()
    e_noisy, e_den = _rel_rmse(noisy, ref), _rel_rmse(den, ref)
    assert np.isfinite(den).all() and (den[..., 3] == 1.0).all()
    assert e_den < 0.7 * e_noisy, (e_den, e_noisy)
    dn.close()


@pytest.mark.parametrize("kind", ["tcgen05", "tcgen05_tiles", "tcgen05_persistent", "tcgen05_unfused",
                                  "tcgen05_wgrad"])
@pytest.mark.parametrize("n,h,w", [(2, 64, 48), (1, 48, 272)])
def test_tcgen05_and_mma_sync_kernels_agree(ctx, kind, n, h, w):
    """The tcgen05 convolutions (TMEM accumulators) against the warp-level
    mma.sync ones on the same network and inputs: the default mix (strip
    kernel where the weights fit), the per-tile kernels alone, and the strip
    kernel on a 16-CTA grid (every CTA walks several row segments, so ring
    slots and accumulators change phase across segments). Partial tiles at
    every level: 2 x 64 x 48 pixels (narrower than one 130-pixel input box)
    and 48 x 272 (three 128-pixel columns at full resolution, the last 16
    wide; 136 at the next level)."""
    import torch
    rng = np.random.default_rng(6)
    ins = [_cuda(rng.gamma(1.0, 0.5, (n, h, w, 4))), _cuda(rng.uniform(0, 1, (n, h, w, 4))),
           _cuda(rng.uniform(0, 1, (n, h, w, 4))), _cuda(rng.gamma(1.0, 0.5, (n, h, w, 4)))]
    dn = Denoiser(ctx, seed=9)
    out = {}
    for k in ("mma_sync", kind):
        dn.set_kernels(k)
        loss, g = dn.gradients(*ins)
        o = torch.zeros((h, w, 4), device="cuda")
        dn.apply(ins[0][0], ins[1][0], ins[2][0], o)
        torch.cuda.synchronize()
        out[k] = (loss, g, o.cpu().numpy())
    (l0, g0, o0), (l1, g1, o1) = out["mma_sync"], out[kind]
    assert abs(l0 - l1) <= 1e-3 * l0
    assert np.linalg.norm(g1 - g0) <= 2e-2 * np.linalg.norm(g0)
    assert np.allclose(o1, o0, rtol=2e-2, atol=1e-3)
    dn.close()


@pytest.mark.parametrize("n,h,w", [(1, 64, 48), (1, 48, 272)])
def test_fused_upsample_concat_is_exact(ctx, n, h, w):
    """Inference reads the decoder's upsample + concat input straight from the
    coarse and skip tensors (an extra warp writes the upsampled channels into
    the strip kernel's ring); the convolution sees the same BF16 values in the
    same order, so the image is bit-identical to the unfused path's."""
    import torch
    rng = np.random.default_rng(8)
    ins = [_cuda(rng.gamma(1.0, 0.5, (h, w, 4))), _cuda(rng.uniform(0, 1, (h, w, 4))),
           _cuda(rng.uniform(0, 1, (h, w, 4)))]
    dn = Denoiser(ctx, seed=4)
    outs = {}
    for kind in ("tcgen05", "tcgen05_unfused", "tcgen05_persistent"):
        dn.set_kernels(kind)
        o = torch.zeros((h, w, 4), device="cuda")
        dn.apply(*ins, o)
        torch.cuda.synchronize()
        outs[kind] = o.cpu().numpy()
    assert np.array_equal(outs["tcgen05"], outs["tcgen05_unfused"])
    assert np.array_equal(outs["tcgen05_persistent"], outs["tcgen05_unfused"])
    dn.close()


def test_timed_out_wait_is_reported_and_the_denoiser_recovers(ctx):
    """Failure handling without a GPU fault: one strip convolution withholds
    its accumulator-ready signal, the drain warps' bounded waits run out, the
    kernel frees its tensor memory and records an error status; apply()
    reports VVPT_ERR_DEVICE and the next apply() gives the normal image."""
    import torch
    rng = np.random.default_rng(9)
    h, w = 32, 48
    ins = [_cuda(rng.gamma(1.0, 0.5, (h, w, 4))), _cuda(rng.uniform(0, 1, (h, w, 4))),
           _cuda(rng.uniform(0, 1, (h, w, 4)))]
    dn = Denoiser(ctx, seed=2)
    ref = torch.zeros((h, w, 4), device="cuda")
    dn.apply(*ins, ref)
    dn.inject_wait_timeout()
    out = torch.zeros((h, w, 4), device="cuda")
    with pytest.raises(N.VvptError) as e:
        dn.apply(*ins, out)
    assert e.value.status == 5  # VVPT_ERR_DEVICE
    dn.apply(*ins, out)
    torch.cuda.synchronize()
    assert torch.equal(out, ref)
    dn.close()


def test_inference_image_matches_oracle(ctx):
    """vvpt_denoiser_apply's output image, pixel by pixel, against the
    oracle's forward pass with the same BF16 rounding points. The yardstick is
    what BF16 rounding itself moves: the oracle's exact forward pass lies
    0.7-0.9 % (L2) from its BF16 one on these inputs. The GPU image must lie
    no farther from the BF16 oracle than that, and 99 % of pixel channels
    within 5e-2. Measured: 0.02 % on 32 x 48; 0.64 % on 64 x 96, where the
    GPU sits as far from the BF16 oracle as the exact pass does (a rounding
    point the restatement does not reproduce there)."""
    rng = np.random.default_rng(11)
    dn = Denoiser(ctx, seed=3)
    p = dn.params()
    for h, w in ((64, 96), (32, 48)):
        rad = rng.gamma(1.0, 0.6, (h, w, 4)).astype(np.float32)
        alb = rng.uniform(0, 1, (h, w, 4)).astype(np.float32)
        nrm = rng.uniform(0, 1, (h, w, 4)).astype(np.float32)
        out = _cuda(np.zeros((h, w, 4)))
        dn.apply(_cuda(rad), _cuda(alb), _cuda(nrm), out)
        got = out.cpu().numpy().astype(np.float64)
        want = D.forward_image(p, rad[None], alb[None], nrm[None])[0]
        exact = D.forward_image(p, rad[None], alb[None], nrm[None], exact=True)[0]
        assert (got[..., 3] == 1.0).all()
        a, b, x = got[..., :3], want[..., :3], exact[..., :3]
        band = np.linalg.norm(x - b) / np.linalg.norm(b)
        err = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert err <= band, (err, band)
        rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-2)
        assert np.percentile(rel, 99) <= 5e-2, np.sort(rel.ravel())[-5:]
    dn.close()
