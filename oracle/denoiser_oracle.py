"""ORACLE — test infrastructure only (tests/ and bench.py's CPU leg).

NumPy restatement of the learned denoiser of vviewer_gb300/csrc/denoise.cu:
the 5-level U-Net's forward pass, L1 loss in the log domain and backward
pass, with the GPU's BF16 rounding points reproduced (features, weights,
every BF16 activation and gradient) and sums in float64. The reference has no
counterpart (its denoising step calls OpenImageDenoise,
VulkanRendererPathTracing.cpp:985-1018); this restatement checks the GPU's
gradients, and `exact=True` (no BF16 rounding) is checked against finite
differences.
"""
from __future__ import annotations

import numpy as np

LEVELS = 5
CH = [32, 48, 64, 96, 128]
IN_CH = 16
OUT_CH = 16


def layers():
    """(cin, cout, relu) per layer, in parameter order."""
    out = []
    prev = IN_CH
    for c in CH:
        out += [(prev, c, True), (c, c, True)]
        prev = c
    for lv in range(LEVELS - 2, -1, -1):
        out += [(CH[lv + 1] + CH[lv], CH[lv], True), (CH[lv], CH[lv], True)]
    out.append((CH[0], OUT_CH, False))
    return out


def unpack_params(flat: np.ndarray):
    """[(W [cout, 3, 3, cin], b [cout]) ...] from the flat parameter vector."""
    res, off = [], 0
    for cin, cout, _ in layers():
        n = cout * 9 * cin
        W = flat[off:off + n].reshape(cout, 3, 3, cin)
        off += n
        b = flat[off:off + cout]
        off += cout
        res.append((W, b))
    assert off == flat.size
    return res


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to bfloat16 (nearest even), returned as float64."""
    f = np.ascontiguousarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


class _R:
    def __init__(self, exact: bool):
        self.exact = exact

    def __call__(self, x):
        return np.asarray(x, dtype=np.float64) if self.exact else bf16(x)


def _shifted(x: np.ndarray, dy: int, dx: int) -> np.ndarray:
    """x[n, y + dy, x + dx, c] with zeros outside."""
    n, h, w, c = x.shape
    out = np.zeros_like(x)
    ys, yd = (slice(dy, h), slice(0, h - dy)) if dy >= 0 else (slice(0, h + dy), slice(-dy, h))
    xs, xd = (slice(dx, w), slice(0, w - dx)) if dx >= 0 else (slice(0, w + dx), slice(-dx, w))
    out[:, yd, xd, :] = x[:, ys, xs, :]
    return out


def conv3x3(x: np.ndarray, W: np.ndarray) -> np.ndarray:
    """sum over taps and input channels; W [cout, 3, 3, cin]."""
    n, h, w, _ = x.shape
    out = np.zeros((n, h, w, W.shape[0]))
    for ky in range(3):
        for kx in range(3):
            out += _shifted(x, ky - 1, kx - 1) @ W[:, ky, kx, :].T
    return out


def conv3x3_input_grad(dy: np.ndarray, W: np.ndarray) -> np.ndarray:
    n, h, w, _ = dy.shape
    out = np.zeros((n, h, w, W.shape[3]))
    for ky in range(3):
        for kx in range(3):
            out += _shifted(dy, 1 - ky, 1 - kx) @ W[:, ky, kx, :]
    return out


def conv3x3_weight_grad(dy: np.ndarray, x: np.ndarray) -> np.ndarray:
    cout, cin = dy.shape[3], x.shape[3]
    g = np.zeros((cout, 3, 3, cin))
    dyf = dy.reshape(-1, cout)
    for ky in range(3):
        for kx in range(3):
            g[:, ky, kx, :] = dyf.T @ _shifted(x, ky - 1, kx - 1).reshape(-1, cin)
    return g


def pool(x):
    n, h, w, c = x.shape
    return x.reshape(n, h // 2, 2, w // 2, 2, c).mean(axis=(2, 4))


def up(x):
    return x.repeat(2, axis=1).repeat(2, axis=2)


def features(rad, alb, nrm, R):
    """x0 [n, h, w, 16] from RGBA arrays [n, h, w, 4]."""
    n, h, w, _ = rad.shape
    x = np.zeros((n, h, w, IN_CH))
    x[..., 0:3] = np.log1p(np.maximum(rad[..., :3].astype(np.float32), 0.0).astype(np.float32)).astype(np.float32)
    x[..., 3:6] = alb[..., :3]
    x[..., 6:9] = nrm[..., :3]
    return R(x)


def forward_image(flat_params, rad, alb, nrm, exact=False):
    """The denoised image vvpt_denoiser_apply returns: the network's forward
    pass with the GPU's rounding points (BF16 features, weights and hidden
    activations; the output layer's sums kept in full precision), then
    expm1(max(y, 0)) per radiance channel and alpha 1. [n, h, w, 4] float64."""
    R = _R(exact)
    P = unpack_params(np.asarray(flat_params, dtype=np.float64))
    L = layers()
    Wq = [(R(W), b.astype(np.float32).astype(np.float64)) for W, b in P]

    def fwd(li, x):
        W, b = Wq[li]
        z = conv3x3(x, W) + b
        return R(np.maximum(z, 0.0)) if L[li][2] else z

    xs, es, ds = [None] * LEVELS, [None] * LEVELS, {}
    xs[0] = features(rad, alb, nrm, R)
    for lv in range(LEVELS):
        if lv > 0:
            xs[lv] = R(pool(es[lv - 1]))
        es[lv] = fwd(2 * lv + 1, fwd(2 * lv, xs[lv]))
    for lv in range(LEVELS - 2, -1, -1):
        coarse = es[LEVELS - 1] if lv == LEVELS - 2 else ds[lv + 1]
        li = 10 + 2 * (LEVELS - 2 - lv)
        ds[lv] = fwd(li + 1, fwd(li, np.concatenate([up(coarse), es[lv]], axis=-1)))
    y = fwd(len(L) - 1, ds[0])
    out = np.ones(y.shape[:3] + (4,))
    out[..., :3] = np.expm1(np.maximum(y[..., :3], 0.0))
    return out


def loss_and_grads(flat_params, rad, alb, nrm, target, exact=False):
    """Loss and flat gradient with the GPU's rounding points (exact=False)."""
    R = _R(exact)
    P = unpack_params(np.asarray(flat_params, dtype=np.float64))
    L = layers()
    Wq = [(R(W), b.astype(np.float32).astype(np.float64)) for W, b in P]

    def fwd(li, x):
        W, b = Wq[li]
        z = conv3x3(x, W) + b
        return R(np.maximum(z, 0.0)) if L[li][2] else z

    xs, as_, es = [None] * LEVELS, [None] * LEVELS, [None] * LEVELS
    us, bs, ds = {}, {}, {}
    xs[0] = features(rad, alb, nrm, R)
    for lv in range(LEVELS):
        if lv > 0:
            xs[lv] = R(pool(es[lv - 1]))
        as_[lv] = fwd(2 * lv, xs[lv])
        es[lv] = fwd(2 * lv + 1, as_[lv])
    for lv in range(LEVELS - 2, -1, -1):
        coarse = es[LEVELS - 1] if lv == LEVELS - 2 else ds[lv + 1]
        us[lv] = np.concatenate([up(coarse), es[lv]], axis=-1)
        li = 10 + 2 * (LEVELS - 2 - lv)
        bs[lv] = fwd(li, us[lv])
        ds[lv] = fwd(li + 1, bs[lv])
    y = fwd(len(L) - 1, ds[0])
    t = np.log1p(np.maximum(target[..., :3].astype(np.float32), 0.0).astype(np.float32)).astype(np.float32)
    diff = y[..., :3] - t
    npix = diff.shape[0] * diff.shape[1] * diff.shape[2]
    loss = np.abs(diff).sum() / (3 * npix)
    dy = np.zeros_like(y)
    dy[..., :3] = np.sign(diff) / (3.0 * npix)
    dy = R(dy)

    grads = [None] * len(L)

    def back(li, dz, x_in, mask):
        W, _ = Wq[li]
        grads[li] = (conv3x3_weight_grad(dz, x_in), dz.reshape(-1, dz.shape[-1]).sum(0))
        if mask is None:
            return R(conv3x3_input_grad(dz, W))
        return R(conv3x3_input_grad(dz, W) * (mask > 0))

    gd = back(len(L) - 1, dy, ds[0], ds[0])
    gskip = {}
    ge4 = None
    for lv in range(LEVELS - 1):
        li = 10 + 2 * (LEVELS - 2 - lv)
        gb = back(li + 1, gd, bs[lv], bs[lv])
        gu = back(li, gb, us[lv], us[lv])
        cc = CH[lv + 1]
        n, h, w, _ = gu.shape
        gcoarse = R(gu[..., :cc].reshape(n, h // 2, 2, w // 2, 2, cc).sum(axis=(2, 4)))
        gskip[lv] = gu[..., cc:]
        if lv == LEVELS - 2:
            ge4 = gcoarse
        else:
            gd = gcoarse
    gx_next = None
    for lv in range(LEVELS - 1, -1, -1):
        if lv == LEVELS - 1:
            ge = ge4
        else:
            ge = R((gskip[lv] + 0.25 * up(gx_next)) * (es[lv] > 0))
        ga = back(2 * lv + 1, ge, as_[lv], as_[lv])
        W, _ = Wq[2 * lv]
        grads[2 * lv] = (conv3x3_weight_grad(ga, xs[lv]), ga.reshape(-1, ga.shape[-1]).sum(0))
        if lv > 0:
            gx_next = R(conv3x3_input_grad(ga, W))
    flat = np.concatenate([np.concatenate([gw.reshape(-1), gb]) for gw, gb in grads])
    return loss, flat
