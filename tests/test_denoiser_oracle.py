"""The denoiser oracle (NumPy restatement of the U-Net, test infrastructure)
checked on the CPU: its backward pass against central finite differences of
its own forward pass (float64, no BF16 rounding), and its BF16 mode against
the exact mode."""
import numpy as np

from oracle import denoiser_oracle as D


def _inputs(rng, n=1, h=16, w=16):
    rad = rng.gamma(1.0, 0.5, (n, h, w, 4)).astype(np.float32)
    alb = rng.uniform(0, 1, (n, h, w, 4)).astype(np.float32)
    nrm = rng.uniform(0, 1, (n, h, w, 4)).astype(np.float32)
    tgt = (rad * rng.uniform(0.5, 1.5, rad.shape)).astype(np.float32)
    return rad, alb, nrm, tgt


def _params(rng):
    ps = []
    for cin, cout, relu in D.layers():
        std = np.sqrt(2.0 / (9 * cin)) if relu else 0.1 * np.sqrt(1.0 / (9 * cin))
        W = rng.normal(0, std, (cout, 3, 3, cin))
        if not relu:
            W[3:] = 0.0
        ps.append(np.concatenate([W.reshape(-1), rng.normal(0, 0.01, cout)]))
    return np.concatenate(ps)


def test_oracle_backward_matches_finite_differences():
    rng = np.random.default_rng(3)
    rad, alb, nrm, tgt = _inputs(rng)
    p = _params(rng)
    loss, g = D.loss_and_grads(p, rad, alb, nrm, tgt, exact=True)
    assert np.isfinite(loss) and loss > 0
    # a few parameters of every layer, central differences
    offs, off = [], 0
    for cin, cout, _ in D.layers():
        n = cout * 9 * cin
        offs.append((off, n))
        off += n + cout
    checked = 0
    for k, (o, n) in enumerate(offs):
        cout = D.layers()[k][1]
        rows = 3 if k == len(offs) - 1 else cout
        for idx in rng.integers(0, rows * n // cout, 2):
            i = o + int(idx)
            eps = 1e-5
            pp, pm = p.copy(), p.copy()
            pp[i] += eps
            pm[i] -= eps
            fd = (D.loss_and_grads(pp, rad, alb, nrm, tgt, exact=True)[0] -
                  D.loss_and_grads(pm, rad, alb, nrm, tgt, exact=True)[0]) / (2 * eps)
            assert abs(fd - g[i]) <= 1e-4 * max(abs(fd), abs(g[i])) + 1e-9, (k, i, fd, g[i])
            checked += 1
    assert checked == 2 * len(offs)


def test_bf16_mode_stays_close_to_exact():
    rng = np.random.default_rng(4)
    rad, alb, nrm, tgt = _inputs(rng, n=2)
    p = _params(rng)
    l0, g0 = D.loss_and_grads(p, rad, alb, nrm, tgt, exact=True)
    l1, g1 = D.loss_and_grads(p, rad, alb, nrm, tgt, exact=False)
    assert abs(l1 - l0) < 2e-2 * l0
    assert np.linalg.norm(g1 - g0) < 0.1 * np.linalg.norm(g0)
