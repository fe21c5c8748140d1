"""Tables of the low-discrepancy sampler (VVPT_RENDER_SAMPLER_PMJ) and the
oracle's PMJ estimator, on the CPU. The reference's own tables are data
blobs missing from its tree (math/PMJSequences.cpp, math/BlueNoise.cpp), so
these check the defining properties of the regenerated ones: every
power-of-two prefix of a (0,2) sequence is stratified in all elementary
intervals, and each blue-noise texture is a permutation of the ranks with
little low-frequency energy."""
import numpy as np
import pytest

from oracle import oracle
from vviewer_gb300 import scenes
from vviewer_gb300.renderer import sampler_tables


@pytest.fixture(scope="module")
def tables():
    return sampler_tables()


def test_table_shapes_and_range(tables):
    pmj, bn = tables
    assert pmj.shape == (16, 16384, 2) and bn.shape == (48, 128, 128)
    assert pmj.min() >= 0.0 and pmj.max() < 1.0
    assert bn.min() >= 0.0 and bn.max() < 1.0
    # deterministic: the same tables on every call
    pmj2, bn2 = sampler_tables()
    assert (pmj2 == pmj).all() and (bn2 == bn).all()


@pytest.mark.parametrize("seq", [0, 7, 15])
def test_pmj_prefixes_are_02_nets(tables, seq):
    """For every m <= 14 the first 2^m points put exactly one point in each
    elementary interval of area 2^-m (all 2^a x 2^(m-a) grids)."""
    pts = tables[0][seq].astype(np.float64)
    for m in range(15):
        n = 1 << m
        p = pts[:n]
        for a in range(m + 1):
            ix = np.floor(p[:, 0] * (1 << a)).astype(np.int64)
            iy = np.floor(p[:, 1] * (1 << (m - a))).astype(np.int64)
            cells = np.bincount(ix * (1 << (m - a)) + iy, minlength=n)
            assert (cells == 1).all(), (seq, m, a)


def test_sequences_differ(tables):
    pmj = tables[0]
    assert not np.allclose(pmj[0], pmj[1])


@pytest.mark.parametrize("tex", [0, 23, 47])
def test_blue_noise_is_a_rank_permutation_with_little_low_frequency_energy(tables, tex):
    b = tables[1][tex].astype(np.float64)
    assert (np.sort(b.ravel()) == np.arange(128 * 128) / (128 * 128)).all()
    spec = np.abs(np.fft.fft2(b - b.mean())) ** 2
    f = np.fft.fftfreq(128)
    r = np.sqrt(f[:, None] ** 2 + f[None, :] ** 2)
    low = spec[(r > 0) & (r < 0.1)].mean()
    high = spec[r > 0.3].mean()
    # white noise has a flat spectrum (ratio ~1); void-and-cluster pushes the
    # energy to high frequencies
    assert low < 0.1 * high, (low, high)


def test_oracle_pmj_estimator_agrees_with_rtgems():
    """Both samplers estimate the same image: on a small Cornell box the
    image means agree within the Monte Carlo noise, and the PMJ pixel
    estimates are at least as close to a high-spp reference."""
    e, info = scenes.cornell_box(1, 24, 24, 64, 8, 4)
    fs = e.scene.build()
    sd = e.scene.scene_data(info.width, info.height)
    pmj = oracle.render(fs, sd, info, sampler="pmj")["radiance"][..., :3].astype(np.float64)
    rtg = oracle.render(fs, sd, info)["radiance"][..., :3].astype(np.float64)
    info.samples = 2048
    ref = oracle.render(fs, sd, info)["radiance"][..., :3].astype(np.float64)
    assert abs(pmj.mean() - ref.mean()) < 0.02 * ref.mean()
    assert abs(rtg.mean() - ref.mean()) < 0.02 * ref.mean()
    e_pmj = np.sqrt(((pmj - ref) ** 2).mean())
    e_rtg = np.sqrt(((rtg - ref) ** 2).mean())
    assert e_pmj < 1.1 * e_rtg, (e_pmj, e_rtg)
