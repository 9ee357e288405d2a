"""Device lognormal catalogue generator (gbp_lognormal, gbp_lognormal_field).

CPU: its Philox4x32-10 block against the published known-answer vectors of
the Random123 distribution (Salmon et al., SC'11).  GPU: determinism, range,
agreement in distribution with the host generator (same recipe, other
random numbers: the measured P_0(k) of the two agree within sample
variance), and the recipe itself, pinned statistically against its
definition (the reference's src/gauss_field.py:5-80 field from a given
P(k), src/populate_field.py:4-29 particles drawn from the density):

* the Gaussian field's measured power, mode by mode, against the input
  P_G(k) = A k exp(-(k/0.3)^2) within sample variance (each independent
  complex mode's |g_k|^2 is exponential with mean P_G(k));
* the field's lattice variance (1 by construction) and its zero mean;
* the particle counts per cell against the multinomial with probabilities
  proportional to 1 + delta_LN = exp(g - 1/2) (Pearson chi-square).
"""
import ctypes as C

import numpy as np
import pytest


def _philox(ctr, key):
    from gbpowspec import _lib
    lib = _lib.load()
    c, k, o = (C.c_uint * 4)(*ctr), (C.c_uint * 2)(*key), (C.c_uint * 4)()
    assert lib.gbp_philox4x32_10(c, k, o) == 0
    return list(o)


@pytest.mark.parametrize("ctr,key,want", [
    ([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
    ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
    ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
     [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]),
])
def test_philox4x32_10_known_answers(ctr, key, want):
    assert _philox(ctr, key) == want


@pytest.mark.gpu
def test_device_catalogue_is_deterministic_and_in_the_box():
    import torch
    from gbpowspec.synth import lognormal_catalogue_gpu
    box, n = 1000.0, 300_000
    a = lognormal_catalogue_gpu(n, box, grid=64, seed=7)
    b = lognormal_catalogue_gpu(n, box, grid=64, seed=7)
    c = lognormal_catalogue_gpu(n, box, grid=64, seed=8)
    torch.cuda.synchronize()
    for u, v in zip(a, b):
        assert torch.equal(u, v)
    assert not torch.equal(a[0], c[0])
    for u in a:
        assert float(u.min()) >= 0.0 and float(u.max()) < box
        assert abs(float(u.double().mean()) - box / 2) < 0.02 * box


@pytest.mark.gpu
def test_device_and_host_generators_agree_in_distribution():
    import torch
    from gbpowspec import PkConfig, PowerSpectrum
    from gbpowspec.synth import lognormal_catalogue, lognormal_catalogue_gpu
    box, n, N = 1000.0, 400_000, 64
    cfg = PkConfig(n_mesh=N, box_size=box, mas="cic", interlace=True, ells=(0,))
    ps = PowerSpectrum(cfg)
    dev, host = [], []
    for seed in range(4):
        d = lognormal_catalogue_gpu(n, box, grid=64, seed=100 + seed)
        dev.append(ps.run(*(t.contiguous() for t in d)).pk[:, 0].cpu().numpy())
        h = lognormal_catalogue(n, box, grid=64, seed=200 + seed)
        host.append(ps.run(*(torch.from_numpy(t).cuda() for t in h)).pk[:, 0].cpu().numpy())
    pd, ph = np.mean(dev, axis=0), np.mean(host, axis=0)
    sel = slice(2, 20)                                  # well-sampled shells below the field's cut-off
    ratio = pd[sel] / ph[sel]
    assert abs(float(np.mean(ratio)) - 1.0) < 0.05, ratio


@pytest.mark.gpu
def test_gaussian_field_power_matches_input_spectrum():
    from gbpowspec.synth import gaussian_power, lognormal_field_gpu
    grid, box = 64, 1000.0
    g, _ = lognormal_field_gpu(grid, box, seed=3)
    g = g.double().cpu().numpy()
    assert abs(g.mean()) < 1e-6
    assert abs(g.var() - 1.0) < 0.05                     # lattice variance sum_k P_G / V = 1
    G = np.fft.rfftn(g)
    kf = 2 * np.pi / box
    ki = np.fft.fftfreq(grid, d=1.0 / grid)
    kz = np.arange(grid // 2 + 1)
    k2 = ki[:, None, None] ** 2 + ki[None, :, None] ** 2 + kz[None, None, :] ** 2
    inner = (kz > 0) & (kz < grid // 2)                  # independent complex modes only
    sel = np.broadcast_to(inner, k2.shape)
    kk = np.sqrt(k2[sel]) * kf
    ratio = (np.abs(G[sel]) ** 2) * box ** 3 / grid ** 6 / gaussian_power(kk, box, grid)
    shell = np.floor(np.sqrt(k2[sel]) + 0.5).astype(int)
    z, used = [], 0
    for s in range(2, grid // 2):
        r = ratio[shell == s]
        z.append((r.mean() - 1.0) * np.sqrt(r.size))       # exponential: unit mean, unit variance
        used += r.size
    z = np.asarray(z)
    assert np.all(np.abs(z) < 5.0), z
    chi2 = float(np.mean(z ** 2))
    assert 0.3 < chi2 < 2.0, chi2
    assert abs(ratio.mean() - 1.0) < 5.0 / np.sqrt(used)


@pytest.mark.gpu
def test_catalogue_counts_follow_the_lognormal_density():
    import torch
    from gbpowspec.synth import lognormal_catalogue_gpu, lognormal_field_gpu
    grid, box, n, seed = 32, 500.0, 1_000_000, 5
    x, y, z = lognormal_catalogue_gpu(n, box, grid=grid, seed=seed, rsd_sigma=0.0)
    _, rho = lognormal_field_gpu(grid, box, seed=seed)
    torch.cuda.synchronize()
    H = box / grid
    idx = [np.clip(np.floor(t.double().cpu().numpy() / H).astype(np.int64), 0, grid - 1) for t in (x, y, z)]
    cells = (idx[0] * grid + idx[1]) * grid + idx[2]
    counts = np.bincount(cells, minlength=grid ** 3)
    assert counts.sum() == n                             # exactly n particles
    p = rho.double().cpu().numpy().ravel()
    p /= p.sum()
    expect = n * p
    chi2 = float(np.sum((counts - expect) ** 2 / expect))
    dof = grid ** 3 - 1
    zscore = (chi2 - dof) / np.sqrt(2.0 * dof)
    assert abs(zscore) < 5.0, zscore
    # a uniform density is rejected by far: the counts do follow rho
    uni = float(np.sum((counts - n / grid ** 3) ** 2 / (n / grid ** 3)))
    assert (uni - dof) / np.sqrt(2.0 * dof) > 50.0
