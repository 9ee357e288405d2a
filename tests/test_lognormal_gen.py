"""Device lognormal catalogue generator (gbp_lognormal).

CPU: its Philox4x32-10 block against the published known-answer vectors of
the Random123 distribution (Salmon et al., SC'11).  GPU: determinism, range,
and agreement in distribution with the host generator (same recipe, other
random numbers): the measured P_0(k) of the two agree within sample variance.
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
