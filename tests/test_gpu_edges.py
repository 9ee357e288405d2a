"""Edge cases of the fused particles -> P_l path (every tile shape).

* non-finite coordinates and coordinates beyond 2^30 cells are dropped and
  counted (gbp_deposit_stats.n_nonfinite), the rest are deposited exactly as
  a catalogue without them;
* positions outside [0, L) -- negative, exactly L, a few boxes away -- wrap
  periodically, so the result equals that of the wrapped catalogue;
* an empty catalogue runs, keeps the exact mode counts, and gives the 0/0 of
  an empty mesh (NaN), as the reference's delta/mean would;
* a single particle gives the flat spectrum of one point (float64 oracle).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

N, BOX = 64, 500.0


def _runs(x, y, z, mas="tsc", interlace=True):
    from gbpowspec import PkConfig, PowerSpectrum, _native, read_stats
    cfg = PkConfig(n_mesh=N, box_size=BOX, mas=mas, interlace=interlace)
    out = []
    for tiles in _native.tile_variants(N):
        r = PowerSpectrum(cfg, tiles=tiles).run(x, y, z)
        torch.cuda.synchronize()
        out.append((r.pk.clone(), r.nmodes.clone(), read_stats(r.stats)))
    return out


def _same(a, b):
    return torch.equal(torch.nan_to_num(a, nan=-7.0), torch.nan_to_num(b, nan=-7.0))


def test_nonfinite_and_far_particles_are_dropped_and_counted():
    from gbpowspec.synth import lognormal_catalogue
    x, y, z = (torch.from_numpy(a).cuda() for a in lognormal_catalogue(50_000, BOX, grid=32, seed=3))
    clean = _runs(x, y, z)
    bad = torch.tensor([float("nan"), float("inf"), -float("inf"), 1e38, -1e38], device="cuda")
    good = torch.full_like(bad, 10.0)
    # each bad value in one coordinate of an otherwise valid particle
    xb = torch.cat([x, bad, good, good])
    yb = torch.cat([y, good, bad, good])
    zb = torch.cat([z, good, good, bad])
    dirty = _runs(xb, yb, zb)
    for (pc, nc, sc), (pd, nd, sd) in zip(clean, dirty):
        assert _same(pc, pd) and torch.equal(nc, nd)
        assert sd.n_kept == sc.n_kept == x.numel()
        assert sd.n_nonfinite == 3 * bad.numel()
        assert sd.mass[0] == sc.mass[0]


def test_positions_outside_the_box_wrap_periodically():
    from gbpowspec.synth import lognormal_catalogue
    x, y, z = (torch.from_numpy(a).cuda() for a in lognormal_catalogue(40_000, BOX, grid=32, seed=5))
    ref = _runs(x, y, z)
    # shift by whole boxes: float32 x + k L is exact for these magnitudes only when k L is a power of
    # two multiple of the spacing; use k in {-2, -1, 1, 3} and compare with the catalogue wrapped by
    # the same float32 arithmetic
    k = torch.tensor([-2.0, -1.0, 1.0, 3.0], device="cuda")[torch.arange(x.numel(), device="cuda") % 4]
    xs = x + k * BOX
    wrapped = torch.remainder(xs, BOX)
    a = _runs(xs, y, z)
    b = _runs(wrapped, y, z)
    for (pa, na, sa), (pb, nb, sb) in zip(a, b):
        assert torch.equal(na, nb)
        assert sa.n_kept == sb.n_kept == x.numel()
        # the grid coordinate of x + kL and of its wrap differ in float32 rounding only
        full = na.cpu().numpy() > 0
        np.testing.assert_allclose(pa.cpu().numpy()[full], pb.cpu().numpy()[full], rtol=1e-4, atol=0)
    # particles exactly at L are at node 0 of the periodic mesh
    edge = torch.full((1000,), BOX, device="cuda")
    zero = torch.zeros(1000, device="cuda")
    yy = torch.rand(1000, device="cuda") * BOX
    for (pa, _, sa), (pb, _, sb) in zip(_runs(edge, yy, yy), _runs(zero, yy, yy)):
        assert _same(pa, pb) and sa.mass[0] == sb.mass[0]


def test_empty_catalogue():
    from gbpowspec import PkConfig
    from oracle import truth_f64 as T
    e = torch.zeros(0, device="cuda")
    ref_counts = T.power_multipoles(np.zeros(1, np.float32), np.zeros(1, np.float32), np.zeros(1, np.float32), None,
                                    box_size=BOX, n_mesh=N, mas=3, interlace=True,
                                    kedges_grid=PkConfig(n_mesh=N, box_size=BOX).kedges_grid())["nmodes"]
    for pk, nm, st in _runs(e, e, e):
        assert st.n_kept == 0 and st.mass[0] == 0.0
        np.testing.assert_array_equal(nm.cpu().numpy(), ref_counts)
        assert not np.isfinite(pk[:, 0].cpu().numpy()).any()


def test_single_particle_against_fp64():
    from gbpowspec import PkConfig
    from oracle import truth_f64 as T
    p = np.array([123.4567], np.float32), np.array([0.25], np.float32), np.array([499.9], np.float32)
    cfg = PkConfig(n_mesh=N, box_size=BOX, mas="pcs", interlace=True)
    ref = T.power_multipoles(*p, None, box_size=BOX, n_mesh=N, mas=4, interlace=True, kedges_grid=cfg.kedges_grid())
    full = ref["nmodes"] > 0
    amp = np.abs(ref["pk"][full, 0] + ref["shot"]) + ref["shot"]
    for pk, nm, st in _runs(*(torch.from_numpy(a).cuda() for a in p), mas="pcs"):
        assert st.n_kept == 1
        np.testing.assert_array_equal(nm.cpu().numpy(), ref["nmodes"])
        got = pk.cpu().numpy()[full]
        for l in range(3):
            assert np.all(np.abs(got[:, l] - ref["pk"][full, l]) <= 1e-5 * amp), l
