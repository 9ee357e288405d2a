"""The fused particle -> P_l(k) pipeline against the FP64 oracle.

Tolerances (from the target spec): mode counts bit-exact; P_0 within 1e-5
relative per bin; P_2 and P_4 within 1e-5 of |P_0|; mode-averaged k within
1e-6 relative.  The oracle deposits, transforms and bins in float64 from the
same float32 grid coordinates.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

RTOL_P = 1e-5


def _cat(n, box, seed, grid=32, weights=False):
    from gbpowspec.synth import lognormal_catalogue
    x, y, z = lognormal_catalogue(n, box, grid=grid, seed=seed)
    w = None
    if weights:
        w = np.random.default_rng(seed).uniform(0.2, 2.0, n).astype(np.float32)
    return x, y, z, w


def _check(res, ref, kmean=True):
    """Relative errors are taken against the monopole amplitude before shot-noise
    subtraction: after it, P_0 can be ~0 in a bin and a relative error is meaningless."""
    nm = res.nmodes.cpu().numpy()
    np.testing.assert_array_equal(nm, ref["nmodes"])
    full = nm > 0
    pk = res.pk.cpu().numpy()
    # scale of the two terms of P_0 = raw - shot (a bin holding only k=0 has raw == 0)
    amp = np.abs(ref["pk"][full, 0] + ref.get("shot", 0.0)) + ref.get("shot", 0.0)
    amp = np.maximum(amp, 1e-9 * amp.max())
    for l in (0, 1, 2):
        err = np.abs(pk[full, l] - ref["pk"][full, l])
        assert np.all(err <= RTOL_P * amp), (l, (err / amp).max())
    if kmean:
        np.testing.assert_allclose(res.k_mean.cpu().numpy()[full], ref["kmean"][full], rtol=1e-6)


@pytest.mark.parametrize("mas", ["ngp", "cic", "tsc", "pcs"])
@pytest.mark.parametrize("interlace", [False, True])
@pytest.mark.parametrize("N", [32, 40])
def test_pipeline_matches_fp64_oracle(mas, interlace, N):
    from gbpowspec import PkConfig, PowerSpectrum
    from gbpowspec._lib import MAS
    from oracle import truth_f64 as T
    box = 300.0
    x, y, z, w = _cat(40_000, box, seed=N + MAS[mas], weights=(mas == "cic"))
    cfg = PkConfig(n_mesh=N, box_size=box, mas=mas, interlace=interlace)
    ps = PowerSpectrum(cfg)
    res = ps.run(*(torch.from_numpy(a).cuda() if a is not None else None for a in (x, y, z, w)))
    ref = T.power_multipoles(x, y, z, w, box_size=box, n_mesh=N, mas=MAS[mas], interlace=interlace,
                             kedges_grid=cfg.kedges_grid())
    _check(res, ref)


def test_pipeline_odd_mesh_and_fine_bins():
    from gbpowspec import PkConfig, PowerSpectrum
    from oracle import truth_f64 as T
    N, box = 33, 250.0
    x, y, z, w = _cat(30_000, box, seed=5)
    edges = np.linspace(0.0, 1.6 * np.pi * N / box, 97).astype(np.float32)
    cfg = PkConfig(n_mesh=N, box_size=box, mas="tsc", interlace=True, k_edges=tuple(edges.tolist()))
    res = PowerSpectrum(cfg).run(*(torch.from_numpy(a).cuda() for a in (x, y, z)))
    ref = T.power_multipoles(x, y, z, None, box_size=box, n_mesh=N, mas=3, interlace=True,
                             kedges_grid=cfg.kedges_grid())
    _check(res, ref)


def test_pipeline_is_bitwise_deterministic():
    from gbpowspec import PkConfig, PowerSpectrum
    x, y, z, _ = _cat(200_000, 1000.0, seed=11, grid=64)
    t = [torch.from_numpy(a).cuda() for a in (x, y, z)]
    ps = PowerSpectrum(PkConfig(n_mesh=64, box_size=1000.0, mas="tsc", interlace=True))
    assert ps.fused
    a = ps.run(*t).pk.clone()
    spec_a = ps.spec.clone()                     # the z,y-transformed spectra the binning read
    perm = torch.randperm(t[0].numel(), device="cuda")
    b = ps.run(*(u[perm].contiguous() for u in t)).pk.clone()
    assert torch.equal(ps.spec, spec_a)          # particle order does not matter
    assert torch.equal(a, b)


def test_shot_noise_and_mass_bookkeeping():
    from gbpowspec import PkConfig, PowerSpectrum, read_stats
    box, N = 500.0, 32
    x, y, z, w = _cat(25_000, box, seed=2, weights=True)
    t = [torch.from_numpy(a).cuda() for a in (x, y, z, w)]
    with_sn = PowerSpectrum(PkConfig(n_mesh=N, box_size=box, mas="cic", interlace=False, shot_noise=True))
    no_sn = PowerSpectrum(PkConfig(n_mesh=N, box_size=box, mas="cic", interlace=False, shot_noise=False))
    a = with_sn.run(*t).pk.cpu().numpy()
    b = no_sn.run(*t).pk.cpu().numpy()
    st = read_stats(with_sn.stats)
    w64 = w.astype(np.float64)
    np.testing.assert_allclose(st.mass[0], w64.sum(), rtol=1e-9)   # exact sum of 2^-s-quantised terms
    np.testing.assert_allclose(st.sum_w, w64.sum(), rtol=1e-7)
    np.testing.assert_allclose(st.sum_w2, (w64 * w64).sum(), rtol=1e-7)
    assert st.n_kept == x.size and st.n_nonfinite == 0
    shot = box ** 3 * st.sum_w2 / st.mass[0] ** 2
    np.testing.assert_allclose(b[:, 0] - a[:, 0], shot, rtol=1e-9)
    np.testing.assert_array_equal(a[:, 1:], b[:, 1:])


def test_ngp_occupancy_counts_are_exact():
    """NGP with unit weights puts integer counts in the cells: exact vs numpy."""
    from gbpowspec import mesh_deposit
    box, N = 100.0, 16
    rng = np.random.default_rng(9)
    p = rng.uniform(0, box, (3, 100_000)).astype(np.float32)
    p[0, :64] = np.float32(box) * np.arange(64, dtype=np.float32) / 64   # exact node and half-cell positions
    mesh, _ = mesh_deposit(*p, box_size=box, n_mesh=N, mas="ngp")
    inv = np.float32(N / box)
    u = [(c - np.float32(0.0)) * inv for c in p]
    idx = [np.mod(np.floor(c.astype(np.float64)) + (c.astype(np.float64) - np.floor(c) >= 0.5), N).astype(int)
           for c in u]
    want = np.zeros((N, N, N))
    np.add.at(want, tuple(idx), 1.0)
    np.testing.assert_array_equal(mesh[0].cpu().numpy(), want.astype(np.float32))


def test_empty_and_nonfinite_catalogues():
    from gbpowspec import mesh_deposit, read_stats
    mesh, st = mesh_deposit(np.zeros(0, np.float32), np.zeros(0, np.float32), np.zeros(0, np.float32),
                            box_size=10.0, n_mesh=8, mas="tsc", interlace=True)
    assert mesh.shape == (2, 8, 8, 8) and torch.count_nonzero(mesh) == 0
    x = np.array([1.0, np.nan, 3.0, np.inf], np.float32)
    mesh, st = mesh_deposit(x, np.ones(4, np.float32), np.ones(4, np.float32), box_size=10.0, n_mesh=8,
                            mas="cic")
    s = read_stats(st)
    assert s.n_nonfinite == 2 and s.n_kept == 2
    np.testing.assert_allclose(mesh.sum().item(), 2.0, rtol=1e-6)


def test_positions_on_box_faces_wrap():
    """x == L, x == 0 and x slightly outside all land on the periodic lattice."""
    from gbpowspec import mesh_deposit
    from oracle import truth_f64 as T
    box, N = 64.0, 16
    x = np.array([0.0, box, np.nextafter(np.float32(box), np.float32(0)), -0.25, box + 0.3, 7.5], np.float32)
    y = np.full_like(x, 3.0)
    z = np.full_like(x, 60.0)
    for mas, m in (("cic", 2), ("tsc", 3), ("pcs", 4)):
        mesh, _ = mesh_deposit(x, y, z, box_size=box, n_mesh=N, mas=mas, interlace=True)
        ref = T.deposit(x, y, z, None, N, np.float32(N / box), mas=m, interlace=True)
        np.testing.assert_allclose(mesh.cpu().numpy(), ref, rtol=0, atol=2e-7)
