"""gbp_fft_power: the x pass of the library FFT fused with the binning.

It must count exactly the modes gbp_fft_r2c + gbp_power count, agree with
that path to float32 round-off, agree with the FP64 oracle within the
target tolerances, and be bitwise reproducible.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _meshes(N, G, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    m = torch.rand((G, N, N, N), generator=g, device="cuda", dtype=torch.float32)
    return m * 2.0 + 0.5


@pytest.mark.parametrize("N", [64, 128, 256, 512])
@pytest.mark.parametrize("G", [1, 2])
@pytest.mark.parametrize("ells", ["l0", "l02", "l024k"])
def test_fused_matches_two_step(N, G, ells):
    from gbpowspec import _lib, _native
    from gbpowspec.batch import shell_edges
    mask = {"l0": _lib.ELL0, "l02": _lib.ELL0 | _lib.ELL2,
            "l024k": _lib.ELL0 | _lib.ELL2 | _lib.ELL4 | _lib.KSUM}[ells]
    dev = torch.device("cuda", 0)
    mesh = _meshes(N, G, seed=N + G)
    plan = _native.fft_plan(N, G, dev)
    spec = torch.empty(plan.spectrum_floats, dtype=torch.float32, device=dev)
    bins = _native.bins_for(shell_edges(N), N, dev)
    mass = torch.tensor([float(mesh[0].double().sum()), float(mesh[-1].double().sum())], dtype=torch.float64,
                        device=dev)
    plan.execute(mesh, spec)
    want = _native.power(spec, G, bins, mas_order=2, ells=mask, z_pitch=plan.pitch, mass=mass)
    got = _native.fft_power(plan, mesh, spec, bins, mas_order=2, ells=mask, mass=mass)
    again = _native.fft_power(plan, mesh, spec, bins, mas_order=2, ells=mask, mass=mass)
    torch.cuda.synchronize()
    assert torch.equal(got.nmodes, want.nmodes)
    assert torch.equal(got.sums, again.sums)                    # bitwise reproducible
    w, g = want.sums.cpu().numpy(), got.sums.cpu().numpy()
    amp = np.abs(w[:, 0]) + 1e-300
    for l in range(3):
        assert np.all(np.abs(g[:, l] - w[:, l]) <= 2e-6 * amp), l
    if mask & _lib.KSUM:
        assert torch.equal(got.ksum, want.ksum)


def test_fused_1024_interlaced_matches_two_step():
    from gbpowspec import _lib, _native
    from gbpowspec.batch import shell_edges
    N, G = 1024, 2
    dev = torch.device("cuda", 0)
    mesh = _meshes(N, G, seed=5)
    plan = _native.fft_plan(N, G, dev)
    spec = torch.empty(plan.spectrum_floats, dtype=torch.float32, device=dev)
    bins = _native.bins_for(shell_edges(N), N, dev)
    mask = _lib.ELL0 | _lib.ELL2 | _lib.ELL4
    plan.execute(mesh, spec)
    want = _native.power(spec, G, bins, mas_order=4, ells=mask, z_pitch=plan.pitch)
    got = _native.fft_power(plan, mesh, spec, bins, mas_order=4, ells=mask)
    torch.cuda.synchronize()
    assert torch.equal(got.nmodes, want.nmodes)
    w, g = want.sums.cpu().numpy(), got.sums.cpu().numpy()
    amp = np.abs(w[:, 0])
    for l in range(3):
        assert np.all(np.abs(g[:, l] - w[:, l]) <= 2e-6 * amp), l


@pytest.mark.parametrize("mas", ["ngp", "cic", "tsc", "pcs"])
@pytest.mark.parametrize("interlace", [False, True])
def test_fused_pipeline_matches_fp64_oracle(mas, interlace):
    from gbpowspec import PkConfig, PowerSpectrum
    from gbpowspec._lib import MAS
    from gbpowspec.synth import lognormal_catalogue
    from oracle import truth_f64 as T
    N, box = 64, 400.0
    x, y, z = lognormal_catalogue(60_000, box, grid=32, seed=11 + MAS[mas])
    cfg = PkConfig(n_mesh=N, box_size=box, mas=mas, interlace=interlace)
    ps = PowerSpectrum(cfg)
    assert ps.fused
    res = ps.run(*(torch.from_numpy(a).cuda() for a in (x, y, z)))
    ref = T.power_multipoles(x, y, z, None, box_size=box, n_mesh=N, mas=MAS[mas], interlace=interlace,
                             kedges_grid=cfg.kedges_grid())
    nm = res.nmodes.cpu().numpy()
    np.testing.assert_array_equal(nm, ref["nmodes"])
    full = nm > 0
    pk = res.pk.cpu().numpy()
    amp = np.abs(ref["pk"][full, 0] + ref["shot"]) + ref["shot"]
    for l in range(3):
        err = np.abs(pk[full, l] - ref["pk"][full, l])
        assert np.all(err <= 1e-5 * amp), (l, (err / amp).max())
    np.testing.assert_allclose(res.k_mean.cpu().numpy()[full], ref["kmean"][full], rtol=1e-6)


@pytest.mark.parametrize("N", [64, 128, 256, 512])
@pytest.mark.parametrize("mas", ["ngp", "cic", "tsc", "pcs"])
@pytest.mark.parametrize("G", [1, 2])
def test_particles_power_matches_mesh_path(N, mas, G):
    """Deposit fused with the z pass vs gbp_deposit + gbp_fft_power on the same particles."""
    from gbpowspec import _lib, _native, read_stats
    from gbpowspec.batch import shell_edges
    from gbpowspec.synth import lognormal_catalogue
    dev = torch.device("cuda", 0)
    box = 700.0
    x, y, z = (torch.from_numpy(a).cuda() for a in lognormal_catalogue(150_000, box, grid=32, seed=N + G))
    w = torch.from_numpy(np.random.default_rng(N).uniform(0.5, 1.5, x.numel()).astype(np.float32)).cuda()
    inv = np.float32(N / box)
    m = _lib.MAS[mas]
    plan = _native.fft_plan(N, G, dev)
    bins = _native.bins_for(shell_edges(N), N, dev)
    mask = _lib.ELL0 | _lib.ELL2 | _lib.ELL4 | _lib.KSUM
    spec = torch.empty(plan.spectrum_floats, dtype=torch.float32, device=dev)
    mesh, st_mesh = _native.deposit(x, y, z, w, n_mesh=N, inv_cell=inv, mas=m, interlace=G == 2)
    want = _native.fft_power(plan, mesh, spec, bins, mas_order=m, ells=mask, mass=st_mesh)
    st = torch.zeros(_lib.STATS_BYTES, dtype=torch.uint8, device=dev)
    got = _native.particles_power(x, y, z, w, plan=plan, bins=bins, mas=m, ells=mask, inv_cell=inv, spec=spec,
                                  stats=st)
    torch.cuda.synchronize()
    assert torch.equal(got.nmodes, want.nmodes)
    assert torch.equal(got.ksum, want.ksum)
    a, b = read_stats(st), read_stats(st_mesh)
    assert a.n_kept == b.n_kept == x.numel()
    # both totals are exact sums of their meshes' fixed-point cells; the fused tiles quantise each
    # contribution at ~2^-(s_g - log2 entries) (about 2^-18 of the largest weight here) instead of 2^-s_g,
    # and stencil tails below half a step round to zero: the fused mass is ~2e-7 low
    np.testing.assert_allclose(a.mass[:G], b.mass[:G], rtol=1e-6)
    wv, gv = want.sums.cpu().numpy(), got.sums.cpu().numpy()
    amp = np.abs(wv[:, 0])
    for l in range(3):
        assert np.all(np.abs(gv[:, l] - wv[:, l]) <= 2e-6 * amp), l


def test_particles_power_1024_runs_and_counts_modes():
    from gbpowspec import _lib, _native
    from gbpowspec.batch import shell_edges
    dev = torch.device("cuda", 0)
    N, G, box, n = 1024, 2, 2000.0, 2_000_000
    gen = torch.Generator(device="cuda").manual_seed(3)
    x, y, z = (torch.rand(n, generator=gen, device="cuda") * box for _ in range(3))
    plan = _native.fft_plan(N, G, dev)
    bins = _native.bins_for(shell_edges(N), N, dev)
    spec = torch.empty(plan.spectrum_floats, dtype=torch.float32, device=dev)
    st = torch.zeros(_lib.STATS_BYTES, dtype=torch.uint8, device=dev)
    mask = _lib.ELL0 | _lib.ELL2 | _lib.ELL4
    got = _native.particles_power(x, y, z, None, plan=plan, bins=bins, mas=4, ells=mask,
                                  inv_cell=np.float32(N / box), spec=spec, stats=st)
    again = _native.particles_power(x, y, z, None, plan=plan, bins=bins, mas=4, ells=mask,
                                    inv_cell=np.float32(N / box), spec=spec, stats=st)
    torch.cuda.synchronize()
    assert torch.equal(got.sums, again.sums)
    # uniform particles: P_0 is shot noise, flat at L^3 / n after normalisation
    from gbpowspec import read_stats
    m = read_stats(st).mass[0]
    p0 = got.sums[:, 0].cpu().numpy() / got.nmodes.cpu().numpy() * box ** 3 / m ** 2
    mid = p0[10:100]                             # k < 0.2 k_Nyq: aliasing of the window is negligible
    assert np.all(np.isfinite(mid))
    np.testing.assert_allclose(mid.mean(), box ** 3 / n, rtol=0.03)
