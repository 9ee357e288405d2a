"""One-pass bucketing and its overflow rebuild.

The particle bucketing gives every tile bucket a fixed capacity (twice the
mean fill of a uniform catalogue of the launch's particle count, plus 64)
and fills it in one pass: the count a particle's atomic returns is its slot.  When a
bucket overflows (a dense clump), a scan of those counts and a second
scatter rebuild all buckets packed, and gbp_deposit_stats.flags says so.
The deposit sums exact integers, so the order of a bucket's entries, and
hence the path, cannot change a bit of the result:

* ordinary catalogues (lognormal, uniform) take the one-pass path, fused
  and mesh deposits alike;
* a clumped catalogue overflows when the buckets are sized for its own
  particle count and fits when they are sized for 32 times as many (a batch
  lane's capacity): both give the same P_l, mass and mesh, bit for bit, for
  every column tile shape.
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

N, BOX = 128, 500.0


def _clumped(n_bg, n_clump, seed):
    rng = np.random.default_rng(seed)
    H = BOX / N
    bg = rng.random((3, n_bg)) * BOX
    clump = (np.array([37.0, 90.0, 11.0])[:, None] + rng.random((3, n_clump)) * 0.5) * H
    p = np.concatenate([bg, clump], axis=1)[:, rng.permutation(n_bg + n_clump)]
    return [torch.from_numpy(a.astype(np.float32)).cuda() for a in p]


def test_ordinary_catalogues_fill_in_one_pass():
    from gbpowspec import PkConfig, PowerSpectrum, _lib, _native, read_stats
    from gbpowspec.synth import lognormal_catalogue
    x, y, z = (torch.from_numpy(a).cuda() for a in lognormal_catalogue(400_000, BOX, grid=64, seed=11,
                                                                           rsd_sigma=3.0))
    for tiles in _native.tile_variants(N):
        r = PowerSpectrum(PkConfig(n_mesh=N, box_size=BOX, mas="tsc", interlace=True), tiles=tiles).run(x, y, z)
        st = read_stats(r.stats)
        assert st.flags & _lib.STATS_REFILLED == 0, tiles
        assert st.n_kept == x.numel()
    mesh, stats = _native.deposit(x, y, z, None, n_mesh=N, inv_cell=float(np.float32(N / BOX)), mas=3,
                                  interlace=True)
    assert read_stats(stats).flags & _lib.STATS_REFILLED == 0


def test_overflow_rebuild_gives_the_same_power_bit_for_bit():
    from gbpowspec import PkConfig, PowerSpectrum, _lib, _native, read_stats
    from gbpowspec.batch import BatchRunner, ParticleArena
    x, y, z = _clumped(200_000, 30_000, seed=5)
    n = x.numel()
    cfg = PkConfig(n_mesh=N, box_size=BOX, mas="tsc", interlace=True, ells=(0, 2, 4))
    arena = ParticleArena([tuple(t.cpu().numpy() for t in (x, y, z))])
    arena.upload()
    jobs = arena.job_table(BOX, N)
    for tiles in _native.tile_variants(N):
        r = PowerSpectrum(cfg, tiles=tiles).run(x, y, z)
        torch.cuda.synchronize()
        st = read_stats(r.stats)
        assert st.flags & _lib.STATS_REFILLED, tiles                 # buckets sized for n: the clump overflows
        big = BatchRunner(N, capacity=32 * n, mas="tsc", interlace=True, ells=(0, 2, 4),
                          kedges_grid=cfg.kedges_grid(), n_lanes=1, tiles=tiles)
        res = big.run(jobs)
        torch.cuda.synchronize()
        sb = res.deposit_stats()[0]
        assert sb.flags & _lib.STATS_REFILLED == 0, tiles            # sized for 32 n: one pass
        assert torch.equal(res.pk[0].to(r.pk.dtype).cpu(), r.pk.cpu()), tiles
        assert torch.equal(res.nmodes[0].cpu(), r.nmodes.cpu())
        assert sb.mass[0] == st.mass[0] and sb.mass[1] == st.mass[1]
        big.close()


def test_overflow_rebuild_gives_the_same_mesh_bit_for_bit():
    from gbpowspec import _lib, _native, read_stats
    from gbpowspec.batch import ParticleArena
    x, y, z = _clumped(150_000, 30_000, seed=9)
    n = x.numel()
    inv_cell = float(np.float32(N / BOX))
    mesh, stats = _native.deposit(x, y, z, None, n_mesh=N, inv_cell=inv_cell, mas=4, interlace=True)
    torch.cuda.synchronize()
    assert read_stats(stats).flags & _lib.STATS_REFILLED
    # the same catalogue as a job with 32 n of capacity (buckets 32 times larger): one pass
    arena = ParticleArena([tuple(t.cpu().numpy() for t in (x, y, z))])
    arena.upload()
    jobs = arena.job_table(BOX, N)
    lib = _lib.load()
    ws_bytes = C.c_size_t(0)
    _lib.check(lib.gbp_deposit_workspace_size(32 * n, N, 4, 1, 0, C.byref(ws_bytes)), "workspace")
    ws = torch.empty(ws_bytes.value, dtype=torch.uint8, device="cuda")
    out = torch.empty((2, N, N, N), dtype=torch.float32, device="cuda")
    st2 = torch.empty(_lib.STATS_BYTES, dtype=torch.uint8, device="cuda")
    _lib.check(lib.gbp_deposit_job(C.c_void_p(jobs.data_ptr()), 32 * n, N, 4, 1, C.c_void_p(out.data_ptr()),
                                   C.c_void_p(st2.data_ptr()), C.c_void_p(ws.data_ptr()), ws_bytes.value,
                                   C.c_void_p(torch.cuda.current_stream().cuda_stream)), "gbp_deposit_job")
    torch.cuda.synchronize()
    s2 = read_stats(st2)
    assert s2.flags & _lib.STATS_REFILLED == 0
    assert torch.equal(out, mesh.reshape(out.shape))
    assert s2.mass[0] == read_stats(stats).mass[0]
