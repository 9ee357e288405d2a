"""Batched runs through lanes (gbp_lane_* / gbp_batch_run) and the Python BatchRunner.

The pipeline is deterministic (integer deposit, fixed reduction orders), so a
mock gives the same bits whether it runs alone through PowerSpectrum, alone
through a lane, or in the middle of a batch of other mocks on several lanes
and streams; graph replay and eager launches agree bit for bit too.  These
are the "same alone and in the mix" checks, here with tolerance zero.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _cats(sizes, box, seed0=100, grid=32):
    from gbpowspec.synth import lognormal_catalogue
    return [lognormal_catalogue(int(n), box, grid=grid, seed=seed0 + i) for i, n in enumerate(sizes)]


def _same(a, b):
    a = torch.nan_to_num(a, nan=-7.0)
    b = torch.nan_to_num(b, nan=-7.0)
    return torch.equal(a, b)


def _alone(cat, N, box, mas, interlace, ells):
    """The single-mock pipeline on the same bins (exact integer edges in units of kF)."""
    from gbpowspec import PkConfig, PowerSpectrum
    from gbpowspec.batch import shell_edges
    cfg = PkConfig(n_mesh=N, box_size=box, mas=mas, interlace=interlace, ells=ells,
                   k_edges_kf=tuple(shell_edges(N).tolist()))
    x, y, z = (torch.from_numpy(a).cuda() for a in cat)
    r = PowerSpectrum(cfg).run(x, y, z)
    torch.cuda.synchronize()
    return r


@pytest.mark.parametrize("graphs", [True, False])
def test_batch_equals_single_mock_pipeline(graphs):
    from gbpowspec.batch import BatchRunner, ParticleArena
    N, box = 64, 600.0
    sizes = [30_000, 55_000, 12_345, 80_000, 41_000]
    cats = _cats(sizes, box)
    arena = ParticleArena(cats)
    arena.upload()
    jobs = arena.job_table(box, N)
    br = BatchRunner(N, capacity=max(sizes), mas="tsc", interlace=True, ells=(0, 2, 4), n_lanes=3, graphs=graphs)
    assert br.graphs == graphs
    res = br.run(jobs)
    torch.cuda.synchronize()
    for i, c in enumerate(cats):
        r = _alone(c, N, box, "tsc", True, (0, 2, 4))
        assert torch.equal(res.nmodes[i], r.nmodes)
        assert _same(res.pk[i], r.pk), i
        assert _same(res.kmean[i], r.k_mean), i
        st = res.deposit_stats()[i]
        assert st.n_kept == sizes[i]


def test_alone_and_in_the_mix_are_identical():
    """One mock alone on one lane vs the same mock inside a mixed batch on 4 lanes, twice."""
    from gbpowspec.batch import BatchRunner, ParticleArena
    from gbpowspec import _lib
    N = 64
    boxes = np.array([500.0, 900.0, 700.0, 1200.0, 650.0, 800.0, 1000.0])
    sizes = [20_000, 70_000, 35_000, 9_000, 64_000, 50_000, 27_000]
    cats = _cats(sizes, 500.0, seed0=300)
    cats = [tuple(a * np.float32(b / 500.0) for a in c) for c, b in zip(cats, boxes)]
    arena = ParticleArena(cats)
    arena.upload()
    jobs = arena.job_table(boxes, N)
    mix = BatchRunner(N, capacity=70_000, mas="cic", interlace=True, ells=(0, 2), n_lanes=4)
    a = mix.run(jobs)
    b = mix.run(jobs)
    torch.cuda.synchronize()
    solo = BatchRunner(N, capacity=70_000, mas="cic", interlace=True, ells=(0, 2), n_lanes=1)
    one = solo.alloc_result(len(sizes))
    for i in range(len(sizes)):
        solo.run_one(jobs, i, one)
    torch.cuda.synchronize()
    assert _same(a.pk, b.pk) and _same(a.pk, one.pk)
    assert _same(a.kmean, one.kmean)
    R = _lib.STATS_RESULT_BYTES
    assert torch.equal(a.stats[:, :R], one.stats[:, :R])
    assert torch.equal(a.nmodes, one.nmodes)


def test_run_mixed_mesh_sizes_concurrently():
    from gbpowspec.batch import BatchRunner, ParticleArena, run_mixed
    box = 800.0
    sizes = [40_000, 25_000, 60_000, 33_000]
    cats = _cats(sizes, box, seed0=500)
    arena = ParticleArena(cats)
    arena.upload()
    j64 = arena.job_table(box, 64, indices=[0, 2])
    j32 = arena.job_table(box, 32, indices=[1, 3])
    r64 = BatchRunner(64, capacity=60_000, n_lanes=2)
    r32 = BatchRunner(32, capacity=60_000, n_lanes=2)
    m64, m32 = run_mixed([(r64, j64), (r32, j32)])
    torch.cuda.synchronize()
    s64 = r64.run(j64)
    s32 = r32.run(j32)
    torch.cuda.synchronize()
    assert _same(m64.pk, s64.pk) and _same(m32.pk, s32.pk)


def test_batch_matches_fp64_oracle():
    from gbpowspec.batch import BatchRunner, ParticleArena, shell_edges
    from oracle import truth_f64 as T
    N, box = 32, 300.0
    cats = _cats([20_000, 45_000], box, seed0=700)
    arena = ParticleArena(cats)
    arena.upload()
    br = BatchRunner(N, capacity=45_000, mas="tsc", interlace=True, ells=(0, 2, 4), n_lanes=2)
    res = br.run(arena.job_table(box, N))
    torch.cuda.synchronize()
    for i, (x, y, z) in enumerate(cats):
        ref = T.power_multipoles(x, y, z, None, box_size=box, n_mesh=N, mas=3, interlace=True,
                                 kedges_grid=shell_edges(N))
        nm = res.nmodes[i].cpu().numpy()
        np.testing.assert_array_equal(nm, ref["nmodes"])
        full = nm > 0
        pk = res.pk[i].cpu().numpy()
        amp = np.abs(ref["pk"][full, 0] + ref["shot"]) + ref["shot"]
        for l in range(3):
            assert np.all(np.abs(pk[full, l] - ref["pk"][full, l]) <= 1e-5 * amp)


def test_lane_bytes_accounts_for_the_allocation():
    from gbpowspec.batch import BatchRunner
    want = BatchRunner.bytes_per_lane(64, capacity=100_000, mas="tsc", ells=(0, 2, 4))
    br = BatchRunner(64, capacity=100_000, mas="tsc", ells=(0, 2, 4), n_lanes=1)
    assert br.lane_bytes == want
    free0, _ = torch.cuda.mem_get_info()
    br2 = BatchRunner(64, capacity=100_000, mas="tsc", ells=(0, 2, 4), n_lanes=2)
    free1, _ = torch.cuda.mem_get_info()
    assert free0 - free1 >= 2 * want * 0.9
    br2.close()
    br.close()


def test_tune_lanes_returns_a_candidate():
    from gbpowspec.batch import ParticleArena, tune_lanes
    cats = _cats([30_000] * 6, 500.0, seed0=900)
    arena = ParticleArena(cats)
    arena.upload()
    best, rates = tune_lanes(64, arena.job_table(500.0, 64), capacity=30_000, candidates=(1, 2), repeats=1)
    assert best in (1, 2) and set(rates) == {1, 2} and all(v > 0 for v in rates.values())


def test_run_from_host_matches_upload_then_run():
    """Chunked uploads overlapping the lanes give the same bits as one upload before the batch."""
    from gbpowspec.batch import BatchRunner, ParticleArena
    from gbpowspec import _lib
    N, box = 64, 600.0
    sizes = [30_000, 12_000, 45_000, 8_000, 27_000, 39_000, 16_000]
    cats = _cats(sizes, box, seed0=700)
    arena = ParticleArena(cats)
    jobs = arena.job_table(box, N)
    runner = BatchRunner(N, capacity=45_000, mas="tsc", interlace=True, ells=(0, 2, 4), n_lanes=3)
    arena.upload()
    want = runner.run(jobs)
    torch.cuda.synchronize()
    arena.dev.zero_()
    for chunk in (None, 1, 2, 5):
        got = runner.run_from_host(arena, jobs, chunk=chunk)
        torch.cuda.synchronize()
        R = _lib.STATS_RESULT_BYTES
        assert _same(got.pk, want.pk) and torch.equal(got.nmodes, want.nmodes)
        assert torch.equal(got.stats[:, :R], want.stats[:, :R])
    runner.close()
