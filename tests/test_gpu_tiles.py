"""Column tile shapes of the fused path give identical results.

The fixed-point scales of the deposit belong to 4x4-pencil blocks, not to
the tile, so every tile shape the library offers (the autotuner's choices)
must produce the same mode counts, the same deposit statistics and the same
P_l bit for bit: on lognormal catalogues for every scheme, one and two grids,
with weights, through PowerSpectrum and through batch lanes, and on a
clustered catalogue whose dense blocks take the 64-bit path.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _same(a, b):
    return torch.equal(torch.nan_to_num(a, nan=-7.0), torch.nan_to_num(b, nan=-7.0))


def _run_all(cfg, x, y, z, w=None):
    from gbpowspec import PowerSpectrum, _native
    out = {}
    for tiles in _native.tile_variants(cfg.n_mesh):
        ps = PowerSpectrum(cfg, tiles=tiles)
        assert ps.fused and ps.tiles == tiles
        r = ps.run(x, y, z, w)
        torch.cuda.synchronize()
        out[tiles] = (r.pk.clone(), r.nmodes.clone(), r.stats.clone())
    return out


@pytest.mark.parametrize("N", [64, 128, 256, 512])
@pytest.mark.parametrize("mas", ["ngp", "cic", "tsc", "pcs"])
@pytest.mark.parametrize("interlace", [False, True])
def test_tile_shapes_agree_bit_for_bit(N, mas, interlace):
    from gbpowspec import PkConfig, _lib
    from gbpowspec.synth import lognormal_catalogue_gpu
    n = {64: 60_000, 128: 400_000, 256: 1_000_000, 512: 2_000_000}[N]
    x, y, z = (t.contiguous() for t in lognormal_catalogue_gpu(n, 1000.0, grid=min(N, 128), seed=N + 7))
    w = torch.from_numpy(np.random.default_rng(N).uniform(0.5, 1.5, n).astype(np.float32)).cuda()
    cfg = PkConfig(n_mesh=N, box_size=1000.0, mas=mas, interlace=interlace)
    res = _run_all(cfg, x, y, z, w)
    ref = next(iter(res.values()))
    for tiles, (pk, nm, st) in res.items():
        assert torch.equal(nm, ref[1]), tiles
        assert torch.equal(st[:_lib.STATS_RESULT_BYTES], ref[2][:_lib.STATS_RESULT_BYTES]), tiles
        assert _same(pk, ref[0]), tiles


@pytest.mark.parametrize("N", [128, 256, 512])
def test_tile_shapes_agree_on_clumps(N):
    """Dense clumps (64-bit blocks) next to sparse blocks of the same tiles."""
    from gbpowspec import PkConfig, _lib
    rng = np.random.default_rng(3)
    box, H = 1000.0, 1000.0 / N
    cells = [(5, 9, 11), (6, 13, 200 % N), (N // 2, N // 2, 3)]
    parts = [rng.random((3, 500_000)) * box] + [np.asarray(c)[:, None] * H + rng.random((3, 200_000)) * H
                                                 for c in cells]
    p = np.concatenate(parts, axis=1).astype(np.float32) % np.float32(box)
    x, y, z = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in p)
    for mas in ("cic", "tsc"):
        res = _run_all(PkConfig(n_mesh=N, box_size=box, mas=mas, interlace=True), x, y, z)
        ref = next(iter(res.values()))
        for tiles, (pk, nm, st) in res.items():
            assert torch.equal(st[:_lib.STATS_RESULT_BYTES], ref[2][:_lib.STATS_RESULT_BYTES]), (mas, tiles)
            assert _same(pk, ref[0]), (mas, tiles)


def test_lanes_with_tiles_match_the_pipeline():
    from gbpowspec import PkConfig, PowerSpectrum, _native
    from gbpowspec.batch import BatchRunner, ParticleArena, shell_edges
    from gbpowspec.synth import lognormal_catalogue
    N, box = 256, 900.0
    cats = [lognormal_catalogue(n, box, grid=64, seed=40 + i) for i, n in enumerate((150_000, 310_000))]
    arena = ParticleArena(cats)
    arena.upload()
    jobs = arena.job_table(box, N)
    cfg = PkConfig(n_mesh=N, box_size=box, mas="tsc", interlace=True, k_edges_kf=tuple(shell_edges(N).tolist()))
    alone = [PowerSpectrum(cfg, tiles=None).run(*(torch.from_numpy(a).cuda() for a in c)).pk.clone() for c in cats]
    for tiles in _native.tile_variants(N) + [None, "auto"]:
        br = BatchRunner(N, capacity=310_000, mas="tsc", interlace=True, ells=(0, 2, 4), n_lanes=2, tiles=tiles)
        res = br.run(jobs)
        torch.cuda.synchronize()
        for i in range(len(cats)):
            assert _same(res.pk[i], alone[i]), (tiles, i)
        br.close()
