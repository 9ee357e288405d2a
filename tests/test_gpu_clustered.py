"""The fixed-point deposit under strong clustering.

The deposit fused with the z transform accumulates each column tile in
32-bit fixed point at a scale of the tile's own, 2^(s_g - ceil(log2 c)),
where c is the largest number of the tile's entries that cover one z plane:
a tile holding a dense clump quantises every contribution in the tile,
clump and background alike, about 2^-12 of the largest weight coarser than
a sparse tile.  These catalogues put 2^20 particles into a handful of cells
over a uniform background of 2^20 and check P_0,2,4 against the float64
estimator at 256^3, CIC and PCS, with and without interlacing, at the same
tolerance as everywhere else: P_0 within 1e-5 of |P_0 + shot| + shot and
P_2, P_4 within 1e-5 of that monopole amplitude, per bin; mode counts exact.
The deposited mass must also match the float64 mass to 1e-6.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

N, BOX = 256, 1000.0


def _clustered(n_bg, n_clump, cells, seed, spread):
    """Uniform background + `len(cells)` clumps, each `n_clump` particles uniform within `spread` cells
    of the lower corner of its cell; float32 positions in [0, BOX)."""
    rng = np.random.default_rng(seed)
    H = BOX / N
    parts = [rng.random((3, n_bg)) * BOX]
    for c in cells:
        corner = np.asarray(c, np.float64)[:, None] * H
        parts.append(corner + rng.random((3, n_clump)) * spread * H)
    p = np.concatenate(parts, axis=1)
    p = p[:, rng.permutation(p.shape[1])]
    top = np.nextafter(np.float32(BOX), np.float32(0))
    return [np.minimum(np.mod(a, BOX).astype(np.float32), top) for a in p]


CASES = {
    # five clumps of ~2^18 particles, each inside one cell
    "five_cells": dict(cells=[(10, 20, 30), (100, 7, 200), (128, 128, 128), (250, 250, 3), (60, 190, 77)],
                       spread=1.0),
    # one point mass: 2^20 particles within 1/1000 of a cell (every stencil nearly identical)
    "point_mass": dict(cells=[(37, 141, 222)], spread=1e-3),
    # two clumps in the same column tile, on different z planes
    "same_tile": dict(cells=[(64, 32, 10), (65, 33, 180)], spread=1.0),
}


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("mas", ["cic", "pcs"])
@pytest.mark.parametrize("interlace", [False, True])
def test_clustered_catalogue_against_fp64(case, mas, interlace):
    import fp64_torch as F
    from gbpowspec import PkConfig, PowerSpectrum, read_stats
    from gbpowspec.batch import shell_edges
    spec = CASES[case]
    n_clump = (1 << 20) // len(spec["cells"])
    x, y, z = (torch.from_numpy(a).cuda() for a in _clustered(1 << 20, n_clump, spec["cells"], seed=17,
                                                             spread=spec["spread"]))
    order = {"cic": 2, "pcs": 4}[mas]
    cfg = PkConfig(n_mesh=N, box_size=BOX, mas=mas, interlace=interlace, k_edges_kf=tuple(shell_edges(N).tolist()))
    ps = PowerSpectrum(cfg)
    assert ps.fused
    res = ps.run(x, y, z)
    torch.cuda.synchronize()
    pk = res.pk.cpu().numpy()
    mass = read_stats(res.stats).mass[0]
    ref = F.power_multipoles(x, y, z, box=BOX, N=N, mas=order, interlace=interlace, kedges_grid=shell_edges(N))
    np.testing.assert_array_equal(res.nmodes.cpu().numpy(), ref["nmodes"])
    np.testing.assert_allclose(mass, ref["mass"], rtol=1e-6)
    full = ref["nmodes"] > 0
    amp = np.abs(ref["pk"][full, 0] + ref["shot"]) + ref["shot"]
    for l in range(3):
        err = np.abs(pk[full, l] - ref["pk"][full, l]) / amp
        assert err.max() <= 1e-5, (l, float(err.max()))


@pytest.mark.parametrize("mas", ["cic", "tsc"])
def test_dense_mesh_every_tile_takes_the_64bit_path(mas):
    """8,388,608 uniform particles on a 64^3 mesh: thousands of entries cover every plane of every
    block, so every tile goes through the 64-bit kernel (many tiles per CTA); against float64, and
    the same bits for every tile shape."""
    import fp64_torch as F
    from gbpowspec import PkConfig, PowerSpectrum, _native, read_stats
    from gbpowspec.batch import shell_edges
    N, box, n = 64, 500.0, 1 << 23
    g = torch.Generator(device="cuda").manual_seed(9)
    x, y, z = (torch.rand(n, generator=g, device="cuda") * box for _ in range(3))
    order = {"cic": 2, "tsc": 3}[mas]
    cfg = PkConfig(n_mesh=N, box_size=box, mas=mas, interlace=True, k_edges_kf=tuple(shell_edges(N).tolist()))
    outs = []
    for tiles in _native.tile_variants(N):
        r = PowerSpectrum(cfg, tiles=tiles).run(x, y, z)
        torch.cuda.synchronize()
        outs.append((r.pk.clone(), r.stats.clone()))
    for pk, st in outs[1:]:
        assert torch.equal(st, outs[0][1])
        assert torch.equal(torch.nan_to_num(pk, nan=-7.0), torch.nan_to_num(outs[0][0], nan=-7.0))
    ref = F.power_multipoles(x, y, z, box=box, N=N, mas=order, interlace=True, kedges_grid=shell_edges(N))
    np.testing.assert_allclose(read_stats(outs[0][1]).mass[0], ref["mass"], rtol=1e-6)
    pk = outs[0][0].cpu().numpy()
    full = ref["nmodes"] > 0
    amp = np.abs(ref["pk"][full, 0] + ref["shot"]) + ref["shot"]
    for l in range(3):
        err = np.abs(pk[full, l] - ref["pk"][full, l]) / amp
        assert err.max() <= 1e-5, (l, float(err.max()))
