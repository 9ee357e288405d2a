"""The serving loop on the GPU: every request's P_l(k) is the same alone and in the mix.

A stream of requests with different meshes, schemes, boxes and particle
counts runs through one Server (several lanes and classes in flight at
once); each result must equal, bit for bit, the same request served alone
by a fresh server, and agree with the FP64 oracle within the target
tolerances.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _requests():
    from gbpowspec.serve import Request
    from gbpowspec.synth import lognormal_catalogue
    rng = np.random.default_rng(5)
    out = []
    for i in range(12):
        n_mesh = (64, 128)[i % 2]
        mas = ("cic", "tsc")[(i // 2) % 2]
        box = float(rng.uniform(500, 2500))
        n = int(10 ** rng.uniform(4, 5.3))
        x, y, z = lognormal_catalogue(n, box, grid=32, seed=40 + i)
        out.append(Request(torch.from_numpy(x).pin_memory(), torch.from_numpy(y).pin_memory(),
                           torch.from_numpy(z).pin_memory(), box=box, n_mesh=n_mesh, mas=mas))
    return out


def test_same_alone_and_in_the_mix():
    from gbpowspec.serve import Server
    reqs = _requests()
    srv = Server(budget_bytes=8e9, lanes_per_class=2, capacity=200_000)
    tickets = [srv.submit(r) for r in reqs]
    mixed = {r.ticket: r for r in srv.drain(timeout=300)}
    assert len(mixed) == len(reqs) and all(r.error is None for r in mixed.values())
    assert max(len(c.slots) for c in srv.classes.values()) == 2        # requests overlapped
    srv.close()
    for q, mt in zip(reqs, tickets):
        alone_srv = Server(budget_bytes=8e9, lanes_per_class=1, capacity=200_000)
        t = alone_srv.submit(q)                         # (re-tickets q within the new server)
        (alone,) = alone_srv.drain(timeout=120)
        alone_srv.close()
        m = mixed[mt]
        assert alone.ticket == t and alone.error is None
        np.testing.assert_array_equal(alone.nmodes, m.nmodes)
        np.testing.assert_array_equal(np.nan_to_num(alone.pk, nan=-1.0), np.nan_to_num(m.pk, nan=-1.0))
        assert alone.n_kept == m.n_kept == q.n


def test_served_result_matches_fp64_oracle():
    from gbpowspec.batch import shell_edges
    from gbpowspec.serve import Request, Server
    from gbpowspec.synth import lognormal_catalogue
    from oracle import truth_f64 as T
    box, N = 800.0, 64
    x, y, z = lognormal_catalogue(50_000, box, grid=32, seed=77)
    srv = Server(budget_bytes=4e9, capacity=100_000)
    srv.submit(Request(x, y, z, box=box, n_mesh=N, mas="tsc"))
    (res,) = srv.drain(timeout=120)
    srv.close()
    ref = T.power_multipoles(x, y, z, None, box_size=box, n_mesh=N, mas=3, interlace=True,
                             kedges_grid=shell_edges(N))
    np.testing.assert_array_equal(res.nmodes, ref["nmodes"])
    full = res.nmodes > 0
    amp = np.abs(ref["pk"][full, 0] + ref["shot"]) + ref["shot"]
    for l in range(3):
        assert np.all(np.abs(res.pk[full, l] - ref["pk"][full, l]) <= 1e-5 * amp)


def test_budget_smaller_than_a_lane_is_refused():
    from gbpowspec.serve import Request, Server
    a = np.random.default_rng(0).uniform(0, 100, 1000).astype(np.float32)
    srv = Server(budget_bytes=1e6, capacity=10_000)
    srv.submit(Request(a, a, a, box=100.0, n_mesh=128))
    (res,) = srv.drain(timeout=60)
    assert res.error and "budget" in res.error
