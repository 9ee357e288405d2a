"""The CPU oracle against fixtures produced by the reference's own source.

tests/golden/reference_outputs.npz was written by tests/golden/make_golden.py,
which runs jax-powspec's src/mas.py and src/correlations.py unmodified.  The
float32 restatement must reproduce it bit for bit; the FP64 truth oracle must
agree with it to float32 accuracy and count the same modes.
"""
import numpy as np
import pytest

from oracle import reference_f32 as R
from oracle import truth_f64 as T


@pytest.mark.parametrize("name", ["a", "b"])
@pytest.mark.parametrize("wrap", [1, 0])
def test_deposit_restatement_bitexact(golden, name, wrap):
    p, w, d0 = golden[f"dep_{name}_pos"], golden[f"dep_{name}_w"], golden[f"dep_{name}_delta0"]
    N, box, ox, oy, oz = golden[f"dep_{name}_meta"]
    N = int(N)
    got = R.cic_mas_vec(d0, p[:, 0], p[:, 1], p[:, 2], w, len(p), ox, oy, oz, box, N, bool(wrap))
    np.testing.assert_array_equal(got, golden[f"dep_{name}_vec_{wrap}"])
    s = slice(0, 64)
    got = R.cic_mas(d0, p[s, 0], p[s, 1], p[s, 2], w[s], 64, ox, oy, oz, box, N, bool(wrap))
    np.testing.assert_array_equal(got, golden[f"dep_{name}_scan_{wrap}"])


def test_powspec_restatement_bitexact(golden):
    for i in range(int(golden["pk_ncases"][0])):
        k, pk, nm = R.powspec_vec(golden[f"pk_{i}_delta"], golden[f"pk_{i}_box"][0], golden[f"pk_{i}_edges"])
        np.testing.assert_array_equal(k, golden[f"pk_{i}_k"])
        np.testing.assert_array_equal(nm, golden[f"pk_{i}_nmodes"])
        np.testing.assert_array_equal(pk, golden[f"pk_{i}_pk"])


def test_fundamental_restatement_bitexact(golden):
    for i in range(int(golden["fund_ncases"][0])):
        k, pk, nm = R.powspec_vec_fundamental(golden[f"fund_{i}_delta"], golden[f"fund_{i}_box"][0])
        np.testing.assert_array_equal(k, golden[f"fund_{i}_k"])
        np.testing.assert_array_equal(nm, golden[f"fund_{i}_nmodes"])
        np.testing.assert_array_equal(pk, golden[f"fund_{i}_pk"])


def test_pipeline_restatement(golden):
    p, N, box = golden["pipe_pos"], int(golden["pipe_N"][0]), golden["pipe_box"][0]
    d = R.cic_mas_vec(np.zeros((N, N, N), np.float32), p[:, 0], p[:, 1], p[:, 2], None, len(p), 0.0, 0.0, 0.0,
                      box, N, True)
    d = d / d.mean() - np.float32(1.0)
    np.testing.assert_allclose(d, golden["pipe_delta"], rtol=0, atol=2e-6)
    k, pk, nm = R.powspec_vec(golden["pipe_delta"], box, golden["pipe_edges"])
    np.testing.assert_array_equal(nm, golden["pipe_nmodes"])
    np.testing.assert_array_equal(pk, golden["pipe_pk"])


def test_truth_f64_matches_reference_estimator(golden):
    """FP64 truth (mas_order=2, delta given) vs the reference's float32 estimator."""
    for i in range(int(golden["pk_ncases"][0])):
        delta, box, edges = golden[f"pk_{i}_delta"], golden[f"pk_{i}_box"][0], golden[f"pk_{i}_edges"]
        kf = np.float32(np.float32(2 * np.pi) / np.float32(box))
        res = T.power(delta, box, (edges / kf).astype(np.float32), mas_order=2, normalize="none")
        np.testing.assert_array_equal(res["nmodes"], golden[f"pk_{i}_nmodes"].astype(np.int64))
        ref = golden[f"pk_{i}_pk"].astype(np.float64)
        full = res["nmodes"] > 0
        p0 = np.abs(ref[full, 0])[:, None]
        assert np.all(np.abs(res["pk"][full] - ref[full]) <= 2e-5 * np.maximum(p0, 1e-30) + 1e-12)
        assert np.all(np.isnan(ref[~full]))


@pytest.mark.parametrize("mas,expect", [(1, {5: 1.0}), (2, {5: 1.0, 6: 0.0}),
                                         (3, {4: 0.125, 5: 0.75, 6: 0.125}),
                                         (4, {4: 1 / 6, 5: 2 / 3, 6: 1 / 6, 7: 0.0})])
def test_bspline_known_answers(mas, expect):
    """A particle exactly on node 5 gets the textbook B-spline weights."""
    first, w = T.bspline(np.array([5.0]), mas, half=False)
    got = {int(first[0]) + r: float(wr[0]) for r, wr in enumerate(w)}
    assert got.keys() == expect.keys()
    for k in expect:
        assert abs(got[k] - expect[k]) < 1e-15


@pytest.mark.parametrize("mas", [1, 2, 3, 4])
def test_truth_deposit_conserves_mass(mas):
    rng = np.random.default_rng(mas)
    x, y, z = (rng.uniform(0, 50, 500).astype(np.float32) for _ in range(3))
    w = rng.uniform(0.1, 3, 500).astype(np.float32)
    m = T.deposit(x, y, z, w, 10, np.float32(10 / 50), mas=mas, interlace=True)
    np.testing.assert_allclose(m.sum(axis=(1, 2, 3)), w.astype(np.float64).sum(), rtol=1e-12)


def test_fast_cpu_stand_in_agrees_with_the_restatement():
    """oracle/reference_fast (the timed CPU stand-in) vs oracle/reference_f32 on one small mock."""
    from oracle import reference_f32 as R
    from oracle import reference_fast as F
    from gbpowspec.synth import lognormal_catalogue
    N, box = 32, 500.0
    x, y, z = lognormal_catalogue(30_000, box, grid=32, seed=3)
    kf = 2 * np.pi / box
    edges = np.arange(kf, np.pi * N / box, kf).astype(np.float32)
    d = R.cic_mas_vec(np.zeros((N, N, N), np.float32), x, y, z, None, x.size, 0.0, 0.0, 0.0, box, N, True)
    d = d / d.mean() - np.float32(1.0)
    k0, p0, n0 = R.powspec_vec(d, box, edges)
    k1, p1, n1 = F.reference_mock(x, y, z, box, N, edges)
    np.testing.assert_array_equal(n0, n1)
    np.testing.assert_allclose(k0, k1, rtol=0)
    np.testing.assert_allclose(p1[:, 0], p0[:, 0], rtol=1e-4)
    amp = np.abs(p0[:, 0])[:, None]
    assert np.all(np.abs(p1[:, 1:] - p0[:, 1:]) <= 1e-4 * amp)


def test_xi_restatement_matches_reference_fixtures(golden):
    """oracle/reference_f32 xi_vec and compute_2pt_correlations vs the reference's own outputs."""
    from oracle import reference_f32 as R
    for i in range(int(golden["xi_ncases"][0])):
        d, box, se = golden[f"xi_{i}_delta"], float(golden[f"xi_{i}_box"][0]), golden[f"xi_{i}_sedges"]
        r, xi, nm = R.xi_vec(d, box, se)
        np.testing.assert_array_equal(r, golden[f"xi_{i}_r"])
        np.testing.assert_array_equal(nm, golden[f"xi_{i}_nmodes"])
        np.testing.assert_array_equal(xi, golden[f"xi_{i}_xi"])
        k, pk, nmk, r2, xi2 = R.compute_2pt_correlations(d, box, se, golden[f"tpc_{i}_kedges"])
        np.testing.assert_array_equal(k, golden[f"tpc_{i}_k"])
        np.testing.assert_array_equal(pk, golden[f"tpc_{i}_pk"])
        np.testing.assert_array_equal(nmk, golden[f"tpc_{i}_nmodes"])
        np.testing.assert_array_equal(r2, golden[f"tpc_{i}_r"])
        np.testing.assert_array_equal(xi2, golden[f"tpc_{i}_xi"])


def test_bispec_restatement_bitexact(golden):
    """oracle/reference_f32.bispec reproduces the reference's own bispec (src/correlations.py:334-462)."""
    for i in range(int(golden["bk_ncases"][0])):
        box, k1, k2 = golden[f"bk_{i}_args"]
        k, pk, th, bk, qk = R.bispec(golden[f"bk_{i}_delta"], box, k1, k2, golden[f"bk_{i}_theta"])
        np.testing.assert_array_equal(k, golden[f"bk_{i}_k"])
        np.testing.assert_array_equal(pk, golden[f"bk_{i}_pk"])
        np.testing.assert_array_equal(bk, golden[f"bk_{i}_b"])
        np.testing.assert_array_equal(qk, golden[f"bk_{i}_q"])


def test_bispec_truth_f64_matches_reference(golden):
    """The FP64 bispectrum agrees with the reference's float32 one to float32 round-off."""
    for i in range(int(golden["bk_ncases"][0])):
        box, k1, k2 = golden[f"bk_{i}_args"]
        k, pk, bk, qk, nm = T.bispec(golden[f"bk_{i}_delta"], box, k1, k2, golden[f"bk_{i}_theta"])
        np.testing.assert_array_equal(k, golden[f"bk_{i}_k"])
        np.testing.assert_allclose(pk, golden[f"bk_{i}_pk"], rtol=2e-6)
        np.testing.assert_allclose(bk, golden[f"bk_{i}_b"], rtol=2e-6)
        np.testing.assert_allclose(qk, golden[f"bk_{i}_q"], rtol=2e-6)
        assert np.all(nm > 0)


def test_bispec_shell_decomposition():
    """Every shell of the drop-in is a run of elementary bins whose limits are exactly its own."""
    from gbpowspec.correlations import bispec_shells, _elementary_bins
    for box, k1, k2, nt in [(100.0, 0.15, 0.25, 6), (300.0, 0.1, 0.1, 7), (2500.0, 0.1, 0.2, 20)]:
        theta = np.linspace(0, np.pi, nt).astype(np.float32)
        k_all, kmin, kmax, _ = bispec_shells(box, k1, k2, theta)
        kr, kminr, kmaxr = R.bispec_shells(box, k1, k2, theta)
        np.testing.assert_array_equal(k_all, kr)
        np.testing.assert_array_equal(kmin, kminr)
        np.testing.assert_array_equal(kmax, kmaxr)
        edges, sb = _elementary_bins(kmin, kmax)
        assert np.all(np.diff(edges) > 0) and edges[-1] > max(kmax.max(), kmin.max())
        np.testing.assert_array_equal(edges[sb[:, 0]], kmin)
        np.testing.assert_array_equal(edges[sb[:, 1]], kmax)


def test_compute_all_correlations_restatement_bitexact(golden):
    """oracle/reference_f32.compute_all_correlations reproduces src/correlations.py:464-637."""
    names = ("k", "pk", "nmk", "r", "xi", "nmx", "kall", "pkb", "theta", "b", "q")
    for i in range(int(golden["all_ncases"][0])):
        box, k1, k2 = golden[f"bk_{i}_args"]
        res = R.compute_all_correlations(golden[f"bk_{i}_delta"], box, golden[f"all_{i}_sedges"],
                                         golden[f"all_{i}_kedges"], k1, k2, golden[f"bk_{i}_theta"])
        for name, v in zip(names, res):
            np.testing.assert_array_equal(np.asarray(v, np.float32), golden[f"all_{i}_{name}"], err_msg=name)
