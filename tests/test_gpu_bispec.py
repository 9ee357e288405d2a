"""Bispectrum (gbp_bispec) against the reference's own bispec (golden fixtures) and the FP64 estimator."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _lognormal_contrast(N, seed, amp=0.8):
    g = np.random.default_rng(seed).standard_normal((N, N, N))
    d = np.exp(amp * g)
    return (d / d.mean() - 1.0).astype(np.float32)


def _assert_close(got, want, rtol, what):
    got, want = np.asarray(got, np.float64), np.asarray(want, np.float64)
    err = np.abs(got - want) / np.abs(want)
    assert np.all(err <= rtol), (what, err.max())


def test_bispec_matches_reference(golden):
    """Drop-in bispec vs the fixtures of src/correlations.py:334-462 (float32 reference; N = 16, 32, 24)."""
    from gbpowspec import bispec
    for i in range(int(golden["bk_ncases"][0])):
        box, k1, k2 = golden[f"bk_{i}_args"]
        k, pk, th, bk, qk = bispec(golden[f"bk_{i}_delta"], box, k1, k2, golden[f"bk_{i}_theta"])
        np.testing.assert_allclose(k.cpu().numpy(), golden[f"bk_{i}_k"], rtol=2e-7)
        np.testing.assert_array_equal(th.cpu().numpy(), golden[f"bk_{i}_theta"])
        _assert_close(pk.cpu().numpy(), golden[f"bk_{i}_pk"], 1e-5, "P")
        _assert_close(bk.cpu().numpy(), golden[f"bk_{i}_b"], 1e-5, "B")
        _assert_close(qk.cpu().numpy(), golden[f"bk_{i}_q"], 1e-5, "Q")


@pytest.mark.parametrize("N,box,k1,k2,nt,mas", [(64, 1000.0, 0.05, 0.1, 12, 2), (128, 2500.0, 0.1, 0.05, 16, 3),
                                                (48, 500.0, 0.08, 0.12, 9, 2)])
def test_bispectrum_against_fp64(N, box, k1, k2, nt, mas):
    """Library (N = 64, 128) and cuFFT (N = 48) transforms: P, B, Q within 1e-5 of the FP64 estimator,
    mode counts exact."""
    from oracle import truth_f64 as T
    from gbpowspec import bispectrum
    d = _lognormal_contrast(N, seed=N)
    theta = np.linspace(0.0, np.pi, nt).astype(np.float32)
    k, pk, bk, qk, nm = bispectrum(d, box, k1, k2, theta, mas_order=mas)
    k6, p6, b6, q6, nm6 = T.bispec(d, box, k1, k2, theta, mas_order=mas)
    np.testing.assert_array_equal(nm.cpu().numpy(), nm6)
    _assert_close(pk.cpu().numpy(), p6, 1e-5, "P")
    _assert_close(bk.cpu().numpy(), b6, 1e-5, "B")
    _assert_close(qk.cpu().numpy(), q6, 1e-5, "Q")


def test_bispectrum_is_deterministic():
    from gbpowspec import bispectrum
    d = torch.from_numpy(_lognormal_contrast(128, seed=3)).cuda()
    theta = np.linspace(0.0, np.pi, 20).astype(np.float32)
    a = bispectrum(d, 2500.0, 0.1, 0.2, theta)
    b = bispectrum(d, 2500.0, 0.1, 0.2, theta)
    for x, y in zip(a, b):
        assert np.array_equal(x.cpu().numpy(), y.cpu().numpy(), equal_nan=True)
    # k3 up to 0.3 h/Mpc reaches past the 128^3 grid's corner: those shells are empty, P = 0/0 (as the reference)
    pk, nm = a[1].cpu().numpy(), a[4].cpu().numpy()
    assert np.array_equal(np.isnan(pk), nm == 0) and (nm == 0).any() and (nm > 0).any()


def test_compute_all_correlations_matches_reference(golden):
    """Drop-in compute_all_correlations vs the fixtures of src/correlations.py:464-637."""
    from gbpowspec import compute_all_correlations
    for i in range(int(golden["all_ncases"][0])):
        box, k1, k2 = golden[f"bk_{i}_args"]
        g = lambda name: golden[f"all_{i}_{name}"]
        k, pk, nmk, r, xi, nmx, kall, pkb, th, bk, qk = (
            t.cpu().numpy() for t in compute_all_correlations(golden[f"bk_{i}_delta"], box, g("sedges"), g("kedges"),
                                                              k1, k2, golden[f"bk_{i}_theta"]))
        np.testing.assert_array_equal(k, g("k"))
        np.testing.assert_array_equal(nmk, g("nmk"))
        np.testing.assert_array_equal(r, g("r"))
        np.testing.assert_array_equal(nmx, g("nmx"))
        np.testing.assert_array_equal(th, g("theta"))
        np.testing.assert_allclose(kall, g("kall"), rtol=2e-7)
        assert np.array_equal(np.isnan(pk), np.isnan(g("pk"))) and np.array_equal(np.isnan(xi), np.isnan(g("xi")))
        scale = np.abs(g("pk")[:, :1]) + 1e-30
        assert np.nanmax(np.abs(pk - g("pk")) / scale) < 1e-5
        # the first shell holds r = 0 (mu = 0 there), whose variance dominates its xi_2, xi_4: scale by all l
        assert np.nanmax(np.abs(xi - g("xi"))) <= 1e-5 * np.nanmax(np.abs(g("xi")))
        _assert_close(pkb, g("pkb"), 1e-5, "P")
        _assert_close(bk, g("b"), 1e-5, "B")
        _assert_close(qk, g("q"), 1e-5, "Q")
