"""Drop-in functions on the GPU against the reference's own outputs.

Tolerances: mode counts and k-bin centres bit-exact; mesh values to float32
accumulation-order rounding; P_0 within 1e-5 relative per bin and P_2, P_4
within 1e-5 of |P_0| (the reference accumulates in float32 scatter order, the
GPU in fixed-point / FP32-then-float-float, so the last bits differ).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

RTOL_P = 1e-5


def _assert_pk(got, want, nmodes):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    full = np.asarray(nmodes) > 0
    assert np.all(np.isnan(got[~full])) and np.all(np.isnan(want[~full]))
    p0 = np.abs(want[full, 0])
    np.testing.assert_allclose(got[full, 0], want[full, 0], rtol=RTOL_P, atol=0)
    for l in (1, 2):
        assert np.all(np.abs(got[full, l] - want[full, l]) <= RTOL_P * p0), l


@pytest.mark.parametrize("name", ["a", "b"])
@pytest.mark.parametrize("wrap", [1, 0])
@pytest.mark.parametrize("variant", ["vec", "scan"])
def test_cic_dropins_match_reference(golden, name, wrap, variant):
    from gbpowspec import cic_mas, cic_mas_vec
    p, w, d0 = golden[f"dep_{name}_pos"], golden[f"dep_{name}_w"], golden[f"dep_{name}_delta0"]
    N, box, ox, oy, oz = golden[f"dep_{name}_meta"]
    N = int(N)
    if variant == "vec":
        got = cic_mas_vec(d0, p[:, 0], p[:, 1], p[:, 2], w, len(p), ox, oy, oz, box, N, bool(wrap))
    else:
        s = slice(0, 64)
        got = cic_mas(d0, p[s, 0], p[s, 1], p[s, 2], w[s], 64, ox, oy, oz, box, N, bool(wrap))
    want = golden[f"dep_{name}_{variant}_{wrap}"]
    got = got.cpu().numpy()
    assert got.shape == want.shape and got.dtype == np.float32
    scale = np.abs(want).max()
    np.testing.assert_allclose(got, want, rtol=0, atol=4e-7 * scale)
    # the fixed-point deposit is order independent: a permuted catalogue gives identical bits
    if variant == "vec":
        perm = np.random.default_rng(0).permutation(len(p))
        q, wq = p[perm], w[perm]
        got2 = cic_mas_vec(d0, q[:, 0], q[:, 1], q[:, 2], wq, len(q), ox, oy, oz, box, N, bool(wrap))
        assert torch.equal(got2.cpu(), torch.from_numpy(got))


def test_powspec_vec_matches_reference(golden):
    from gbpowspec import powspec_vec
    for i in range(int(golden["pk_ncases"][0])):
        delta, box, edges = golden[f"pk_{i}_delta"], golden[f"pk_{i}_box"][0], golden[f"pk_{i}_edges"]
        k, pk, nm = powspec_vec(delta, box, edges)
        np.testing.assert_array_equal(k.cpu().numpy(), golden[f"pk_{i}_k"])
        np.testing.assert_array_equal(nm.cpu().numpy(), golden[f"pk_{i}_nmodes"])
        _assert_pk(pk.cpu().numpy(), golden[f"pk_{i}_pk"], golden[f"pk_{i}_nmodes"])


def test_powspec_vec_fundamental_matches_reference(golden):
    from gbpowspec import powspec_vec_fundamental
    for i in range(int(golden["fund_ncases"][0])):
        k, pk, nm = powspec_vec_fundamental(golden[f"fund_{i}_delta"], golden[f"fund_{i}_box"][0])
        np.testing.assert_array_equal(nm.cpu().numpy(), golden[f"fund_{i}_nmodes"])
        np.testing.assert_allclose(k.cpu().numpy(), golden[f"fund_{i}_k"], rtol=2e-7)
        _assert_pk(pk.cpu().numpy(), golden[f"fund_{i}_pk"], golden[f"fund_{i}_nmodes"])


def test_reference_caller_pipeline(golden):
    """tests/correlations.py:42-50,78: deposit, normalise in float32, powspec_vec."""
    from gbpowspec import cic_mas_vec, powspec_vec
    p, N, box = golden["pipe_pos"], int(golden["pipe_N"][0]), golden["pipe_box"][0]
    d = cic_mas_vec(torch.zeros((N, N, N)), p[:, 0], p[:, 1], p[:, 2], np.ones(len(p), np.float32), len(p),
                    0.0, 0.0, 0.0, box, N, True)
    d = d / d.mean()
    d -= 1.0
    np.testing.assert_allclose(d.cpu().numpy(), golden["pipe_delta"], rtol=0, atol=3e-6)
    k, pk, nm = powspec_vec(golden["pipe_delta"], box, golden["pipe_edges"])
    np.testing.assert_array_equal(nm.cpu().numpy(), golden["pipe_nmodes"])
    _assert_pk(pk.cpu().numpy(), golden["pipe_pk"], golden["pipe_nmodes"])


def test_powspec_vec_against_fp64_truth_config1_shape():
    """Configuration-1 shape (128^3, 1,048,576 uniform particles, L=1000): counts
    bit-exact and P_0 within 1e-5 of the FP64 estimator on the same mesh."""
    from gbpowspec import cic_mas_vec, powspec_vec
    from gbpowspec.synth import uniform_catalogue
    from oracle import truth_f64 as T
    N, box = 128, 1000.0
    x, y, z = uniform_catalogue(1 << 20, box, seed=0)
    d = cic_mas_vec(torch.zeros((N, N, N)), x, y, z, np.ones(x.size, np.float32), x.size, 0.0, 0.0, 0.0,
                    box, N, True)
    d = d / d.mean() - 1.0
    kf = 2 * np.pi / box
    edges = np.arange(kf, np.pi * N / box, kf).astype(np.float32)
    k, pk, nm = powspec_vec(d, box, edges)
    kfe = np.float32(np.float32(2 * np.pi) / np.float32(box))
    ref = T.power(d.cpu().numpy(), box, (edges / kfe).astype(np.float32), mas_order=2, normalize="none")
    np.testing.assert_array_equal(nm.cpu().numpy().astype(np.int64), ref["nmodes"])
    _assert_pk(pk.cpu().numpy(), ref["pk"], ref["nmodes"])


def _assert_xi(got, want, nm):
    """xi to float32 round-off of the inverse FFT: within 1e-5 of the largest |xi_0| (the r ~ 0 variance)."""
    got, want = np.asarray(got, np.float64), np.asarray(want, np.float64)
    scale = np.nanmax(np.abs(want[:, 0]))
    both_nan = np.isnan(got) & np.isnan(want)
    assert np.array_equal(np.isnan(got), np.isnan(want))
    d = np.where(both_nan, 0.0, np.abs(got - want))
    assert np.all(d <= 1e-5 * scale), (d / scale).max()


def test_xi_vec_matches_reference(golden):
    from gbpowspec import xi_vec
    for i in range(int(golden["xi_ncases"][0])):
        d, box, se = golden[f"xi_{i}_delta"], float(golden[f"xi_{i}_box"][0]), golden[f"xi_{i}_sedges"]
        r, xi, nm = xi_vec(d, box, se)
        np.testing.assert_array_equal(r.cpu().numpy(), golden[f"xi_{i}_r"])
        np.testing.assert_array_equal(nm.cpu().numpy(), golden[f"xi_{i}_nmodes"])
        _assert_xi(xi.cpu().numpy(), golden[f"xi_{i}_xi"], golden[f"xi_{i}_nmodes"])


def test_compute_2pt_correlations_matches_reference(golden):
    from gbpowspec import compute_2pt_correlations
    for i in range(int(golden["xi_ncases"][0])):
        d, box, se = golden[f"xi_{i}_delta"], float(golden[f"xi_{i}_box"][0]), golden[f"xi_{i}_sedges"]
        k, pk, nmk, r, xi = compute_2pt_correlations(d, box, se, golden[f"tpc_{i}_kedges"])
        np.testing.assert_array_equal(k.cpu().numpy(), golden[f"tpc_{i}_k"])
        np.testing.assert_array_equal(nmk.cpu().numpy(), golden[f"tpc_{i}_nmodes"])
        _assert_pk(pk.cpu().numpy(), golden[f"tpc_{i}_pk"], golden[f"tpc_{i}_nmodes"])
        np.testing.assert_array_equal(r.cpu().numpy(), golden[f"tpc_{i}_r"])
        _assert_xi(xi.cpu().numpy(), golden[f"tpc_{i}_xi"], None)


def test_xi_of_a_large_mesh_against_fp64():
    """256^3 lognormal contrast: xi_0,2,4 from gbp_xi vs an FP64 numpy evaluation on the same mesh."""
    from gbpowspec import xi_vec
    from gbpowspec.synth import lognormal_density
    N, box = 128, 1000.0
    d = (lognormal_density(N, box, seed=4) - 1.0).astype(np.float32)
    se = np.arange(4.0, 200.0, 8.0).astype(np.float32)
    r, xi, nm = xi_vec(d, box, se)
    # FP64: same shells, same conventions
    dk = np.fft.rfftn(d.astype(np.float64))
    kk = np.fft.fftfreq(N, 1.0 / N)
    kz = np.arange(N // 2 + 1)
    w = lambda k: np.sinc(k / N) ** -4
    p = np.abs(dk) ** 2 * w(kk)[:, None, None] * w(kk)[None, :, None] * w(kz)[None, None, :]
    field = np.fft.irfftn(p, s=d.shape, axes=(0, 1, 2))
    ri = np.where(np.arange(N) > N // 2, np.arange(N) - N, np.arange(N))
    r2 = ri[:, None, None] ** 2 + ri[None, :, None] ** 2 + ri[None, None, :] ** 2
    rr = np.sqrt(r2.astype(np.float32))
    from gbpowspec.correlations import reference_sedges
    e = reference_sedges(se, box, N)
    idx = np.searchsorted(e, rr.ravel(), side="right")
    idx = np.where(rr.ravel() == e[-1], e.size - 1, idx)
    keep = (idx >= 1) & (idx <= e.size - 1)
    b = idx[keep] - 1
    with np.errstate(invalid="ignore", divide="ignore"):
        mu2 = np.where(r2 > 0, (ri[None, None, :] ** 2) / r2, np.nan).ravel()[keep]
    f = field.ravel()[keep]
    nb = e.size - 1
    cnt = np.bincount(b, minlength=nb).astype(np.float64)
    want = np.stack([np.bincount(b, weights=f, minlength=nb),
                     5 * np.bincount(b, weights=f * (1.5 * mu2 - 0.5), minlength=nb),
                     9 * np.bincount(b, weights=f * (35 * mu2 ** 2 - 30 * mu2 + 3) / 8, minlength=nb)], 1)
    want = want / cnt[:, None] / N ** 3
    np.testing.assert_array_equal(nm.cpu().numpy(), cnt.astype(np.float32))
    _assert_xi(xi.cpu().numpy(), want, None)


def test_xi_from_concurrent_threads_matches_serial():
    """Two host threads on their own streams share the cached inverse-transform plan: same bits as one at a time."""
    import threading
    from gbpowspec import xi_vec
    rng = np.random.default_rng(11)
    deltas = [torch.from_numpy(rng.standard_normal((64, 64, 64)).astype(np.float32)).cuda() for _ in range(2)]
    se = np.arange(2.0, 60.0, 4.0).astype(np.float32)
    want = [xi_vec(d, 500.0, se)[1].cpu() for d in deltas]
    got = [None, None]

    def work(i):
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            for _ in range(20):
                r = xi_vec(deltas[i], 500.0, se)[1]
            s.synchronize()
            got[i] = r.cpu()

    ts = [threading.Thread(target=work, args=(i,)) for i in range(2)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    for a, b in zip(got, want):
        assert np.array_equal(a.numpy(), b.numpy(), equal_nan=True)
