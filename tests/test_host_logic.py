"""Host-side logic that runs without a GPU: exact bin thresholds, argument
checks, the fundamental-shell geometry helper and the synthetic catalogues."""
import numpy as np
import pytest

from oracle import reference_f32 as R
from oracle import truth_f64 as T


def _all_k2(N):
    h = N // 2
    return np.arange(3 * h * h + 1)


EDGE_SETS = {
    "integers": lambda N: np.arange(1, max(N // 2, 3), dtype=np.float32),
    "fine": lambda N: np.linspace(0.3, N, 211).astype(np.float32),
    "from_zero": lambda N: np.linspace(0.0, 0.9 * N, 17).astype(np.float32),
    "negative_start": lambda N: np.array([-3.0, 0.0, 0.5, 1.0, 2.5, 4.0], np.float32),
    "duplicates": lambda N: np.array([1, 1, 2, 2, 2, 3.5, 7, 7], np.float32),
    "sqrt_ties": lambda N: np.sqrt(np.array([1, 2, 3, 5, 8, 13, 21, 34], np.float32)).astype(np.float32),
    "f32_rounded": lambda N: (np.float32(2 * np.pi / 1000) * np.arange(1, max(N // 2, 3), dtype=np.float32))
    / np.float32(np.float32(2 * np.pi) / np.float32(1000)),
    "beyond_kmax": lambda N: np.array([N * 0.5, N * 0.8, N * 2.0, N * 3.0], np.float32),
}


@pytest.mark.parametrize("N", [4, 9, 16, 33, 64, 128])
@pytest.mark.parametrize("edges", sorted(EDGE_SETS))
def test_thresholds_reproduce_histogram_rule(N, edges):
    """For every integer k^2 on the grid, the integer thresholds put it in the
    same bin as jnp.histogram's rule on sqrtf(k^2) does."""
    from gbpowspec import _native
    e = EDGE_SETS[edges](N).astype(np.float32)
    thr, last, reach = _native.bin_thresholds(e, N)
    k2 = _all_k2(N)
    want = T.bin_index(k2, e)
    r = np.searchsorted(thr, k2, side="right")           # number of thresholds <= k2
    got = np.where((k2 <= last) & (r >= 1), np.minimum(r, e.size - 1) - 1, -1)
    np.testing.assert_array_equal(got, want)
    assert reach == (want.max() + 1 if (want >= 0).any() else reach)


def test_thresholds_reject_bad_edges():
    from gbpowspec import _native, GbpError
    with pytest.raises(GbpError):
        _native.bin_thresholds(np.array([1.0, 0.5, 2.0], np.float32), 16)
    with pytest.raises(GbpError):
        _native.bin_thresholds(np.array([1.0, np.nan], np.float32), 16)
    with pytest.raises(GbpError):
        _native.bin_thresholds(np.array([1.0], np.float32), 16)


@pytest.mark.parametrize("N", [8, 9, 12, 16])
def test_fundamental_last_writer_geometry(N):
    """k of the last mode per int32(|k|) slot == numpy's last-duplicate assignment."""
    from gbpowspec.correlations import _fundamental_last_k
    kx, ky, kz = R._kgrid(N)
    k = np.sqrt((kx * kx + ky * ky + kz * kz).astype(np.float32)).ravel()
    slot = k.astype(np.int32)
    want = np.zeros(slot.max() + 1, np.float32)
    want[slot] = k
    np.testing.assert_array_equal(_fundamental_last_k(N), want)


def test_deposit_workspace_rejects_bad_args():
    from gbpowspec import _native, GbpError
    with pytest.raises(GbpError):
        _native.deposit_workspace_size(10, 16, 5, False, 0)          # no such MAS
    with pytest.raises(GbpError):
        _native.deposit_workspace_size(10, 16, 3, False, 1)          # compat needs CIC
    with pytest.raises(GbpError):
        _native.deposit_workspace_size(10, 16, 2, True, 1)           # compat has no interlacing


def test_lognormal_catalogue_shape_and_determinism():
    from gbpowspec.synth import lognormal_catalogue
    a = lognormal_catalogue(50_000, 500.0, grid=32, seed=3)
    b = lognormal_catalogue(50_000, 500.0, grid=32, seed=3)
    for u, v in zip(a, b):
        assert u.dtype == np.float32 and u.size == 50_000
        np.testing.assert_array_equal(u, v)
        assert u.min() >= 0 and u.max() < 500.0


def test_lognormal_field_unit_variance():
    from gbpowspec.synth import lognormal_density
    rho = lognormal_density(64, 1000.0, seed=1)
    g = np.log(rho) + 0.5
    assert abs(g.var() - 1.0) < 0.05
    assert abs(rho.mean() - 1.0) < 0.05


def test_algorithmic_bytes_formula():
    from gbpowspec import algorithmic_bytes
    b = algorithmic_bytes(4_194_304, 512, 2)
    assert abs(b / 1e6 - 4353.7) < 0.1
