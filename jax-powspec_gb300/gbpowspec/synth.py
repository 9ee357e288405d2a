"""Seeded synthetic catalogues with the shapes of the benchmark configurations.

No survey data is used: the lognormal recipe follows the reference's mock
pipeline (tests/create_lognormal.py:42-55 with src/gauss_field.py:5-80 and
src/populate_field.py:4-29) with these documented choices:

* Gaussian field on a ``grid^3`` lattice with P_G(k) = A k exp(-(k/0.3)^2),
  A fixed so that the lattice variance sigma_G^2 = sum_k P_G(k)/V equals 1;
* delta_LN = exp(g - sigma_G^2/2) - 1;
* exactly ``n`` particles drawn multinomially with probabilities proportional
  to 1 + delta_LN (the reference draws Poisson counts; an exact n keeps the
  benchmark shape fixed), placed uniformly inside their cell;
* optional redshift-space shift along z by N(0, sigma_v) with periodic wrap;
* float32 positions clamped below the box size, in random order.
"""
from __future__ import annotations

import numpy as np

__all__ = ["uniform_catalogue", "lognormal_catalogue", "lognormal_density", "lognormal_catalogue_gpu",
           "lognormal_field_gpu", "gaussian_power"]


def _clamp_box(a: np.ndarray, box: float) -> np.ndarray:
    a = np.mod(a, box).astype(np.float32)
    top = np.nextafter(np.float32(box), np.float32(0))
    return np.minimum(a, top)


def uniform_catalogue(n: int, box: float, seed: int = 0):
    rng = np.random.default_rng(seed)
    p = (rng.random((3, n), dtype=np.float64) * box).astype(np.float32)
    return tuple(_clamp_box(c, box) for c in p)


def lognormal_density(grid: int, box: float, seed: int, k_cut: float = 0.3) -> np.ndarray:
    """1 + delta_LN on a grid^3 lattice (float64), mean ~1."""
    rng = np.random.default_rng(seed)
    eps = rng.standard_normal((grid, grid, grid))
    ek = np.fft.rfftn(eps)
    kf = 2 * np.pi / box
    ki = np.fft.fftfreq(grid, d=1.0 / grid) * kf
    kz = np.fft.rfftfreq(grid, d=1.0 / grid) * kf
    k = np.sqrt(ki[:, None, None] ** 2 + ki[None, :, None] ** 2 + kz[None, None, :] ** 2)
    shape = k * np.exp(-((k / k_cut) ** 2))
    V = box ** 3
    # lattice variance of the field: sum over the full (Hermitian) grid of P/V
    weight = np.full(k.shape, 2.0)
    weight[..., 0] = 1.0
    if grid % 2 == 0:
        weight[..., -1] = 1.0
    A = 1.0 / ((weight * shape).sum() / V)
    pk = A * shape
    gk = ek * np.sqrt(grid ** 3 * pk / V)
    gk[0, 0, 0] = 0.0
    g = np.fft.irfftn(gk, s=(grid, grid, grid), axes=(0, 1, 2))
    sigma2 = 1.0
    return np.exp(g - sigma2 / 2.0)


def lognormal_catalogue(n: int, box: float, grid: int = 256, seed: int = 0, rsd_sigma: float = 3.0):
    """(x, y, z) float32 arrays of exactly n particles from a lognormal field."""
    rho = lognormal_density(grid, box, seed)
    rng = np.random.default_rng(seed + 7919)
    p = rho.ravel() / rho.sum()
    counts = rng.multinomial(n, p)
    cells = np.repeat(np.arange(grid ** 3, dtype=np.int64), counts)
    H = box / grid
    ix, rem = np.divmod(cells, grid * grid)
    iy, iz = np.divmod(rem, grid)
    off = rng.random((3, n))
    x = (ix + off[0]) * H
    y = (iy + off[1]) * H
    z = (iz + off[2]) * H
    if rsd_sigma:
        z = z + rng.normal(0.0, rsd_sigma, size=n)
    perm = rng.permutation(n)
    return _clamp_box(x[perm], box), _clamp_box(y[perm], box), _clamp_box(z[perm], box)


def lognormal_catalogue_gpu(n: int, box: float, grid: int = 256, seed: int = 0, rsd_sigma: float = 3.0,
                            k_cut: float = 0.3, device=None, out=None):
    """The same recipe generated on the device (gbp_lognormal): (x, y, z) float32 CUDA tensors.

    The random numbers differ from the host generator's (counter-based
    Philox4x32-10 instead of numpy's), so catalogues agree in distribution,
    not value by value.  `out` = (x, y, z) tensors of >= n elements to reuse.
    """
    import ctypes as C

    import torch

    from . import _lib, _native
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    lib = _lib.load()
    need = C.c_size_t(0)
    _lib.check(lib.gbp_lognormal_workspace_size(int(grid), C.byref(need)), "gbp_lognormal_workspace_size")
    ws = _native.workspace(need.value, dev)
    if out is None:
        out = tuple(torch.empty(int(n), dtype=torch.float32, device=dev) for _ in range(3))
    x, y, z = out
    _lib.check(lib.gbp_lognormal(int(grid), float(box), float(k_cut), float(rsd_sigma), int(n),
                                 int(seed) & 0xFFFFFFFFFFFFFFFF, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                                 C.c_void_p(z.data_ptr()), C.c_void_p(ws.data_ptr()), ws.numel(),
                                 _native._stream_of(dev)), "gbp_lognormal")
    return x[:n], y[:n], z[:n]


def gaussian_power(k, box: float, grid: int, k_cut: float = 0.3) -> np.ndarray:
    """P_G(k) = A k exp(-(k/k_cut)^2) of the generators, A set so that the lattice variance
    sum_k P_G(k) / V over the grid^3 lattice is 1 (h^-3 Mpc^3; k in h/Mpc)."""
    kf = 2 * np.pi / box
    ki = np.fft.fftfreq(grid, d=1.0 / grid) * kf
    kz = np.fft.rfftfreq(grid, d=1.0 / grid) * kf
    kk = np.sqrt(ki[:, None, None] ** 2 + ki[None, :, None] ** 2 + kz[None, None, :] ** 2)
    shape = kk * np.exp(-((kk / k_cut) ** 2))
    weight = np.full(kk.shape, 2.0)
    weight[..., 0] = 1.0
    if grid % 2 == 0:
        weight[..., -1] = 1.0
    A = box ** 3 / (weight * shape).sum()
    k = np.asarray(k, dtype=np.float64)
    return A * k * np.exp(-((k / k_cut) ** 2))


def lognormal_field_gpu(grid: int, box: float, seed: int = 0, k_cut: float = 0.3, device=None):
    """(g, rho): the device generator's Gaussian field and rho = exp(g - 1/2) = 1 + delta_LN on the
    grid^3 lattice (float32 CUDA tensors [grid, grid, grid]), the field lognormal_catalogue_gpu samples
    its particles from for the same (grid, box, seed, k_cut)."""
    import ctypes as C

    import torch

    from . import _lib, _native
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    lib = _lib.load()
    need = C.c_size_t(0)
    _lib.check(lib.gbp_lognormal_workspace_size(int(grid), C.byref(need)), "gbp_lognormal_workspace_size")
    ws = _native.workspace(need.value, dev)
    g = torch.empty((grid, grid, grid), dtype=torch.float32, device=dev)
    rho = torch.empty_like(g)
    _lib.check(lib.gbp_lognormal_field(int(grid), float(box), float(k_cut), int(seed) & 0xFFFFFFFFFFFFFFFF,
                                       C.c_void_p(g.data_ptr()), C.c_void_p(rho.data_ptr()),
                                       C.c_void_p(ws.data_ptr()), ws.numel(), _native._stream_of(dev)),
               "gbp_lognormal_field")
    return g, rho
