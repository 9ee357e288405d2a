"""TEST ORACLE -- not product code.  Only bench.py's CPU-baseline and
reference legs import this module: it is the timed CPU stand-in for the
reference's path when the reference's own JAX code cannot run.

The same computation as reference_f32.cic_mas_vec -> delta/mean - 1 ->
reference_f32.powspec_vec (src/mas.py:88-153, tests/correlations.py:49-50,
src/correlations.py:7-56), written for speed rather than bit-exactness:
scatter-adds and histograms accumulate with np.bincount (float64) instead of
sequential float32 ``np.add.at``, the corner-weight bug of src/mas.py:149 is
kept, and the FFT runs on all host threads (scipy.fft workers).  Agreement
with reference_f32 is to float32 round-off (checked in the tests).
"""
from __future__ import annotations

import os

import numpy as np
import scipy.fft

F32 = np.float32


def threads() -> int:
    return os.cpu_count() or 1


def cic_mas_vec_wrap(x, y, z, box_size: float, N: int) -> np.ndarray:
    """src/mas.py:88-153 with wrap=True, w = 1, xmin = 0 (the reference path's CIC with its corner bug)."""
    bin_size = F32(box_size) / F32(N)
    inv = F32(F32(1.0) / bin_size)
    pos = [np.asarray(c, F32) * inv for c in (x, y, z)]
    i0 = [p.astype(np.int32) for p in pos]
    dd = [p - i.astype(F32) for p, i in zip(pos, i0)]
    md = [F32(1.0) - d for d in dd]
    ip = [np.mod(i + 1 + N, N) for i in i0]
    i0 = [np.where(i < 0, i + N, i) for i in i0]
    (ix, iy, iz), (ixp, iyp, izp) = i0, ip
    (dx, dy, dz), (mx, my, mz) = dd, md
    corners = [
        (ix, iy, iz, mx * my * mz), (ix, iy, izp, mx * my * dz), (ix, iyp, iz, mx * dy * mz),
        (ix, iyp, izp, mx * my * dz),                                # the reference's weight (src/mas.py:149)
        (ixp, iy, iz, dx * my * mz), (ixp, iy, izp, dx * my * dz), (ixp, iyp, iz, dx * dy * mz),
        (ixp, iyp, izp, dx * dy * dz),
    ]
    idx = np.concatenate([((a.astype(np.int64) * N + b) * N + c) for a, b, c, _ in corners])
    wts = np.concatenate([w for *_, w in corners]).astype(np.float64)
    ok = np.concatenate([(a >= 0) & (a < N) & (b >= 0) & (b < N) & (c >= 0) & (c < N)
                         for a, b, c, _ in corners])          # out-of-range updates are dropped
    mesh = np.bincount(idx[ok], weights=wts[ok], minlength=N ** 3)
    return mesh.astype(F32).reshape(N, N, N)


def powspec_vec(delta: np.ndarray, box_size: float, k_edges: np.ndarray):
    """src/correlations.py:7-56 with bincount histograms and a threaded FFT."""
    dims = delta.shape[0]
    dk = scipy.fft.rfftn(np.asarray(delta, F32), workers=threads())
    middle = dims // 2
    r = np.arange(dims, dtype=np.int32)
    ki = np.where(r > middle, r - dims, r).astype(np.int32)
    kx = ki[:, None, None]
    ky = ki[None, :, None]
    kz = ki[None, None, : middle + 1]

    def corr(k):
        x = (F32(np.pi / dims) * k.astype(F32)) / F32(np.pi)
        return (F32(1.0) / np.sinc(x).astype(F32)) ** 2

    c = corr(kx) * corr(ky) * corr(kz)
    k2 = (kx * kx + ky * ky + kz * kz)
    k = np.sqrt(k2.astype(F32))
    with np.errstate(invalid="ignore", divide="ignore"):
        mu2 = np.where(k == 0, F32(0), (kz.astype(F32) / k) ** 2).astype(F32)
    p = (np.abs(dk) ** 2).astype(F32) * c * c
    kF = F32(F32(2.0 * np.pi) / F32(box_size))
    edges = (np.asarray(k_edges, F32) / kF).astype(F32)
    kk = np.broadcast_to(k, p.shape).ravel()
    idx = np.searchsorted(edges, kk, side="right")
    idx = np.where(kk == edges[-1], edges.size - 1, idx)
    keep = (idx >= 1) & (idx < edges.size)
    b = idx[keep] - 1
    pf = p.ravel()[keep].astype(np.float64)
    m2 = np.broadcast_to(mu2, p.shape).ravel()[keep].astype(np.float64)
    nb = edges.size - 1
    mono = np.bincount(b, weights=pf, minlength=nb)
    quad = np.bincount(b, weights=pf * (1.5 * m2 - 0.5), minlength=nb)
    hexa = np.bincount(b, weights=pf * (35 * m2 * m2 - 30 * m2 + 3) / 8, minlength=nb)
    nmodes = np.bincount(b, minlength=nb).astype(np.float64)
    norm = (float(box_size) / dims ** 2) ** 3
    with np.errstate(invalid="ignore", divide="ignore"):
        pk = np.stack([mono / nmodes, 5 * quad / nmodes, 9 * hexa / nmodes], axis=1) * norm
    k3d = 0.5 * (edges[1:] + edges[:-1]) * kF
    return k3d.astype(F32), pk.astype(F32), nmodes.astype(F32)


def reference_mock(x, y, z, box_size: float, N: int, k_edges: np.ndarray):
    """The reference path for one mock: deposit, delta = rho/mean - 1, P_l(k)."""
    d = cic_mas_vec_wrap(x, y, z, box_size, N)
    d = d / d.mean() - F32(1.0)
    return powspec_vec(d, box_size, k_edges)
