"""TEST ORACLE -- not product code.  Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg may import this module.

FP64 "truth" estimator of the same P_l(k) that the GPU pipeline computes:
  deposit (NGP/CIC/TSC/PCS B-splines, nodes at origin + i*H, optional
  half-cell-shifted second grid) -> delta = rho/mean - 1 -> rfftn ->
  window deconvolution and interlacing -> |delta|^2 L_l(mu) -> k shells.

Everything after the float32 grid coordinate u = (x - origin) * inv_cell is
double precision (the kernel computes u the same way, so both sides see the
same particle positions).  Bin membership applies jnp.histogram's rule to
k = sqrtf(k^2) against float32 edges -- computed here directly with
searchsorted, independently of the integer thresholds the GPU uses.

The reference's own estimator (src/correlations.py:7-56) is the special case
mas_order=2, one grid, delta given.
"""
from __future__ import annotations

import numpy as np

F32 = np.float32


def grid_coords(c, origin, inv_cell) -> np.ndarray:
    """u = (c - origin) * inv_cell in float32 (as the deposit kernel), returned as float64."""
    return ((np.asarray(c, F32) - F32(origin)) * F32(inv_cell)).astype(np.float64)


def bspline(u: np.ndarray, mas: int, half: bool):
    """First node index and the weights of the order-`mas` B-spline at u (float64)."""
    if half:
        u = u + 0.5
    i = np.floor(u)
    d = u - i
    i = i.astype(np.int64)
    if mas == 1:
        up = (d >= 0.5).astype(np.int64)
        return i + up, [np.ones_like(d)]
    if mas == 2:
        return i, [1.0 - d, d]
    if mas == 3:
        up = (d >= 0.5)
        s = np.where(up, d - 1.0, d)
        return i + up.astype(np.int64) - 1, [0.5 * (0.5 - s) ** 2, 0.75 - s * s, 0.5 * (0.5 + s) ** 2]
    if mas == 4:
        t, m = d, 1.0 - d
        return i - 1, [m ** 3 / 6, (4 - 6 * t * t + 3 * t ** 3) / 6, (4 - 6 * m * m + 3 * m ** 3) / 6, t ** 3 / 6]
    raise ValueError(mas)


def deposit(x, y, z, w, n_mesh: int, inv_cell, origin=(0.0, 0.0, 0.0), mas: int = 2, interlace: bool = False):
    """float64 meshes [G, N, N, N] of a periodic B-spline deposit."""
    N = int(n_mesh)
    us = [grid_coords(c, o, inv_cell) for c, o in zip((x, y, z), origin)]
    wt = np.ones(us[0].shape) if w is None else np.asarray(w, F32).astype(np.float64)
    out = []
    for half in ([False, True] if interlace else [False]):
        st = [bspline(u, mas, half) for u in us]
        mesh = np.zeros(N ** 3)
        (fx, wx), (fy, wy), (fz, wz) = st
        R = len(wx)
        for a in range(R):
            ix = np.mod(fx + a, N)
            for b in range(R):
                iy = np.mod(fy + b, N)
                wab = wx[a] * wy[b] * wt
                for c in range(R):
                    iz = np.mod(fz + c, N)
                    mesh += np.bincount((ix * N + iy) * N + iz, weights=wab * wz[c], minlength=N ** 3)
        out.append(mesh.reshape(N, N, N))
    return np.stack(out)


def kgrid(N: int):
    h = N // 2
    r = np.arange(N)
    ki = np.where(r > h, r - N, r)
    kx = ki[:, None, None]
    ky = ki[None, :, None]
    kz = ki[None, None, : h + 1]
    return kx, ky, kz


def bin_index(k2: np.ndarray, kedges_grid: np.ndarray) -> np.ndarray:
    """jnp.histogram bin of k = sqrtf(k2) for float32 edges; -1 when dropped."""
    e = np.asarray(kedges_grid, F32)
    k = np.sqrt(np.asarray(k2).astype(F32))
    idx = np.searchsorted(e, k, side="right")
    idx = np.where(k == e[-1], e.size - 1, idx)
    b = idx - 1
    return np.where((idx >= 1) & (idx <= e.size - 1), b, -1)


def power(meshes: np.ndarray, box_size: float, kedges_grid, mas_order: int = 2, normalize: str = "mean",
          sum_w2: float | None = None):
    """P_0,2,4 of one mesh or an interlaced pair, in float64.

    normalize="mean": meshes are densities; delta = rho/mean - 1 per grid.
    normalize="none": meshes[0] already is delta (the reference's input).
    sum_w2: when given, subtract the shot noise L^3 sum_w2 / (sum rho)^2 from P_0.
    Returns dict(sums[nb,3], nmodes[nb], ksum[nb], pk[nb,3], kmean[nb]).
    """
    meshes = np.asarray(meshes, dtype=np.float64)
    if meshes.ndim == 3:
        meshes = meshes[None]
    G, N = meshes.shape[0], meshes.shape[1]
    L = float(box_size)
    mass = meshes[0].sum()
    fields = []
    for g in range(G):
        d = meshes[g]
        if normalize == "mean":
            d = d / d.mean() - 1.0
        fields.append(np.fft.rfftn(d))
    kx, ky, kz = kgrid(N)
    if G == 2:
        ph = np.exp(1j * np.pi * (kx + ky + kz) / N)
        dk = 0.5 * (fields[0] + fields[1] * ph)
    else:
        dk = fields[0]
    def win(k):
        return np.sinc(k / N) ** (-2 * mas_order)
    p = np.abs(dk) ** 2 * win(kx) * win(ky) * win(kz)
    k2 = (kx ** 2 + ky ** 2 + kz ** 2) + np.zeros_like(p, dtype=np.int64)
    with np.errstate(invalid="ignore", divide="ignore"):
        mu2 = np.where(k2 > 0, kz.astype(np.float64) ** 2 / k2, 0.0)
    legs = [np.ones_like(mu2), 1.5 * mu2 - 0.5, (35 * mu2 ** 2 - 30 * mu2 + 3) / 8]
    b = bin_index(k2, kedges_grid).ravel()
    nb = np.asarray(kedges_grid).size - 1
    keep = b >= 0
    bb = b[keep]
    sums = np.stack([np.bincount(bb, weights=(p * lg).ravel()[keep], minlength=nb) for lg in legs], axis=1)
    nmodes = np.bincount(bb, minlength=nb).astype(np.int64)
    ksum = np.bincount(bb, weights=np.sqrt(k2.astype(np.float64)).ravel()[keep], minlength=nb)
    norm = (L / N ** 2) ** 3
    with np.errstate(invalid="ignore", divide="ignore"):
        pk = sums / nmodes[:, None] * np.array([1.0, 5.0, 9.0]) * norm
        kmean = ksum / nmodes * (2 * np.pi / L)
    shot = 0.0
    if sum_w2 is not None:
        shot = L ** 3 * float(sum_w2) / mass ** 2
        pk[:, 0] -= shot
    return {"sums": sums, "nmodes": nmodes, "ksum": ksum, "pk": pk, "kmean": kmean, "mass": mass, "shot": shot}


def power_multipoles(x, y, z, w, *, box_size: float, n_mesh: int, mas: int, interlace: bool,
                     kedges_grid, shot_noise: bool = True, origin=(0.0, 0.0, 0.0)):
    """End-to-end FP64 estimate with the same conventions as gbpowspec.PowerSpectrum."""
    inv_cell = F32(float(n_mesh) / float(box_size))
    meshes = deposit(x, y, z, w, n_mesh, inv_cell, origin, mas, interlace)
    wt = np.ones(np.asarray(x).size) if w is None else np.asarray(w, F32).astype(np.float64)
    return power(meshes, box_size, kedges_grid, mas_order=mas, normalize="mean",
                 sum_w2=float((wt * wt).sum()) if shot_noise else None)


def bispec(delta, box_size, k1, k2, theta, mas_order: int = 2):
    """The FFT bispectrum estimator of src/correlations.py:334-462 in float64: per shell the
    inverse transforms of the masked, window-corrected spectrum and of the mask itself, real-space
    sums of squares and of triple products.  Shell membership is the reference's float32 rule
    (k = sqrtf(k^2) against float32 limits (k_i -+ kF) / kF), so only the arithmetic differs.
    The window is sinc^(-p) per axis on the amplitude, p = mas_order (the reference: p = 2).
    Returns (k_all, P [S], B [S-2], Q [S-2], nmodes [S]) with nmodes counted on the full grid."""
    F32 = np.float32
    delta = np.asarray(delta, np.float64)
    N = delta.shape[0]
    box = F32(box_size)
    kF = F32(F32(2.0 * np.pi) / box)
    theta = np.asarray(theta, F32)
    k1f, k2f = F32(k1), F32(k2)
    k3 = np.sqrt((k2f * np.sin(theta)) ** 2 + (k2f * np.cos(theta) + k1f) ** 2).astype(F32)
    k_all = np.concatenate([[k1f, k2f], k3]).astype(F32)
    k_min = ((k_all - kF) / kF).astype(F32)
    k_max = ((k_all + kF) / kF).astype(F32)
    dk = np.fft.rfftn(delta)
    r = np.arange(N)
    ki = np.where(r > N // 2, r - N, r)
    kx, ky, kz = ki[:, None, None], ki[None, :, None], np.arange(N // 2 + 1)[None, None, :]
    w = lambda q: np.sinc(q / N) ** (-float(mas_order))
    dk = dk * w(kx) * w(ky) * w(kz)
    k = np.sqrt((kx * kx + ky * ky + kz * kz).astype(F32))
    S = k_all.size
    d, one, nm = [], [], np.zeros(S, np.int64)
    for i in range(S):
        m = (k >= k_min[i]) & (k < k_max[i])
        d.append(np.fft.irfftn(m * dk, s=delta.shape, axes=(0, 1, 2)))
        one.append(np.fft.irfftn(m.astype(np.float64), s=delta.shape, axes=(0, 1, 2)))
        wz = np.where((kz == 0) | ((N % 2 == 0) & (kz == N // 2)), 1, 2)
        nm[i] = int((np.broadcast_to(m, dk.shape) * wz).sum())
    L = float(box)
    pk = np.array([(d[i] ** 2).sum() / (one[i] ** 2).sum() for i in range(S)]) * (L / N ** 2) ** 3
    with np.errstate(invalid="ignore", divide="ignore"):
        bk = np.array([(d[0] * d[1] * d[j]).sum() / (one[0] * one[1] * one[j]).sum() for j in range(2, S)])
        bk = bk * (L * L / N ** 3) ** 3
        qk = bk / (pk[0] * pk[1] + pk[0] * pk[2:] + pk[1] * pk[2:])
    return k_all, pk, bk, qk, nm
