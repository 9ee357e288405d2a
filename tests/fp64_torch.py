"""TEST HELPER -- not product code.  The FP64 estimator of oracle/truth_f64.py
restated with torch float64 on the GPU, for meshes too large for the numpy
oracle (the 1024^3 precision study).  Same conventions, function by
function: float32 grid coordinates u = (x - origin) * inv_cell, B-spline
nodes and weights in float64, periodic index_add deposits, rfftn in
float64, window (sinc)^(-2p) per axis, interlacing phase, integer-k^2 shells
binned by jnp.histogram's rule on k = sqrtf(k^2) against float32 edges.
"""
from __future__ import annotations

import math

import numpy as np
import torch


def grid_coords(c: torch.Tensor, inv_cell) -> torch.Tensor:
    return (c.to(torch.float32) * torch.tensor(np.float32(inv_cell), device=c.device)).to(torch.float64)


def bspline(u: torch.Tensor, mas: int, half: bool):
    if half:
        u = u + 0.5
    i = torch.floor(u)
    d = u - i
    i = i.to(torch.int64)
    if mas == 1:
        return i + (d >= 0.5).to(torch.int64), [torch.ones_like(d)]
    if mas == 2:
        return i, [1.0 - d, d]
    if mas == 3:
        up = d >= 0.5
        s = torch.where(up, d - 1.0, d)
        return i + up.to(torch.int64) - 1, [0.5 * (0.5 - s) ** 2, 0.75 - s * s, 0.5 * (0.5 + s) ** 2]
    t, m = d, 1.0 - d
    return i - 1, [m ** 3 / 6, (4 - 6 * t * t + 3 * t ** 3) / 6, (4 - 6 * m * m + 3 * m ** 3) / 6, t ** 3 / 6]


def deposit(x, y, z, N: int, inv_cell, mas: int, half: bool) -> torch.Tensor:
    """float64 mesh [N^3] (flat) of one grid."""
    us = [grid_coords(c, inv_cell) for c in (x, y, z)]
    (fx, wx), (fy, wy), (fz, wz) = (bspline(u, mas, half) for u in us)
    mesh = torch.zeros(N ** 3, dtype=torch.float64, device=x.device)
    R = len(wx)
    for a in range(R):
        ix = torch.remainder(fx + a, N)
        for b in range(R):
            iy = torch.remainder(fy + b, N)
            base = (ix * N + iy) * N
            wab = wx[a] * wy[b]
            for c in range(R):
                mesh.index_add_(0, base + torch.remainder(fz + c, N), wab * wz[c])
    return mesh


def bin_index(k2: torch.Tensor, edges: torch.Tensor) -> torch.Tensor:
    k = torch.sqrt(k2.to(torch.float32))
    idx = torch.searchsorted(edges, k, right=True)
    idx = torch.where(k == edges[-1], torch.full_like(idx, edges.numel() - 1), idx)
    return torch.where((idx >= 1) & (idx <= edges.numel() - 1), idx - 1, torch.full_like(idx, -1))


def power_multipoles(x, y, z, *, box: float, N: int, mas: int, interlace: bool, kedges_grid, slab: int = 64):
    """P_0,2,4 (shot noise subtracted), mode counts; float64 throughout after the float32 coordinates."""
    dev = x.device
    inv = np.float32(N / box)
    fields, mass = [], None
    for half in ([False, True] if interlace else [False]):
        m = deposit(x, y, z, N, inv, mas, half)
        if mass is None:
            mass = float(m.sum())
        d = (m / m.mean() - 1.0).view(N, N, N)
        del m
        fields.append(torch.fft.rfftn(d))
        del d
    h = N // 2
    r = torch.arange(N, device=dev)
    ki = torch.where(r > h, r - N, r)
    kzv = ki[: h + 1].abs()
    edges = torch.tensor(np.asarray(kedges_grid, np.float32), device=dev)
    nb = edges.numel() - 1
    sums = torch.zeros((3, nb), dtype=torch.float64, device=dev)
    nmodes = torch.zeros(nb, dtype=torch.float64, device=dev)
    win = lambda k: torch.sinc(k.to(torch.float64) / N) ** (-2 * mas)
    for x0 in range(0, N, slab):
        kx = ki[x0:x0 + slab].view(-1, 1, 1)
        ky = ki.view(1, -1, 1)
        kz = kzv.view(1, 1, -1)
        if interlace:
            ph = torch.exp(1j * math.pi * (kx + ky + kz).to(torch.float64) / N)
            dk = 0.5 * (fields[0][x0:x0 + slab] + fields[1][x0:x0 + slab] * ph)
        else:
            dk = fields[0][x0:x0 + slab]
        p = dk.abs() ** 2 * win(kx) * win(ky) * win(kz)
        k2 = kx * kx + ky * ky + kz * kz
        k2 = k2.expand(p.shape)
        mu2 = torch.where(k2 > 0, (kz * kz).to(torch.float64) / k2.to(torch.float64), torch.zeros_like(p))
        if x0 == 0:
            p[0, 0, 0] = 0.0
        b = bin_index(k2, edges).reshape(-1)
        keep = b >= 0
        bb = b[keep]
        pf = p.reshape(-1)[keep]
        mf = mu2.reshape(-1)[keep]
        for l, lg in enumerate((torch.ones_like(mf), 1.5 * mf - 0.5, (35 * mf * mf - 30 * mf + 3) / 8)):
            sums[l] += torch.bincount(bb, weights=pf * lg, minlength=nb)
        nmodes += torch.bincount(bb, minlength=nb).to(torch.float64)
    norm = (box / N ** 2) ** 3
    pk = (sums / nmodes * torch.tensor([[1.0], [5.0], [9.0]], dtype=torch.float64, device=dev) * norm).T
    n = x.numel()
    shot = box ** 3 * n / mass ** 2
    pk[:, 0] -= shot
    return {"pk": pk.cpu().numpy(), "nmodes": nmodes.cpu().numpy().astype(np.int64), "shot": shot, "mass": mass}


def ngp_counts(x, y, z, N: int, box: float) -> torch.Tensor:
    """Particles per cell under the NGP rule (float32 coordinates, nearest node), int64 [N^3]."""
    inv = np.float32(N / box)
    (fx, _), (fy, _), (fz, _) = (bspline(grid_coords(c, inv), 1, False) for c in (x, y, z))
    idx = (torch.remainder(fx, N) * N + torch.remainder(fy, N)) * N + torch.remainder(fz, N)
    return torch.bincount(idx, minlength=N ** 3)


def power_multipoles_autograd(x, y, z, w, *, box: float, N: int, mas: int, interlace: bool, kedges_grid,
                              shot_noise: bool = True):
    """The production estimator in float64 with torch autograd end to end (positions and weights),
    the reference for the GPU gradients.  Grid coordinates u = x * N / L in float64 (the float32
    rounding of the kernels is below the gradient test's tolerance)."""
    dev = x.device
    inv = N / box
    wt = torch.ones_like(x, dtype=torch.float64) if w is None else w.to(torch.float64)
    grids = []
    for half in ([False, True] if interlace else [False]):
        st = [bspline(c.to(torch.float64) * inv, mas, half) for c in (x, y, z)]
        (fx, wx), (fy, wy), (fz, wz) = st
        R = len(wx)
        mesh = torch.zeros(N ** 3, dtype=torch.float64, device=dev)
        for a in range(R):
            ix = torch.remainder(fx + a, N)
            for b in range(R):
                iy = torch.remainder(fy + b, N)
                for c in range(R):
                    iz = torch.remainder(fz + c, N)
                    mesh = mesh.index_add(0, (ix * N + iy) * N + iz, wx[a] * wy[b] * wz[c] * wt)
        grids.append(mesh.view(N, N, N))
    M = grids[0].sum()
    F = [torch.fft.rfftn(m) for m in grids]
    h = N // 2
    r = torch.arange(N, device=dev)
    ki = torch.where(r > h, r - N, r)
    kx, ky, kz = ki.view(-1, 1, 1), ki.view(1, -1, 1), ki[: h + 1].abs().view(1, 1, -1)
    if interlace:
        ph = torch.exp(1j * math.pi * (kx + ky + kz).to(torch.float64) / N)
        D = 0.5 * (F[0] + F[1] * ph)
    else:
        D = F[0]
    win = lambda k: torch.sinc(k.to(torch.float64) / N) ** (-2 * mas)
    p = (D.real ** 2 + D.imag ** 2) * win(kx) * win(ky) * win(kz)
    k2 = (kx * kx + ky * ky + kz * kz).expand(p.shape)
    mu2 = torch.where(k2 > 0, (kz * kz).to(torch.float64) / k2.clamp(min=1).to(torch.float64), torch.zeros_like(p))
    p = torch.where(k2 == 0, torch.zeros_like(p), p)
    edges = torch.tensor(np.asarray(kedges_grid, np.float32), device=dev)
    b = bin_index(k2, edges).reshape(-1)
    keep = b >= 0
    bb = b[keep]
    nb = edges.numel() - 1
    pf = p.reshape(-1)[keep]
    mf = mu2.reshape(-1)[keep]
    sums = []
    for lg in (torch.ones_like(mf), 1.5 * mf - 0.5, (35 * mf * mf - 30 * mf + 3) / 8):
        sums.append(torch.zeros(nb, dtype=torch.float64, device=dev).scatter_add(0, bb, pf * lg))
    nmodes = torch.bincount(bb, minlength=nb).to(torch.float64)
    norm = box ** 3 / (M * M)
    pk = torch.stack([s / nmodes * f for s, f in zip(sums, (1.0, 5.0, 9.0))], dim=1) * norm
    if shot_noise:
        shot = box ** 3 * (wt * wt).sum() / (M * M)
        pk = torch.cat([pk[:, :1] - shot, pk[:, 1:]], dim=1)
    return pk
