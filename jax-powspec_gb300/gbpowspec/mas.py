"""Mass assignment: drop-ins for jax-powspec's src/mas.py, plus mesh_deposit.

``cic_mas_vec`` and ``cic_mas`` keep the reference's signatures and results,
reference bugs included (see the C ABI notes in include/gbpowspec.h):

* the corner (ix, iyp, izp) is weighted mdx*mdy*ddz (src/mas.py:149, :76),
  so a particle deposits 1 + mdx*ddz*(1 - 2*ddy) instead of 1;
* cic_mas_vec with wrap=False zeroes the +1 index but keeps its fraction
  (src/mas.py:125-126), which wraps that weight onto cell 0;
* indices are truncated toward zero (src/mas.py:107), negative indices wrap
  once and indices >= n are dropped (jax scatter rules).

The deposit runs on the GPU (libgbpowspec.so); inputs may be torch tensors or
numpy arrays and the result is a torch CUDA tensor.  The mesh values are
accumulated in exact fixed point, so they do not depend on particle order.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib, _native

__all__ = ["cic_mas_vec", "cic_mas", "mesh_deposit", "reference_inv_cell"]


def _f32_scalar(v) -> np.float32:
    if isinstance(v, torch.Tensor):
        v = v.detach().reshape(()).cpu().item()
    return np.float32(np.asarray(v, dtype=np.float32).reshape(()))


def reference_inv_cell(box_size, n_bins) -> np.float32:
    """1 / (box_size / n_bins) in float32, as src/mas.py:100-101 computes it."""
    bin_size = _f32_scalar(box_size) / np.float32(n_bins)
    return np.float32(np.float32(1.0) / bin_size)


def _compat_deposit(compat, delta, x, y, z, w, xmin, ymin, zmin, box_size, n_bins, wrap):
    d = _native.as_cuda_f32(delta, name="delta")
    if d.ndim != 3 or not (d.shape[0] == d.shape[1] == d.shape[2]):
        raise ValueError(f"delta must be a cubic 3-D mesh, got shape {tuple(d.shape)}")
    N = int(d.shape[0])
    if int(n_bins) != N:
        raise ValueError(f"n_bins ({n_bins}) must equal the mesh side ({N})")
    dev = d.device
    xs = _native.as_cuda_f32(x, dev).reshape(-1)
    ys = _native.as_cuda_f32(y, dev).reshape(-1)
    zs = _native.as_cuda_f32(z, dev).reshape(-1)
    if not (xs.numel() == ys.numel() == zs.numel()):
        raise ValueError("x, y and z must have the same length")
    ws = None if w is None else _native.as_cuda_f32(w, dev).reshape(-1)
    if ws is not None and ws.numel() != xs.numel():
        raise ValueError("w must have one weight per particle")
    origin = (_f32_scalar(xmin), _f32_scalar(ymin), _f32_scalar(zmin))
    mesh, _ = _native.deposit(xs, ys, zs, ws, n_mesh=N, inv_cell=reference_inv_cell(box_size, n_bins),
                              origin=origin, mas=_lib.MAS["cic"], interlace=False, compat=compat,
                              wrap=bool(wrap), mesh_in=d.reshape(1, N, N, N))
    return mesh.reshape(N, N, N)


def cic_mas_vec(delta, x, y, z, w, n_part, xmin, ymin, zmin, box_size, n_bins, wrap):
    """Drop-in for src/mas.py:88-153 (``cic_mas_vec``).

    Returns ``delta + CIC(x, y, z, w)`` as a new float32 CUDA tensor; `delta`
    is not modified.  `n_part` is unused, as in the reference.
    """
    del n_part
    return _compat_deposit(_lib.COMPAT_VEC, delta, x, y, z, w, xmin, ymin, zmin, box_size, n_bins, wrap)


def cic_mas(delta, x, y, z, w, n_part, xmin, ymin, zmin, box_size, n_bins, wrap):
    """Drop-in for src/mas.py:5-87 (``cic_mas``, the sequential scan variant).

    Same result as the reference's per-particle loop: with wrap=False the
    +1 neighbour beyond the last cell gets zero weight (src/mas.py:30-38),
    and with wrap=True an index >= n has n subtracted once (src/mas.py:20-28).
    """
    del n_part
    return _compat_deposit(_lib.COMPAT_SCAN, delta, x, y, z, w, xmin, ymin, zmin, box_size, n_bins, wrap)


def mesh_deposit(x, y, z, w=None, *, box_size: float, n_mesh: int, mas: str = "cic", interlace: bool = False,
                 origin=(0.0, 0.0, 0.0), device=None):
    """Periodic B-spline deposit (NGP/CIC/TSC/PCS), optionally interlaced.

    Nodes sit at ``origin + i * box_size / n_mesh`` (the reference's
    convention); the interlaced second grid deposits every particle shifted by
    +half a cell on all axes.  Returns ``(mesh, stats)``: mesh is float32
    [G, n, n, n] (G = 2 when interlaced) and stats a device
    ``gbp_deposit_stats`` (read it with ``gbpowspec.read_stats``).
    """
    mas_id = _lib.MAS[mas.lower()]
    xs = _native.as_cuda_f32(x, device).reshape(-1)
    dev = xs.device
    ys = _native.as_cuda_f32(y, dev).reshape(-1)
    zs = _native.as_cuda_f32(z, dev).reshape(-1)
    ws = None if w is None else _native.as_cuda_f32(w, dev).reshape(-1)
    inv_cell = np.float32(float(n_mesh) / float(box_size))
    return _native.deposit(xs, ys, zs, ws, n_mesh=int(n_mesh), inv_cell=inv_cell,
                           origin=tuple(np.float32(o) for o in origin), mas=mas_id, interlace=interlace,
                           compat=_lib.COMPAT_NONE, wrap=True)
