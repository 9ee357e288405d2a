"""P(k) multipoles: drop-ins for jax-powspec's src/correlations.py P(k) path.

``powspec_vec(delta, box_size, k_edges)`` and
``powspec_vec_fundamental(delta, box_size)`` keep the reference's signatures
and return tuples ``(k3D, Pk3D, Nmodes3D)`` as float32 CUDA tensors:

* the mesh is FFT'd (R2C) by the library's own transform for power-of-two
  sides 64..1024 and by cuFFT otherwise, then one fused kernel applies the CIC
  window correction (1/sinc)^2 per axis (src/correlations.py:20-21,32,39),
  squares, weights by L_0, L_2, L_4 of mu = kz/k (:36-38,45-47) and bins;
* binning reproduces jnp.histogram on k = sqrtf(kx^2+ky^2+kz^2) against the
  float32 edges k_edges / kF (:34,42), so mode counts are bit-identical;
* P_l = (2l+1) sum / N_modes * (L/N^2)^3 (:49-52), NaN in empty bins;
* k3D are the arithmetic bin centres (:54).

Per-bin sums are accumulated in FP32 inside a warp and in float-float /
FP64 beyond, so they are more accurate than the reference's float32
scatter-add; P agrees with it to float32 rounding.
"""
from __future__ import annotations

import functools

import numpy as np
import torch

from . import _lib, _native

__all__ = ["powspec_vec", "powspec_vec_fundamental", "xi_vec", "compute_2pt_correlations", "bispec", "bispectrum",
           "compute_all_correlations", "bispec_shells", "reference_kedges", "reference_sedges", "default_kedges"]

_F32 = np.float32


def _box_f32(box_size) -> np.float32:
    if isinstance(box_size, torch.Tensor):
        box_size = box_size.detach().reshape(()).cpu().item()
    return _F32(np.asarray(box_size, dtype=np.float32).reshape(()))


def reference_kedges(k_edges, box_size):
    """(k_edges / kF, kF) in float32 with kF = 2 pi / box (src/correlations.py:12,42)."""
    if isinstance(k_edges, torch.Tensor):
        k_edges = k_edges.detach().cpu().numpy()
    kf = _F32(_F32(2.0 * np.pi) / _box_f32(box_size))
    ke = np.asarray(k_edges, dtype=np.float32).reshape(-1)
    return (ke / kf).astype(np.float32), kf


def default_kedges(n_mesh: int, box_size: float) -> np.ndarray:
    """k edges from kF to k_Nyquist in steps of kF (h/Mpc), as float32."""
    kf = 2.0 * np.pi / float(box_size)
    return np.arange(kf, np.pi * n_mesh / float(box_size), kf).astype(np.float32)


def _cubic_mesh(delta) -> torch.Tensor:
    d = _native.as_cuda_f32(delta, name="delta")
    if d.ndim != 3 or not (d.shape[0] == d.shape[1] == d.shape[2]):
        raise ValueError(f"delta must be a cubic 3-D mesh, got shape {tuple(d.shape)}")
    return d


def _binned_power(d: torch.Tensor, kedges_grid: np.ndarray, box: np.float32):
    N = int(d.shape[0])
    dev = d.device
    bins = _native.bins_for(kedges_grid, N, dev)
    plan = _native.fft_plan(N, 1, dev)
    spec = torch.empty(plan.spectrum_floats, dtype=torch.float32, device=dev)
    plan.execute(d, spec)
    ps = _native.power(spec, 1, bins, mas_order=2, ells=_lib.ELL0 | _lib.ELL2 | _lib.ELL4, z_pitch=plan.pitch)
    pk, _ = _native.normalize(ps, n_mesh=N, box_size=float(box))
    return ps, pk


def powspec_vec(delta, box_size, k_edges):
    """Drop-in for src/correlations.py:7-56 (``powspec_vec``)."""
    d = _cubic_mesh(delta)
    kedges, kf = reference_kedges(k_edges, box_size)
    ps, pk = _binned_power(d, kedges, _box_f32(box_size))
    k3d = ((_F32(0.5) * (kedges[1:] + kedges[:-1])) * kf).astype(np.float32)
    return (torch.from_numpy(k3d).to(d.device), pk.to(torch.float32), ps.nmodes.to(torch.float32))


@functools.lru_cache(maxsize=8)
def _fundamental_last_k(N: int) -> np.ndarray:
    """float32 |k| of the LAST mode (C order over the rfft grid) in each slot int32(|k|).

    src/correlations.py:100 sets k3D[int32(k)] = k for every mode with one
    scatter; the reference's CPU path applies duplicate writes in order, so
    the surviving value is the last mode's.  This is pure geometry.
    """
    h = N // 2
    kmax = int(np.int32(np.sqrt(np.float32(3 * h * h))))
    out = np.zeros(kmax + 1, dtype=np.float32)
    found = np.zeros(kmax + 1, dtype=bool)
    ki = np.where(np.arange(N) > h, np.arange(N) - N, np.arange(N)).astype(np.int64)
    kz2 = (ki[: h + 1] ** 2)[None, :]
    ky2 = (ki ** 2)[:, None]
    for ix in range(N - 1, -1, -1):
        k2 = ki[ix] ** 2 + ky2 + kz2                          # [N, h+1], C order = (iy, iz)
        kk = np.sqrt(k2.astype(np.float32)).ravel()
        slot = kk.astype(np.int32)
        todo = ~found[slot]
        if not todo.any():
            continue
        # last occurrence of each slot in this plane
        rev = slot[::-1]
        uniq, first_rev = np.unique(rev, return_index=True)
        last_idx = kk.size - 1 - first_rev
        new = ~found[uniq]
        out[uniq[new]] = kk[last_idx[new]]
        found[uniq[new]] = True
        if found.all():
            break
    return out


def powspec_vec_fundamental(delta, box_size):
    """Drop-in for src/correlations.py:60-117 (``powspec_vec_fundamental``).

    Bins are the integer shells int32(|k|) = 1 .. kmax (slot 0 dropped, :106-109).
    The returned k3D keeps the reference's formula (:100,110): the |k| of the
    last mode written to each slot, divided by the slot's mode count, times kF.
    """
    d = _cubic_mesh(delta)
    N = int(d.shape[0])
    h = N // 2
    kmax = int(np.int32(np.sqrt(np.float32(3 * h * h))))
    edges = np.arange(kmax + 2, dtype=np.float32)              # slot i = [i, i+1)
    box = _box_f32(box_size)
    # not jitted in the reference: kF is a Python float64, rounded where it meets float32 (:64,:110)
    kf = _F32(2.0 * np.pi / float(box_size))
    ps, pk = _binned_power(d, edges, box)
    nmodes = ps.nmodes.to(torch.float32)
    lastk = torch.from_numpy(_fundamental_last_k(N)).to(d.device)
    k3d = (lastk / nmodes) * float(kf)
    return k3d[1:], pk[1:].to(torch.float32), nmodes[1:]


def reference_sedges(s_edges, box_size, n_mesh: int):
    """Separation edges in cell units as the reference computes them in float32:
    k_edges = kF * s_edges * dims / box_size, kedges = k_edges / kF (src/correlations.py:124-125,172)."""
    if isinstance(s_edges, torch.Tensor):
        s_edges = s_edges.detach().cpu().numpy()
    box = _box_f32(box_size)
    kf = _F32(_F32(2.0 * np.pi) / box)
    se = np.asarray(s_edges, dtype=np.float32).reshape(-1)
    k_edges = (((kf * se).astype(np.float32) * _F32(n_mesh)).astype(np.float32) / box).astype(np.float32)
    return (k_edges / kf).astype(np.float32)


def _xi(d: torch.Tensor, box: np.float32, s_edges, nan_mu_at_origin: bool):
    """(r3D, xi3D, Nmodes3D) of a density contrast mesh through gbp_xi."""
    import ctypes as C
    N = int(d.shape[0])
    dev = d.device
    kedges = reference_sedges(s_edges, box, N)
    bins = _native.bins_for(kedges, N, dev)
    plan = _native.fft_plan(N, 1, dev)
    lib = _lib.load()
    need = C.c_size_t(0)
    _lib.check(lib.gbp_xi_workspace_size(plan.handle, bins.handle, C.byref(need)), "gbp_xi_workspace_size")
    spec = torch.empty(plan.spectrum_floats, dtype=torch.float32, device=dev)
    field = torch.empty((N, N, N), dtype=torch.float32, device=dev)
    ws = _native.workspace(need.value, dev)
    nb = bins.n_bins
    sums = torch.empty((nb, 3), dtype=torch.float64, device=dev)
    counts = torch.empty(nb, dtype=torch.int64, device=dev)
    p = lambda t: C.c_void_p(t.data_ptr())
    _lib.check(lib.gbp_xi(plan.handle, p(d), p(spec), p(field), bins.handle, 2, int(nan_mu_at_origin), p(sums),
                          p(counts), p(ws), ws.numel(), _native._stream_of(dev)), "gbp_xi")
    n3 = float(N) ** 3
    nm = counts.to(torch.float64)
    nm = torch.where(nm == 0, torch.full_like(nm, float("inf")), nm)               # :180
    xi = sums / nm[:, None] / (n3 * n3) * torch.tensor([1.0, 5.0, 9.0], dtype=torch.float64, device=dev)
    r3d = ((_F32(0.5) * (kedges[1:] + kedges[:-1])) * (box * _F32(1.0) / _F32(N))).astype(np.float32)  # :185
    return torch.from_numpy(r3d).to(dev), xi.to(torch.float32), nm.to(torch.float32)


def xi_vec(delta, box_size, s_edges):
    """Drop-in for src/correlations.py:120-187 (``xi_vec``): (r3D, xi3D, Nmodes3D).

    |delta_k|^2 with the CIC correction, inverse FFT, separation shells in
    cell units on the full grid, L_0, L_2, L_4 of mu = r_z / r (NaN at r = 0,
    as the reference's 0/0), xi_l = (2l+1) sum / N_cells / N^3 (the inverse
    transform's own 1/N^3 included), empty bins N = inf.
    """
    d = _cubic_mesh(delta)
    return _xi(d, _box_f32(box_size), s_edges, nan_mu_at_origin=True)


def compute_2pt_correlations(delta, box_size, s_edges, k_edges):
    """Drop-in for src/correlations.py:641-712: (k3D, Pk3D, Nmodes3D_pk, r3D, xi3D), mu = 0 at r = 0."""
    d = _cubic_mesh(delta)
    k3d, pk, nm = powspec_vec(d, box_size, k_edges)
    r3d, xi, _ = _xi(d, _box_f32(box_size), s_edges, nan_mu_at_origin=False)
    return k3d, pk, nm, r3d, xi


def bispec_shells(box_size, k1, k2, theta):
    """src/correlations.py:340-358 in float32: k_all = (k1, k2, k3(theta)), k3 = |k1 + k2| at angle theta,
    and the shell limits (k_all -+ kF) / kF in units of kF.  Returns (k_all, k_min, k_max, theta)."""
    box = _box_f32(box_size)
    kF = _F32(_F32(2.0 * np.pi) / box)                                           # :340
    theta = np.asarray(theta.detach().cpu() if isinstance(theta, torch.Tensor) else theta, dtype=np.float32)
    if theta.ndim != 1:
        raise ValueError("theta must be a 1-D array of angles")
    k1f, k2f = _F32(k1), _F32(k2)
    k3 = np.sqrt((k2f * np.sin(theta)) ** 2 + (k2f * np.cos(theta) + k1f) ** 2).astype(np.float32)   # :351
    k_all = np.concatenate([np.array([k1f, k2f], np.float32), k3]).astype(np.float32)               # :352-355
    return k_all, ((k_all - kF) / kF).astype(np.float32), ((k_all + kF) / kF).astype(np.float32), theta


def _elementary_bins(k_min: np.ndarray, k_max: np.ndarray):
    """Sorted distinct shell limits (+ one edge above them all, so that the closed last bin of the
    histogram rule is never a shell's) and each shell's [first, one-past-last) elementary bin."""
    e = np.unique(np.concatenate([k_min, k_max]).astype(np.float32))
    top = _F32(e[-1] + max(_F32(1.0), abs(e[-1])))
    edges = np.append(e, top).astype(np.float32)
    lo = np.searchsorted(edges, k_min, side="left")
    hi = np.searchsorted(edges, k_max, side="left")
    return edges, np.stack([lo, hi], axis=1).astype(np.int32)


def bispectrum(delta, box_size, k1, k2, theta, *, mas_order: int = 2):
    """The bispectrum estimator of src/correlations.py:334-462 through gbp_bispec, in double:
    (k_all [S] float32, P [S], B [S-2], Q [S-2], modes per shell [S]) as CUDA tensors, S = len(theta) + 2."""
    import ctypes as C
    d = _cubic_mesh(delta)
    N = int(d.shape[0])
    dev = d.device
    k_all, k_min, k_max, theta_f = bispec_shells(box_size, k1, k2, theta)
    edges, shell_bins = _elementary_bins(k_min, k_max)
    bins = _native.bins_for(edges, N, dev)
    plan = _native.fft_plan(N, 1, dev)
    lib = _lib.load()
    need = C.c_size_t(0)
    _lib.check(lib.gbp_bispec_workspace_size(plan.handle, bins.handle, C.byref(need)), "gbp_bispec_workspace_size")
    spec = torch.empty(plan.spectrum_floats, dtype=torch.float32, device=dev)
    ws = _native.workspace(need.value, dev)
    S = k_all.size
    sb = torch.from_numpy(shell_bins).to(dev)
    pk = torch.empty(S, dtype=torch.float64, device=dev)
    bk = torch.empty(max(S - 2, 1), dtype=torch.float64, device=dev)
    qk = torch.empty(max(S - 2, 1), dtype=torch.float64, device=dev)
    nm = torch.empty(S, dtype=torch.int64, device=dev)
    p = lambda t: C.c_void_p(t.data_ptr())
    _lib.check(lib.gbp_bispec(plan.handle, p(d), p(spec), bins.handle, int(mas_order), p(sb), S,
                              float(_box_f32(box_size)), p(pk), p(bk), p(qk), p(nm), p(ws), ws.numel(),
                              _native._stream_of(dev)), "gbp_bispec")
    return torch.from_numpy(k_all).to(dev), pk, bk[: S - 2], qk[: S - 2], nm


def bispec(delta, box_size, k1, k2, theta):
    """Drop-in for src/correlations.py:334-462 (``bispec``): (k_all, Pk, theta, B, Q), float32 CUDA tensors.

    Shells [k_i - kF, k_i + kF) around k1, k2 and k3(theta); CIC window on the amplitude; P of every
    shell, B and the reduced bispectrum Q = B / (P1 P2 + P1 P3 + P2 P3) per angle.
    """
    k_all, pk, bk, qk, _ = bispectrum(delta, box_size, k1, k2, theta, mas_order=2)
    _, _, _, theta_f = bispec_shells(box_size, k1, k2, theta)
    dev = pk.device
    return (k_all, pk.to(torch.float32), torch.from_numpy(theta_f).to(dev), bk.to(torch.float32),
            qk.to(torch.float32))


def compute_all_correlations(delta, box_size, s_edges, k_edges, k1, k2, theta):
    """Drop-in for src/correlations.py:464-637: (k3D, Pk3D, Nmodes3D_pk, r3D, xi3D, Nmodes3D_xi, k_all, Pk,
    theta, B, Q), float32 CUDA tensors.

    P_l(k) and xi_l(r) as ``compute_2pt_correlations`` (mu = 0 at r = 0), the xi shells' cell counts
    (inf for an empty shell, as the reference), and the bispectrum of ``bispec``; the contrast is
    transformed once per estimator on the device.
    """
    d = _cubic_mesh(delta)
    k3d, pk, nm = powspec_vec(d, box_size, k_edges)
    r3d, xi, nmx = _xi(d, _box_f32(box_size), s_edges, nan_mu_at_origin=False)
    k_all, pkb, th, bk, qk = bispec(d, box_size, k1, k2, theta)
    return k3d, pk, nm, r3d, xi, nmx, k_all, pkb, th, bk, qk
