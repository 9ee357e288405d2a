"""Differentiable P_l(k): gradients with respect to particle positions and weights.

The reference exists to differentiate its estimator (tests/lognormal.py:60-103
optimises particle positions through cic_mas_vec -> powspec_vec with JAX
autodiff).  `power_multipoles_diff` is the same capability for the production
estimator (B-spline deposit, optional interlacing, mass normalisation, shot
noise), as a torch.autograd.Function whose backward pass runs on the GPU:

    pk = power_multipoles_diff(x, y, z, w, box_size=1000.0, n_mesh=64)   # [nb, 3]
    loss = ((pk[:, 0] - target) ** 2).sum()
    loss.backward()                                                      # x.grad, y.grad, z.grad, w.grad

Forward: deposit (gbp_deposit) -> R2C (gbp_fft_r2c, spectra kept) -> binning
(gbp_power) -> normalisation.  Backward: gbp_power_backward forms the adjoint
spectrum from dLoss/dP and transforms it back to gradient meshes (C2R);
gbp_deposit_backward gathers them at the particles with the B-spline
derivatives; the explicit dependence of L^3/M^2 and of the shot noise on the
weights (M = sum w, Q = sum w^2) is added here:
    dP_l/dM = -2 P_l / M,   dP_0/dQ = -L^3 / M^2.
Empty bins (NaN) carry no gradient.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib, _native
from ._lib import check
from .pipeline import PkConfig

__all__ = ["power_multipoles_diff"]


def _p(t):
    return None if t is None else C.c_void_p(t.data_ptr())


class _PowerFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, y, z, w, cfg: PkConfig):
        dev = x.device
        N, G = cfg.n_mesh, cfg.grids
        xs, ys, zs = (t.detach().contiguous().to(torch.float32) for t in (x, y, z))
        ws = None if w is None else w.detach().contiguous().to(torch.float32)
        inv = np.float32(N / cfg.box_size)
        mesh, stats = _native.deposit(xs, ys, zs, ws, n_mesh=N, inv_cell=inv, origin=cfg.origin,
                                      mas=cfg.mas_order, interlace=cfg.interlace)
        plan = _native.fft_plan(N, G, dev)
        spec = torch.empty(plan.spectrum_floats, dtype=torch.float32, device=dev)
        plan.execute(mesh, spec)
        bins = _native.bins_for(cfg.kedges_grid(), N, dev)
        mask = _lib.ELL0 | _lib.ELL2 | _lib.ELL4
        sums = _native.power(spec, G, bins, mas_order=cfg.mas_order, ells=mask, z_pitch=plan.pitch, mass=stats)
        pk, _ = _native.normalize(sums, n_mesh=N, box_size=cfg.box_size, mass=stats, stats=stats,
                                  subtract_shot=cfg.shot_noise)
        ctx.cfg, ctx.plan, ctx.bins = cfg, plan, bins
        ctx.has_w = w is not None
        ctx.save_for_backward(xs, ys, zs, ws if ws is not None else torch.empty(0, device=dev), spec, stats,
                              sums.nmodes, pk)
        return pk

    @staticmethod
    def backward(ctx, grad_pk):
        xs, ys, zs, ws, spec, stats, nmodes, pk = ctx.saved_tensors
        cfg, plan, bins = ctx.cfg, ctx.plan, ctx.bins
        dev = xs.device
        N, G = cfg.n_mesh, cfg.grids
        ws = ws if ctx.has_w else None
        g = torch.nan_to_num(grad_pk.detach().to(torch.float64), nan=0.0).contiguous()
        empty = ~torch.isfinite(pk)
        g = torch.where(empty, torch.zeros_like(g), g)
        lib = _lib.load()
        need = C.c_size_t(0)
        check(lib.gbp_power_backward_workspace_size(plan.handle, C.byref(need)), "gbp_power_backward_workspace_size")
        wsb = _native.workspace(need.value, dev)
        gmesh = torch.empty((G, N, N, N), dtype=torch.float32, device=dev)
        stream = _native._stream_of(dev)
        check(lib.gbp_power_backward(_p(spec), plan.handle, bins.handle, cfg.mas_order, _p(g), _p(nmodes),
                                     _p(stats), float(cfg.box_size), _p(gmesh), _p(wsb), wsb.numel(), stream),
              "gbp_power_backward")
        n = xs.numel()
        gx, gy, gz = (torch.empty(n, dtype=torch.float32, device=dev) for _ in range(3))
        gw = torch.empty(n, dtype=torch.float32, device=dev)
        inv = float(np.float32(N / cfg.box_size))
        o = [float(np.float32(v)) for v in cfg.origin]
        check(lib.gbp_deposit_backward(_p(xs), _p(ys), _p(zs), _p(ws), n, o[0], o[1], o[2], inv, N, cfg.mas_order,
                                       int(cfg.interlace), _p(gmesh), _p(gx), _p(gy), _p(gz), _p(gw), stream),
              "gbp_deposit_backward")
        grad_w = None
        if ctx.has_w and ctx.needs_input_grad[3]:
            st = _native.read_stats(stats)
            M = float(st.mass[0])
            pk0 = torch.nan_to_num(pk, nan=0.0)
            c_mass = float((g * (-2.0 * pk0 / M)).sum())               # dP_l/dM = -2 P_l / M
            grad_w = gw.to(torch.float64) + c_mass
            if cfg.shot_noise:
                grad_w = grad_w - 2.0 * ws.to(torch.float64) * (cfg.box_size ** 3 / M ** 2) * float(g[:, 0].sum())
            grad_w = grad_w.to(ws.dtype)
        return gx, gy, gz, grad_w, None


def power_multipoles_diff(x, y, z, w=None, *, box_size: float, n_mesh: int, mas: str = "tsc", interlace: bool = True,
                          shot_noise: bool = True, k_edges=None, origin=(0.0, 0.0, 0.0)) -> torch.Tensor:
    """P_0,2,4(k) [nb, 3] (float64) of float32 CUDA particle tensors, differentiable in x, y, z and w."""
    cfg = PkConfig(n_mesh=int(n_mesh), box_size=float(box_size), mas=mas, interlace=bool(interlace),
                   shot_noise=bool(shot_noise),
                   k_edges=None if k_edges is None else tuple(np.asarray(k_edges, np.float32).tolist()),
                   origin=tuple(float(v) for v in origin))
    return _PowerFn.apply(x, y, z, w, cfg)
