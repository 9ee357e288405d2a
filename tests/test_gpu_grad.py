"""Gradients of P_l(k) with respect to positions and weights (gbp_power_backward + gbp_deposit_backward)
against torch autograd through the float64 estimator (tests/fp64_torch.py)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mas,interlace,weights,N", [("cic", False, True, 32), ("tsc", True, True, 32),
                                                     ("pcs", True, False, 32), ("tsc", False, False, 32),
                                                     ("tsc", True, True, 64), ("cic", False, False, 64)])
def test_gradients_match_fp64_autograd(mas, interlace, weights, N):
    """N = 32: cuFFT spectra (rows of N/2+1); N = 64: the library transform's (rows of N/2+8)."""
    import fp64_torch as F
    from gbpowspec.grad import power_multipoles_diff
    from gbpowspec.pipeline import PkConfig
    from gbpowspec.synth import lognormal_catalogue
    from gbpowspec._lib import MAS
    box, n = 400.0, 3000
    x, y, z = lognormal_catalogue(n, box, grid=32, seed=5)
    rng = np.random.default_rng(6)
    w = rng.uniform(0.5, 1.5, n).astype(np.float32) if weights else None
    cfg = PkConfig(n_mesh=N, box_size=box, mas=mas, interlace=interlace)
    nb = cfg.kedges_grid().size - 1
    g = torch.from_numpy(rng.standard_normal((nb, 3))).cuda()

    t = [torch.from_numpy(a).cuda().requires_grad_(True) for a in (x, y, z)]
    tw = None if w is None else torch.from_numpy(w).cuda().requires_grad_(True)
    pk = power_multipoles_diff(*t, tw, box_size=box, n_mesh=N, mas=mas, interlace=interlace)
    torch.nan_to_num(pk * g, nan=0.0).sum().backward()

    r = [torch.from_numpy(a).cuda().to(torch.float64).requires_grad_(True) for a in (x, y, z)]
    rw = None if w is None else torch.from_numpy(w).cuda().to(torch.float64).requires_grad_(True)
    ref = F.power_multipoles_autograd(*r, rw, box=box, N=N, mas=MAS[mas], interlace=interlace,
                                      kedges_grid=cfg.kedges_grid())
    # forward values: float32 round-off relative to each bin's monopole before the shot noise is taken off
    # (P_2, P_4 and the shot-subtracted P_0 may cancel to ~0)
    got, want = pk.detach().cpu().numpy(), ref.detach().cpu().numpy()
    scale = np.abs(want[:, :1]) + box ** 3 / n
    assert np.array_equal(np.isnan(got), np.isnan(want))
    assert np.nanmax(np.abs(got - want) / scale) < 1e-5
    torch.nan_to_num(ref * g, nan=0.0).sum().backward()

    for a, b in zip(t, r):
        ga, gb = a.grad.double(), b.grad
        rel = float((ga - gb).norm() / gb.norm())
        assert rel < 1e-3, rel
    if w is not None:
        rel = float((tw.grad.double() - rw.grad).norm() / rw.grad.norm())
        assert rel < 1e-3, rel


def test_gradient_descent_fits_a_target_monopole():
    """Gradient descent on particle positions drives P_0 of a uniform catalogue to the P_0 of a
    clustered one (the reference's use case: fitting positions through the estimator).  Loss
    sum_b ((P_0 - T) / T)^2 over the first 8 bins, TSC, no shot-noise subtraction, steps of at
    most 0.25 length units along -grad; the FP64 torch estimator takes the same path
    (0.124 -> 0.0007 in 8 steps)."""
    from gbpowspec.grad import power_multipoles_diff
    from gbpowspec.synth import lognormal_catalogue, uniform_catalogue
    N, box, n = 32, 500.0, 4000
    kw = dict(box_size=box, n_mesh=N, mas="tsc", interlace=False, shot_noise=False)
    target = power_multipoles_diff(*(torch.from_numpy(a).cuda() for a in lognormal_catalogue(n, box, grid=32, seed=9)),
                                   **kw).detach()[:8, 0]
    pos = [torch.from_numpy(a).cuda().requires_grad_(True) for a in uniform_catalogue(n, box, seed=10)]
    losses = []
    for _ in range(10):
        pk = power_multipoles_diff(*pos, **kw)
        loss = (((pk[:8, 0] - target) / target) ** 2).sum()
        grads = torch.autograd.grad(loss, pos)
        gmax = max(float(g.abs().max()) for g in grads)
        with torch.no_grad():
            for p, g in zip(pos, grads):
                p.sub_(0.25 * g / gmax).remainder_(box)
        losses.append(float(loss.detach()))
    assert losses[-1] < 0.05 * losses[0], losses
