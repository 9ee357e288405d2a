"""TEST ORACLE -- not product code.  Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg may import this module, and only as the checker or
as the timed CPU stand-in for the reference.

A numpy restatement, in float32 where the reference computes in float32, of
jax-powspec's P(k) path (dforero0896/jax-powspec, src/mas.py and
src/correlations.py).  Each function cites the reference lines it follows.

JAX itself is absent from this environment, so the JAX primitives the
reference relies on are restated from their published semantics:
  * ``x.at[idx].add(v)`` (scatter-add): updates applied in order; negative
    indices count once from the end, indices still outside [0, n) drop the
    update (jax's default FILL_OR_DROP for scatters).  ``np.add.at`` on a
    float32 array accumulates sequentially in float32, like XLA:CPU.
  * ``jnp.histogram(a, bins, weights)``: ``searchsorted(bins, a, 'right')``,
    values equal to the last edge go to the last bin, then
    ``zeros(len(bins)).at[idx].add(weights)[1:]``.
  * ``jnp.int32(x)`` truncates toward zero; ``jnp.sqrt`` of an int32 array is
    computed in float32 (x64 disabled).
  * ``jnp.fft.rfftn`` in complex64 (scipy.fft's single-precision pocketfft
    stands in for ducc).
The restatement is pinned against fixtures produced by running the
reference's own source (tests/golden/make_golden.py).
"""
from __future__ import annotations

import numpy as np
import scipy.fft

F32 = np.float32


def _f32(v) -> np.float32:
    return F32(np.asarray(v, dtype=np.float32).reshape(()))


def scatter_add(mesh: np.ndarray, idx, vals: np.ndarray) -> None:
    """In-place ``mesh.at[idx].add(vals)`` with jax's default index rules."""
    ok = np.ones(vals.shape, dtype=bool)
    norm = []
    for a, n in zip(idx, mesh.shape):
        a = np.asarray(a).astype(np.int64)
        a = np.where(a < 0, a + n, a)
        ok &= (a >= 0) & (a < n)
        norm.append(a)
    np.add.at(mesh, tuple(a[ok] for a in norm), vals.astype(mesh.dtype)[ok])


def _cube(v):
    """v**3 as lax.integer_pow evaluates it (binary exponentiation): v * (v * v)."""
    return v * (v * v)


def _inv_bin_size(box_size, n_bins):
    bin_size = _f32(box_size) / F32(n_bins)          # src/mas.py:100 (and :17)
    return F32(F32(1.0) / bin_size)                  # src/mas.py:101 (and :18)


def cic_mas_vec(delta, x, y, z, w, n_part, xmin, ymin, zmin, box_size, n_bins, wrap):
    """src/mas.py:88-153."""
    inv = _inv_bin_size(box_size, n_bins)
    pos = [(np.asarray(c, F32) - _f32(o)) * inv for c, o in ((x, xmin), (y, ymin), (z, zmin))]  # :103-105
    i0 = [p.astype(np.int32) for p in pos]                                  # :107-109 (trunc)
    dd = [p - i.astype(F32) for p, i in zip(pos, i0)]                       # :111-113
    ip = [i + 1 for i in i0]                                                 # :115-117
    n = int(n_bins)
    if wrap:                                                                  # :119-122
        ip = [np.mod(i + n, n) for i in ip]
    else:                                                                     # :123-134
        new_ip, new_dd = [], []
        for i, d in zip(ip, dd):
            i = np.where(i >= n, 0, i)
            d = np.where(i >= n, F32(0), d)       # tests the already-zeroed index: never true
            new_ip.append(i)
            new_dd.append(d.astype(F32))
        ip, dd = new_ip, new_dd
    md = [F32(1.0) - d for d in dd]                                          # :138-140
    w = np.ones_like(pos[0]) if w is None else np.asarray(w, F32)
    (ix, iy, iz), (ixp, iyp, izp) = i0, ip
    (dx, dy, dz), (mx, my, mz) = dd, md
    out = np.array(delta, dtype=F32, copy=True)
    scatter_add(out, (ix, iy, iz), mx * my * mz * w)                          # :142
    scatter_add(out, (ixp, iy, iz), dx * my * mz * w)                         # :143
    scatter_add(out, (ix, iyp, iz), mx * dy * mz * w)                         # :144
    scatter_add(out, (ix, iy, izp), mx * my * dz * w)                         # :145
    scatter_add(out, (ixp, iyp, iz), dx * dy * mz * w)                        # :147
    scatter_add(out, (ixp, iy, izp), dx * my * dz * w)                        # :148
    scatter_add(out, (ix, iyp, izp), mx * my * dz * w)                        # :149 (sic: mdy)
    scatter_add(out, (ixp, iyp, izp), dx * dy * dz * w)                       # :151
    return out


def cic_mas(delta, x, y, z, w, n_part, xmin, ymin, zmin, box_size, n_bins, wrap):
    """src/mas.py:5-87: a lax.scan over particles doing 8 scatter-adds each."""
    inv = _inv_bin_size(box_size, n_bins)
    n = int(n_bins)
    out = np.array(delta, dtype=F32, copy=True)
    xs, ys, zs = (np.asarray(c, F32) for c in (x, y, z))
    ws = np.ones_like(xs) if w is None else np.asarray(w, F32)
    o = (_f32(xmin), _f32(ymin), _f32(zmin))
    for p in range(xs.size):
        pos = [(c[p] - oo) * inv for c, oo in zip((xs, ys, zs), o)]          # :44-46
        i0 = [int(np.int32(q)) for q in pos]                                  # :48-50
        dd = [F32(q - F32(i)) for q, i in zip(pos, i0)]                       # :52-54
        md = [F32(F32(1.0) - d) for d in dd]                                  # :56-58 (before the cond)
        ip = [i + 1 for i in i0]                                              # :60-62
        if wrap:                                                              # :20-28
            ip = [i - n if i >= n else i for i in ip]
        else:                                                                 # :30-38
            for k in range(3):
                if ip[k] >= n:
                    ip[k], dd[k] = 0, F32(0.0)
        wt = ws[p]
        (ix, iy, iz), (ixp, iyp, izp) = i0, ip
        (dx, dy, dz), (mx, my, mz) = dd, md
        for idx, val in (((ix, iy, iz), mx * my * mz * wt),                   # :69
                         ((ixp, iy, iz), dx * my * mz * wt),                  # :70
                         ((ix, iyp, iz), mx * dy * mz * wt),                  # :71
                         ((ix, iy, izp), mx * my * dz * wt),                  # :72
                         ((ixp, iyp, iz), dx * dy * mz * wt),                 # :74
                         ((ixp, iy, izp), dx * my * dz * wt),                 # :75
                         ((ix, iyp, izp), mx * my * dz * wt),                 # :76 (sic: mdy)
                         ((ixp, iyp, izp), dx * dy * dz * wt)):               # :78
            scatter_add(out, tuple(np.array([i]) for i in idx), np.array([val], F32))
    return out


def histogram_f32(a: np.ndarray, edges: np.ndarray, weights: np.ndarray | None):
    """jnp.histogram with array bins: right-searchsorted, last edge closed, float32 scatter-add."""
    a = np.asarray(a, F32).ravel()
    edges = np.asarray(edges, F32)
    idx = np.searchsorted(edges, a, side="right")
    idx = np.where(a == edges[-1], edges.size - 1, idx)
    wts = np.ones_like(a) if weights is None else np.asarray(weights, F32).ravel()
    counts = np.zeros(edges.size, F32)
    keep = idx < edges.size                      # the out-of-range index is dropped
    np.add.at(counts, idx[keep], wts[keep])
    return counts[1:]


def _kgrid(dims: int):
    middle = dims // 2
    r = np.arange(dims, dtype=np.int32)
    ki = np.where(r > middle, r - dims, r).astype(np.int32)                     # src/correlations.py:25
    kx = np.broadcast_to(ki[:, None, None], (dims, dims, middle + 1))           # :29
    ky = np.broadcast_to(ki[None, :, None], (dims, dims, middle + 1))           # :30
    kz = np.broadcast_to(ki[None, None, : middle + 1], (dims, dims, middle + 1))  # :31
    return kx, ky, kz


def _cic_correction(kk: np.ndarray, dims: int) -> np.ndarray:
    """(1 / jnp.sinc(prefact*k / pi))**2 in float32 (src/correlations.py:15,20-21)."""
    prefact = F32(np.pi / dims)
    x = (prefact * kk.astype(F32)) / F32(np.pi)
    s = np.sinc(x).astype(F32)
    return (F32(1.0) / s) ** F32(2.0)


def _power_core(delta, box_size):
    dims = delta.shape[0]
    delta_k = scipy.fft.rfftn(np.asarray(delta, F32), axes=(0, 1, 2)).astype(np.complex64)  # :22
    kx, ky, kz = _kgrid(dims)
    corr = _cic_correction(kx, dims) * _cic_correction(ky, dims) * _cic_correction(kz, dims)  # :32
    k = np.sqrt((kx * kx + ky * ky + kz * kz).astype(F32))                  # :34
    with np.errstate(invalid="ignore", divide="ignore"):
        mu = np.where(k == 0, F32(0), kz.astype(F32) / k).astype(F32)       # :36-37
    mu2 = (mu ** 2).ravel()                                                 # :38
    delta_k = (delta_k * corr).astype(np.complex64)                         # :39
    delta2 = (delta_k * delta_k.conj()).real.astype(F32).ravel()            # :40
    return dims, k, mu2, delta2


def powspec_vec(delta, box_size, k_edges):
    """src/correlations.py:7-56."""
    dims, k, mu2, delta2 = _power_core(delta, box_size)
    kF = F32(F32(2.0 * np.pi) / _f32(box_size))                              # :12
    kedges = (np.asarray(k_edges, F32) / kF).astype(F32)                     # :42
    kf = k.ravel()
    mono = histogram_f32(kf, kedges, delta2)                                  # :45
    quad = histogram_f32(kf, kedges, delta2 * (F32(3.0) * mu2 - F32(1.0)) / F32(2.0))       # :46
    hexa = histogram_f32(kf, kedges, delta2 * (F32(35.0) * mu2 * mu2 - F32(30.0) * mu2 + F32(3.0)) / F32(8.0))  # :47
    nmodes = histogram_f32(kf, kedges, None)                                  # :48
    norm = _cube(_f32(box_size) / F32(dims ** 2))
    with np.errstate(invalid="ignore", divide="ignore"):
        pk = np.zeros((mono.size, 3), F32)
        pk[:, 0] = mono / nmodes * norm                                       # :50
        pk[:, 1] = quad / nmodes * F32(5.0) * norm                            # :51
        pk[:, 2] = hexa / nmodes * F32(9.0) * norm                            # :52
    k3d = (F32(0.5) * (kedges[1:] + kedges[:-1])) * kF                        # :54
    return k3d.astype(F32), pk, nmodes


def powspec_vec_fundamental(delta, box_size):
    """src/correlations.py:60-117 (k3D keeps the last-writer scatter-set of :100).

    This function is not jitted in the reference, so with a Python float box
    size its constants kF (:64) and (box/dims^2)^3 (:112) are Python float64
    values, rounded to float32 only where they meet a float32 array.
    """
    dims, k, mu2, delta2 = _power_core(delta, box_size)
    middle = dims // 2
    kF = F32(2.0 * np.pi / float(box_size))                                   # :64
    kmax = int(np.int32(np.sqrt(F32(3 * middle * middle))))                   # :69
    kf = k.ravel()
    kidx = kf.astype(np.int32)                                                # :87
    k3d = np.zeros(kmax + 1, F32)
    k3d[kidx] = kf            # numpy fancy assignment keeps the last duplicate   :100
    pk = np.zeros((kmax + 1, 3), F32)
    np.add.at(pk[:, 0], kidx, delta2)                                         # :101
    np.add.at(pk[:, 1], kidx, delta2 * (F32(3.0) * mu2 - F32(1.0)) / F32(2.0))  # :102
    np.add.at(pk[:, 2], kidx, delta2 * (F32(35.0) * mu2 * mu2 - F32(30.0) * mu2 + F32(3.0)) / F32(8.0))  # :103
    nmodes = np.zeros(kmax + 1, F32)
    np.add.at(nmodes, kidx, F32(1.0))                                         # :104
    k3d, nmodes, pk = k3d[1:], nmodes[1:], pk[1:]                             # :106-108
    norm = F32((float(box_size) / dims ** 2) ** 3)
    with np.errstate(invalid="ignore", divide="ignore"):
        k3d = k3d / nmodes * kF                                               # :110
        out = np.zeros_like(pk)
        out[:, 0] = pk[:, 0] / nmodes * norm                                  # :112
        out[:, 1] = pk[:, 1] / nmodes * F32(5.0) * norm                       # :113
        out[:, 2] = pk[:, 2] / nmodes * F32(9.0) * norm                       # :114
    return k3d.astype(F32), out, nmodes


def _xi_core(delta, box_size, s_edges, mu_zero_at_origin: bool):
    """src/correlations.py:120-187 (xi_vec) and :692-712 (the xi half of compute_2pt_correlations)."""
    dims = delta.shape[0]
    box = _f32(box_size)
    kF = F32(F32(2.0 * np.pi) / box)                                          # :124 / :646
    s_edges = np.asarray(s_edges, F32)
    k_edges = (((kF * s_edges).astype(F32) * F32(dims)).astype(F32) / box).astype(F32)   # :125 / :698
    kedges = (k_edges / kF).astype(F32)                                       # :172 / :699
    delta_k = scipy.fft.rfftn(np.asarray(delta, F32), axes=(0, 1, 2)).astype(np.complex64)
    kx, ky, kz = _kgrid(dims)
    corr = _cic_correction(kx, dims) * _cic_correction(ky, dims) * _cic_correction(kz, dims)
    delta_k = (delta_k * corr).astype(np.complex64)                            # :147-148 / :666
    delta2 = (delta_k * delta_k.conj()).astype(np.complex64)                   # :149 (complex)
    if mu_zero_at_origin:
        delta2 = delta2.real.astype(F32)                                       # :674 takes .real first
    delta_xi = scipy.fft.irfftn(delta2.astype(np.complex64), s=delta.shape, axes=(0, 1, 2)).astype(F32)  # :151 / :697
    middle = dims // 2
    r = np.arange(dims, dtype=np.int32)
    ki = np.where(r > middle, r - dims, r).astype(np.int32)
    gx = ki[:, None, None]
    gy = ki[None, :, None]
    gz = ki[None, None, :]
    kk = np.sqrt((gx * gx + gy * gy + gz * gz).astype(F32))                   # :158 / :692
    with np.errstate(invalid="ignore", divide="ignore"):
        mu = (np.broadcast_to(gz, kk.shape).astype(F32) / kk).astype(F32)      # :162 (0/0 -> NaN)
        if mu_zero_at_origin:
            mu = np.where(kk == 0, F32(0), mu).astype(F32)                    # :694
    mu2 = (mu ** 2).ravel()
    kf = kk.ravel()
    w = delta_xi.ravel()
    mono = histogram_f32(kf, kedges, w)
    quad = histogram_f32(kf, kedges, w * (F32(3.0) * mu2 - F32(1.0)) / F32(2.0))
    hexa = histogram_f32(kf, kedges, w * (F32(35.0) * mu2 * mu2 - F32(30.0) * mu2 + F32(3.0)) / F32(8.0))
    nmodes = histogram_f32(kf, kedges, None)
    nmodes = np.where(nmodes == 0, F32(np.inf), nmodes).astype(F32)          # :180 / :705
    d3 = F32(dims ** 3)
    with np.errstate(invalid="ignore", divide="ignore"):
        xi = np.zeros((mono.size, 3), F32)
        xi[:, 0] = mono / nmodes / d3
        xi[:, 1] = quad / nmodes * F32(5.0) / d3
        xi[:, 2] = hexa / nmodes * F32(9.0) / d3
    r3d = (F32(0.5) * (kedges[1:] + kedges[:-1])) * (box * F32(1.0) / F32(dims))   # :185 / :710
    return r3d.astype(F32), xi, nmodes


def xi_vec(delta, box_size, s_edges):
    """src/correlations.py:120-187: (r3D, xi3D, Nmodes3D), mu = 0/0 = NaN at r = 0."""
    return _xi_core(delta, box_size, s_edges, mu_zero_at_origin=False)


def compute_2pt_correlations(delta, box_size, s_edges, k_edges):
    """src/correlations.py:641-712: (k3D, Pk3D, Nmodes3D_pk, r3D, xi3D), mu = 0 at the origin."""
    k3d, pk, nm = powspec_vec(delta, box_size, k_edges)
    r3d, xi, _ = _xi_core(delta, box_size, s_edges, mu_zero_at_origin=True)
    return k3d, pk, nm, r3d, xi


def bispec_shells(box_size, k1, k2, theta):
    """src/correlations.py:340-358: k_all = (k1, k2, k3(theta)) and the shell limits in units of kF, float32.

    bispec is jitted, so the box size, k1 and k2 are float32 scalars there; k3 = |k1 + k2| for the angle
    theta between them.
    """
    box = _f32(box_size)
    kF = F32(F32(2.0 * np.pi) / box)                                           # :340
    theta = np.asarray(theta, F32)
    k1f, k2f = _f32(k1), _f32(k2)
    k3 = np.sqrt((k2f * np.sin(theta)) ** 2 + (k2f * np.cos(theta) + k1f) ** 2).astype(F32)   # :351
    k_all = np.zeros(theta.size + 2, F32)
    k_all[0], k_all[1], k_all[2:] = k1f, k2f, k3                              # :352-355
    k_min = ((k_all - kF) / kF).astype(F32)                                     # :357
    k_max = ((k_all + kF) / kF).astype(F32)                                     # :358
    return k_all, k_min, k_max


def bispec(delta, box_size, k1, k2, theta):
    """src/correlations.py:334-462: (k_all, Pk, theta, B, Q), every step in float32.

    delta_i = irfftn(mask_i * W delta_k) and I_i = irfftn(mask_i) per shell (:384-387, :410-413,
    :427-431); P_i = sum delta_i^2 / sum I_i^2 * (L / N^2)^3 (:396-400, :421-425, :436-441);
    B = sum delta_1 delta_2 delta_3 / sum I_1 I_2 I_3 * (L^2 / N^3)^3 (:443-449); Q = B / (P1 P2 + P1 P3 +
    P2 P3) (:450).
    """
    delta = np.asarray(delta, F32)
    dims = delta.shape[0]
    box = _f32(box_size)
    theta = np.asarray(theta, F32)
    k_all, k_min, k_max = bispec_shells(box_size, k1, k2, theta)
    delta_k = scipy.fft.rfftn(delta, axes=(0, 1, 2)).astype(np.complex64)    # :363
    kx, ky, kz = _kgrid(dims)
    corr = _cic_correction(kx, dims) * _cic_correction(ky, dims) * _cic_correction(kz, dims)   # :372
    delta_k = (delta_k * corr).astype(np.complex64)                           # :373
    k = np.sqrt((kx * kx + ky * ky + kz * kz).astype(F32))                    # :374

    def fields(i):
        m = (k >= k_min[i]) & (k < k_max[i])                                  # :379
        d = scipy.fft.irfftn((m * delta_k).astype(np.complex64), s=delta.shape, axes=(0, 1, 2)).astype(F32)
        one = scipy.fft.irfftn(m.astype(np.complex64), s=delta.shape, axes=(0, 1, 2)).astype(F32)
        return d, one

    pnorm = _cube(box / F32(dims ** 2))
    bnorm = _cube((box * box) / F32(dims ** 3))
    d1, i1 = fields(0)
    d2, i2 = fields(1)
    pk = np.zeros(theta.size + 2, F32)
    pk[0] = (np.nansum(d1 * d1) / (i1 * i1).sum()) * pnorm                    # :394-400
    pk[1] = (np.nansum(d2 * d2) / (i2 * i2).sum()) * pnorm                    # :419-425
    bk = np.zeros(theta.size, F32)
    qk = np.zeros(theta.size, F32)
    with np.errstate(invalid="ignore", divide="ignore"):
        for j in range(theta.size):                                          # the lax.scan of :427-454
            d3, i3 = fields(j + 2)
            pv = (np.nansum(d3 * d3) / np.nansum(i3 * i3)) * pnorm
            bv = (np.nansum(d1 * d2 * d3) / (i1 * i2 * i3).sum()) * bnorm
            qk[j] = bv / (pk[0] * pk[1] + pk[0] * pv + pk[1] * pv)
            pk[j + 2], bk[j] = pv, bv
    return k_all, pk, theta, bk, qk


def compute_all_correlations(delta, box_size, s_edges, k_edges, k1, k2, theta):
    """src/correlations.py:464-637: P_l(k) and xi_l(r) as compute_2pt_correlations (mu = 0 at the
    origin, the real part of |delta_k|^2 transformed), the xi shells' cell counts (inf when empty), then
    the bispectrum of bispec.  Returns (k3D, Pk3D, Nmodes3D_pk, r3D, xi3D, Nmodes3D_xi, k_all, Pk, theta, B, Q)."""
    k3d, pk, nm = powspec_vec(delta, box_size, k_edges)
    r3d, xi, nmx = _xi_core(delta, box_size, s_edges, mu_zero_at_origin=True)
    k_all, pkb, th, bk, qk = bispec(delta, box_size, k1, k2, theta)
    return k3d, pk, nm, r3d, xi, nmx, k_all, pkb, th, bk, qk
