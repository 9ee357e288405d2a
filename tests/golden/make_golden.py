"""Generate golden fixtures by running jax-powspec's own source.

The reference (dforero0896/jax-powspec) is imported unmodified from its
checkout -- src/mas.py and src/correlations.py -- on top of jaxshim, a numpy
restatement of the JAX primitives those files use (JAX is not installed
here).  Inputs are small and seeded; outputs are written to
tests/golden/*.npz next to this script.  The GPU tests and the CPU oracle are
both checked against these files, which never need the reference at run time.

    python tests/golden/make_golden.py path/to/jax-powspec   (or JAX_POWSPEC_ROOT=...)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
F32 = np.float32


def load_reference(root: str):
    sys.path.insert(0, HERE)
    import jaxshim

    jaxshim.install()
    sys.path.insert(0, root)
    from src import correlations, mas  # noqa: E402  (the reference's own modules)

    return mas, correlations, jaxshim


def particles_with_edges(rng, n, box, n_mesh):
    """Uniform particles plus positions on and beyond the box faces."""
    H = box / n_mesh
    p = rng.uniform(0, box, size=(n, 3)).astype(F32)
    specials = np.array([0.0, box, box - 1e-4, -0.3 * H, -H - 0.2, box + 0.2 * H, 2.3 * box, -1.5 * box,
                         H, 2 * H, 0.5 * H], dtype=F32)
    rows = []
    for s in specials:
        r = rng.uniform(0, box, size=3).astype(F32)
        r[rng.integers(0, 3)] = s
        rows.append(r)
    return np.concatenate([p, np.array(rows, dtype=F32)])


def main(root: str) -> None:
    mas, corr, shim = load_reference(root)
    rng = np.random.default_rng(20261203)
    out = {}

    # ---- deposits: cic_mas_vec (src/mas.py:88-153) and cic_mas (:5-87)
    for name, N, box, n, origin in (("a", 8, 100.0, 300, (0.0, 0.0, 0.0)), ("b", 12, 37.5, 200, None)):
        p = particles_with_edges(rng, n, box, N)
        w = rng.uniform(0.5, 2.0, size=p.shape[0]).astype(F32)
        d0 = (rng.standard_normal((N, N, N)) * 0.1).astype(F32)
        if origin is None:                          # tests/correlations.py:45 passes the minima
            origin = tuple(float(v) for v in p.min(axis=0))
        for wrap in (True, False):
            res = mas.cic_mas_vec(d0, p[:, 0], p[:, 1], p[:, 2], w, p.shape[0], origin[0], origin[1], origin[2],
                                  box, N, wrap)
            out[f"dep_{name}_vec_{int(wrap)}"] = np.asarray(res, dtype=F32)
            sub = slice(0, 64)
            res2 = mas.cic_mas(d0, p[sub, 0], p[sub, 1], p[sub, 2], w[sub], 64, origin[0], origin[1], origin[2],
                               box, N, wrap)
            out[f"dep_{name}_scan_{int(wrap)}"] = np.asarray(res2, dtype=F32)
        out[f"dep_{name}_pos"] = p
        out[f"dep_{name}_w"] = w
        out[f"dep_{name}_delta0"] = d0
        out[f"dep_{name}_meta"] = np.array([N, box, origin[0], origin[1], origin[2]], dtype=np.float64)

    # ---- powspec_vec (src/correlations.py:7-56) on random meshes and edge sets
    cases = []
    for N, box in ((16, 100.0), (9, 50.0), (32, 1000.0)):
        kf = 2 * np.pi / box
        kny = np.pi * N / box
        cases.append((N, box, np.arange(kf, kny, kf).astype(F32)))                       # kF .. kNyq
        cases.append((N, box, np.linspace(0.0, 1.2 * np.sqrt(3) * kny, 37).astype(F32)))  # from 0, beyond kmax
        cases.append((N, box, (F32(kf) * np.arange(1, 9, dtype=F32)).astype(F32)))       # integer shells in f32
    # box = 2 pi: kF == 1 exactly, so edges can sit exactly on sqrtf(k^2) values
    ties = np.sqrt(np.array([1, 2, 3, 4, 5, 6, 8, 9, 12], dtype=F32)).astype(F32)
    cases.append((8, float(F32(2 * np.pi)), ties))
    for i, (N, box, edges) in enumerate(cases):
        delta = rng.standard_normal((N, N, N)).astype(F32)
        k3d, pk, nm = corr.powspec_vec(delta, box, edges)
        out[f"pk_{i}_delta"] = delta
        out[f"pk_{i}_edges"] = edges
        out[f"pk_{i}_box"] = np.array([box], dtype=np.float64)
        out[f"pk_{i}_k"] = np.asarray(k3d, F32)
        out[f"pk_{i}_pk"] = np.asarray(pk, F32)
        out[f"pk_{i}_nmodes"] = np.asarray(nm, F32)
    out["pk_ncases"] = np.array([len(cases)])

    # ---- powspec_vec_fundamental (src/correlations.py:60-117)
    for i, (N, box) in enumerate(((16, 100.0), (9, 50.0), (12, 300.0))):
        delta = rng.standard_normal((N, N, N)).astype(F32)
        k3d, pk, nm = corr.powspec_vec_fundamental(delta, box)
        out[f"fund_{i}_delta"] = delta
        out[f"fund_{i}_box"] = np.array([box], dtype=np.float64)
        out[f"fund_{i}_k"] = np.asarray(k3d, F32)
        out[f"fund_{i}_pk"] = np.asarray(pk, F32)
        out[f"fund_{i}_nmodes"] = np.asarray(nm, F32)
    out["fund_ncases"] = np.array([3])

    # ---- the caller pipeline of tests/correlations.py:42-50,78: deposit, normalise, P(k)
    N, box = 16, 200.0
    p = rng.uniform(0, box, size=(4000, 3)).astype(F32)
    w = np.ones(p.shape[0], F32)
    delta = mas.cic_mas_vec(np.zeros((N, N, N), F32), p[:, 0], p[:, 1], p[:, 2], w, p.shape[0], 0.0, 0.0, 0.0,
                            box, N, True)
    delta = delta / delta.mean()
    delta = delta - 1.0
    kf = 2 * np.pi / box
    edges = np.arange(kf, np.pi * N / box, kf).astype(F32)
    k3d, pk, nm = corr.powspec_vec(delta, box, edges)
    out.update(pipe_pos=p, pipe_box=np.array([box]), pipe_N=np.array([N]), pipe_delta=np.asarray(delta, F32),
               pipe_edges=edges, pipe_k=np.asarray(k3d, F32), pipe_pk=np.asarray(pk, F32),
               pipe_nmodes=np.asarray(nm, F32))

    # ---- xi_vec (src/correlations.py:120-187) and compute_2pt_correlations (:641-712)
    xcases = [(16, 100.0, np.arange(0.5, 12.0, 1.0) * 6.25), (12, 60.0, np.linspace(0.0, 40.0, 13)),
              (32, 1000.0, np.arange(20.0, 600.0, 31.25))]
    for i, (N, box, s_edges) in enumerate(xcases):
        s_edges = np.asarray(s_edges, F32)
        delta = rng.standard_normal((N, N, N)).astype(F32)
        r3d, xi, nm = corr.xi_vec(delta, box, s_edges)
        out[f"xi_{i}_delta"] = delta
        out[f"xi_{i}_box"] = np.array([box], dtype=np.float64)
        out[f"xi_{i}_sedges"] = s_edges
        out[f"xi_{i}_r"] = np.asarray(r3d, F32)
        out[f"xi_{i}_xi"] = np.asarray(xi, F32)
        out[f"xi_{i}_nmodes"] = np.asarray(nm, F32)
        kf = 2 * np.pi / box
        k_edges = np.arange(kf, np.pi * N / box, kf).astype(F32)
        k3d, pk, nmk, r3d2, xi2 = corr.compute_2pt_correlations(delta, box, s_edges, k_edges)
        out[f"tpc_{i}_kedges"] = k_edges
        out[f"tpc_{i}_k"] = np.asarray(k3d, F32)
        out[f"tpc_{i}_pk"] = np.asarray(pk, F32)
        out[f"tpc_{i}_nmodes"] = np.asarray(nmk, F32)
        out[f"tpc_{i}_r"] = np.asarray(r3d2, F32)
        out[f"tpc_{i}_xi"] = np.asarray(xi2, F32)
    out["xi_ncases"] = np.array([len(xcases)])

    # ---- bispec (src/correlations.py:334-462) on lognormal contrasts (a non-zero bispectrum)
    bcases = [(16, 100.0, 0.15, 0.25, 6), (32, 1000.0, 0.05, 0.03, 9), (24, 300.0, 0.1, 0.1, 7)]
    for i, (N, box, k1, k2, nt) in enumerate(bcases):
        g = rng.standard_normal((N, N, N))
        d = np.exp(0.8 * g)
        delta = (d / d.mean() - 1.0).astype(F32)
        theta = np.linspace(0.0, np.pi, nt).astype(F32)
        k_all, pk, th, bk, qk = corr.bispec(delta, box, k1, k2, theta)
        out[f"bk_{i}_delta"] = delta
        out[f"bk_{i}_args"] = np.array([box, k1, k2], dtype=np.float64)
        out[f"bk_{i}_theta"] = theta
        out[f"bk_{i}_k"] = np.asarray(k_all, F32)
        out[f"bk_{i}_pk"] = np.asarray(pk, F32)
        out[f"bk_{i}_b"] = np.asarray(bk, F32)
        out[f"bk_{i}_q"] = np.asarray(qk, F32)
    out["bk_ncases"] = np.array([len(bcases)])

    # ---- compute_all_correlations (src/correlations.py:464-637) on the bispectrum cases' contrasts
    for i, (N, box, k1, k2, nt) in enumerate(bcases):
        delta, theta = out[f"bk_{i}_delta"], out[f"bk_{i}_theta"]
        kf = 2 * np.pi / box
        k_edges = np.arange(kf, np.pi * N / box, kf).astype(F32)
        s_edges = np.linspace(0.0, 0.5 * box, 9).astype(F32)
        res = corr.compute_all_correlations(delta, box, s_edges, k_edges, k1, k2, theta)
        out[f"all_{i}_kedges"] = k_edges
        out[f"all_{i}_sedges"] = s_edges
        for name, v in zip(("k", "pk", "nmk", "r", "xi", "nmx", "kall", "pkb", "theta", "b", "q"), res):
            out[f"all_{i}_{name}"] = np.asarray(v, F32)
    out["all_ncases"] = np.array([len(bcases)])

    path = os.path.join(HERE, "reference_outputs.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KiB, {len(out)} arrays)")


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("JAX_POWSPEC_ROOT")
    if not root:
        sys.exit("usage: python make_golden.py <path to a jax-powspec checkout>  (or set JAX_POWSPEC_ROOT)")
    main(root)
