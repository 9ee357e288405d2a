"""Programmatic dependent launch changes timing only.

Every kernel of the fused pipeline, the lanes and the normalisation is
launched with the programmatic-serialisation attribute and waits for its
predecessor (griddepcontrol.wait) before touching memory.  GBP_PDL=0 turns
the attribute off; a subprocess computes the same spectra that way, through
PowerSpectrum and through graph-replaying batch lanes, and they must equal
this process's bit for bit.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import sys, numpy as np, torch
sys.path.insert(0, sys.argv[1]); sys.path.insert(0, sys.argv[1] + "/jax-powspec_gb300")
from gbpowspec import PkConfig, PowerSpectrum
from gbpowspec.batch import BatchRunner, ParticleArena
from gbpowspec.synth import lognormal_catalogue
out = {}
for N, n, mas in ((64, 50_000, "tsc"), (128, 300_000, "pcs")):
    cats = [lognormal_catalogue(n, 700.0, grid=32, seed=s) for s in (1, 2, 3)]
    cfg = PkConfig(n_mesh=N, box_size=700.0, mas=mas, interlace=True, ells=(0, 2, 4))
    x, y, z = (torch.from_numpy(a).cuda() for a in cats[0])
    out[f"plain{N}"] = PowerSpectrum(cfg).run(x, y, z).pk.cpu().numpy()
    arena = ParticleArena(cats)
    arena.upload()
    runner = BatchRunner(N, capacity=n, mas=mas, interlace=True, ells=(0, 2, 4), kedges_grid=cfg.kedges_grid(),
                         n_lanes=2)
    out[f"batch{N}"] = runner.run(arena.job_table(700.0, N)).pk.cpu().numpy()
    runner.close()
np.savez(sys.argv[2], **out)
"""


def _run(tmp_path, pdl):
    path = str(tmp_path / f"pk_pdl{pdl}.npz")
    env = dict(os.environ, GBP_PDL=str(pdl))
    r = subprocess.run([sys.executable, "-c", SCRIPT, ROOT, path], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return np.load(path)


def test_ordinary_launches_give_the_same_bits(tmp_path):
    on, off = _run(tmp_path, 1), _run(tmp_path, 0)
    assert sorted(on.files) == sorted(off.files)
    for k in on.files:
        a, b = on[k], off[k]
        assert a.shape == b.shape
        assert np.array_equal(np.nan_to_num(a, nan=-7.0), np.nan_to_num(b, nan=-7.0)), k
