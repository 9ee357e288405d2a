"""Job-mode entry points (a mock described in device memory).

gbp_deposit_job must give the same mesh and statistics, bit for bit, as
gbp_deposit on the same particles, whatever the capacity the launches were
sized for; gbp_power_normalize_job must match gbp_power_normalize.  The same
workspace and launch sizes serve mocks of different sizes and boxes, which is
what lets one captured launch sequence serve every mock of a batch.
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _job_tensor(x, y, z, w, n, box, N, origin=(0.0, 0.0, 0.0)):
    from gbpowspec import _lib
    j = _lib.Job()
    j.x, j.y, j.z = x.data_ptr(), y.data_ptr(), z.data_ptr()
    j.w = None if w is None else w.data_ptr()
    j.n = n
    j.inv_cell = float(np.float32(N / box))
    j.xmin, j.ymin, j.zmin = (float(np.float32(o)) for o in origin)
    j.box_size = float(box)
    raw = np.frombuffer(bytes(j), dtype=np.uint8)
    return torch.from_numpy(raw.copy()).cuda()


@pytest.mark.parametrize("mas,interlace", [("cic", True), ("tsc", True), ("pcs", False), ("ngp", False)])
def test_deposit_job_matches_deposit(mas, interlace):
    from gbpowspec import _lib, _native
    from gbpowspec.synth import lognormal_catalogue
    lib = _lib.load()
    N, cap = 64, 120_000
    G = 2 if interlace else 1
    dev = torch.device("cuda", 0)
    ws = _native.workspace(_native.deposit_workspace_size(cap, N, _lib.MAS[mas], interlace, 0), dev)
    for n, box, seed in ((100_000, 500.0, 3), (37_123, 800.0, 4), (cap, 650.0, 5)):
        x, y, z = (torch.from_numpy(a).cuda() for a in lognormal_catalogue(n, box, grid=32, seed=seed))
        w = torch.from_numpy(np.random.default_rng(seed).uniform(0.5, 1.5, n).astype(np.float32)).cuda()
        want, want_stats = _native.deposit(x, y, z, w, n_mesh=N, inv_cell=np.float32(N / box),
                                           mas=_lib.MAS[mas], interlace=interlace)
        job = _job_tensor(x, y, z, w, n, box, N)
        mesh = torch.full((G, N, N, N), float("nan"), device=dev)
        stats = torch.zeros(_lib.STATS_BYTES, dtype=torch.uint8, device=dev)
        st = lib.gbp_deposit_job(C.c_void_p(job.data_ptr()), cap, N, _lib.MAS[mas], int(interlace),
                                 C.c_void_p(mesh.data_ptr()), C.c_void_p(stats.data_ptr()),
                                 C.c_void_p(ws.data_ptr()), ws.numel(),
                                 C.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert st == 0, _lib.strerror(st)
        torch.cuda.synchronize()
        assert torch.equal(mesh, want)
        R = _lib.STATS_RESULT_BYTES
        assert bytes(_native.read_stats(stats))[:R] == bytes(_native.read_stats(want_stats))[:R]


def test_deposit_job_clamps_to_capacity():
    """A job claiming more particles than the capacity deposits only the first `capacity`."""
    from gbpowspec import _lib, _native
    lib = _lib.load()
    N, cap, n = 32, 5_000, 9_000
    dev = torch.device("cuda", 0)
    g = torch.Generator().manual_seed(7)
    x, y, z = (torch.rand(n, generator=g) * 100.0 for _ in range(3))
    x, y, z = x.cuda(), y.cuda(), z.cuda()
    ws = _native.workspace(_native.deposit_workspace_size(cap, N, 2, False, 0), dev)
    job = _job_tensor(x, y, z, None, n, 100.0, N)
    mesh = torch.empty((1, N, N, N), device=dev)
    stats = torch.zeros(_lib.STATS_BYTES, dtype=torch.uint8, device=dev)
    st = lib.gbp_deposit_job(C.c_void_p(job.data_ptr()), cap, N, 2, 0, C.c_void_p(mesh.data_ptr()),
                             C.c_void_p(stats.data_ptr()), C.c_void_p(ws.data_ptr()), ws.numel(),
                             C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0
    want, _ = _native.deposit(x[:cap].contiguous(), y[:cap].contiguous(), z[:cap].contiguous(), None,
                              n_mesh=N, inv_cell=np.float32(N / 100.0), mas=2)
    torch.cuda.synchronize()
    assert torch.equal(mesh, want)
    assert _native.read_stats(stats).n_kept == cap


def test_normalize_job_matches_normalize():
    from gbpowspec import PkConfig, PowerSpectrum, _lib, _native
    from gbpowspec.synth import lognormal_catalogue
    lib = _lib.load()
    box, N = 700.0, 64
    x, y, z = (torch.from_numpy(a).cuda() for a in lognormal_catalogue(50_000, box, grid=32, seed=9))
    ps = PowerSpectrum(PkConfig(n_mesh=N, box_size=box, mas="tsc", interlace=True))
    res = ps.run(x, y, z)
    job = _job_tensor(x, y, z, None, x.numel(), box, N)
    nb = ps.bins.n_bins
    pk = torch.empty((nb, 3), dtype=torch.float64, device=x.device)
    km = torch.empty(nb, dtype=torch.float64, device=x.device)
    st = lib.gbp_power_normalize_job(C.c_void_p(ps.sums.sums.data_ptr()), C.c_void_p(ps.sums.nmodes.data_ptr()),
                                     C.c_void_p(ps.sums.ksum.data_ptr()), nb, N, C.c_void_p(job.data_ptr()),
                                     C.c_void_p(ps.stats.data_ptr()), C.c_void_p(ps.stats.data_ptr()), 1,
                                     C.c_void_p(pk.data_ptr()), C.c_void_p(km.data_ptr()),
                                     C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0
    torch.cuda.synchronize()
    assert torch.equal(torch.nan_to_num(pk, nan=-1.0), torch.nan_to_num(res.pk, nan=-1.0))
    assert torch.equal(torch.nan_to_num(km, nan=-1.0), torch.nan_to_num(res.k_mean, nan=-1.0))
