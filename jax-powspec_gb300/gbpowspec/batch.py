"""Batched P_l(k): many mocks through resident lanes (no reference counterpart).

The reference computes one mock per call.  Covariance work needs hundreds of
mocks with uneven particle counts and several mesh sizes, so this module
runs them as a batch:

* ``ParticleArena`` packs every mock's particles back to back in one device
  buffer (SoA x | y | z [| w]) with per-mock offsets; one host-to-device copy
  uploads the whole batch.
* A job table (one ``gbp_job`` per mock, in device memory) points each mock
  at its slice of the arena and carries its box.
* ``BatchRunner`` holds ``n_lanes`` lanes of one shape class (mesh, MAS,
  interlacing, multipoles, k bins).  Each lane keeps its meshes, spectra and
  workspaces resident and replays one captured CUDA graph per mock; the
  lanes run on their own streams so one mock's deposit overlaps another's
  FFT and binning.  ``gbp_batch_run`` (C ABI) does the scheduling.
* ``run_mixed`` runs several classes (e.g. 256^3 and 128^3 halves of a
  covariance set) concurrently; ``covariance`` forms the sample covariance.

Bins are given in units of the fundamental frequency kF = 2 pi / L, so mocks
with different boxes share a class.  ``shell_edges(N)`` is the default
binning (kF .. kNyq in steps of kF) with exact integer edges: the same for
every box, whereas float32 edges in h/Mpc divided by a float32 kF land a
little above or below the integers depending on L, which moves the modes
whose |k| is exactly an integer (|k|^2 a perfect square) between bins.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib, _native
from ._lib import check

__all__ = ["shell_edges", "ParticleArena", "BatchRunner", "BatchResult", "run_mixed", "covariance",
           "tune_lanes"]

_ELL_BITS = {0: _lib.ELL0, 2: _lib.ELL2, 4: _lib.ELL4}


def shell_edges(n_mesh: int) -> np.ndarray:
    """k edges 1, 2, ..., N/2 - 1 in units of kF (float32, exact integers)."""
    return np.arange(1, n_mesh // 2, dtype=np.float32)


def _ells_mask(ells, kmean: bool) -> int:
    m = 0
    for l in ells:
        m |= _ELL_BITS[int(l)]
    return m | (_lib.KSUM if kmean else 0)


class ParticleArena:
    """Catalogues packed back to back: host pinned staging + one device buffer.

    ``catalogues`` is a sequence of (x, y, z) or (x, y, z, w) float arrays
    (numpy or CPU tensors).  ``upload()`` enqueues one host-to-device copy on
    the current stream; ``job_table()`` builds the per-mock job descriptors.
    """

    def __init__(self, catalogues, device=None, weighted: bool | None = None):
        if not torch.cuda.is_available():
            raise RuntimeError("gbpowspec needs a CUDA device; there is no CPU fallback")
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        cats = list(catalogues)
        if weighted is None:
            weighted = any(len(c) > 3 and c[3] is not None for c in cats)
        self.weighted = bool(weighted)
        self.counts = np.array([len(c[0]) for c in cats], dtype=np.int64)
        self.offsets = np.zeros(len(cats) + 1, dtype=np.int64)
        np.cumsum(self.counts, out=self.offsets[1:])
        total = int(self.offsets[-1])
        ncol = 4 if self.weighted else 3
        self.host = torch.empty((ncol, max(total, 1)), dtype=torch.float32, pin_memory=True)
        hv = self.host.numpy()
        for i, c in enumerate(cats):
            a, b = self.offsets[i], self.offsets[i + 1]
            for k in range(3):
                hv[k, a:b] = np.asarray(c[k], dtype=np.float32).reshape(-1)
            if self.weighted:
                hv[3, a:b] = 1.0 if len(c) < 4 or c[3] is None else np.asarray(c[3], np.float32).reshape(-1)
        self.dev = torch.empty_like(self.host, device=self.device)

    @classmethod
    def empty(cls, counts, device=None, weighted: bool = False) -> "ParticleArena":
        """A device-only arena for mocks of the given sizes (filled on the device, e.g. by the
        lognormal generator through views(i)); upload() is not available."""
        self = cls.__new__(cls)
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self.weighted = bool(weighted)
        self.counts = np.asarray(counts, dtype=np.int64)
        self.offsets = np.zeros(len(self.counts) + 1, dtype=np.int64)
        np.cumsum(self.counts, out=self.offsets[1:])
        self.host = None
        self.dev = torch.empty((4 if weighted else 3, max(int(self.offsets[-1]), 1)), dtype=torch.float32,
                               device=self.device)
        return self

    def views(self, i: int) -> tuple:
        """Device views (x, y, z[, w]) of mock i."""
        a, b = int(self.offsets[i]), int(self.offsets[i + 1])
        return tuple(self.dev[k, a:b] for k in range(self.dev.shape[0]))

    def __len__(self) -> int:
        return len(self.counts)

    @property
    def nbytes(self) -> int:
        return self.dev.numel() * 4

    def upload(self) -> int:
        """Enqueue the host-to-device copy of every mock; returns the bytes copied."""
        if self.host is None:
            raise RuntimeError("this arena lives on the device only")
        self.dev.copy_(self.host, non_blocking=True)
        return self.nbytes

    def upload_range(self, first: int, last: int) -> int:
        """Enqueue the host-to-device copy of mocks first .. last-1 on the current stream (one copy per
        particle column: the mocks are packed back to back); returns the bytes copied."""
        if self.host is None:
            raise RuntimeError("this arena lives on the device only")
        a, b = int(self.offsets[first]), int(self.offsets[last])
        for k in range(self.dev.shape[0]):
            self.dev[k, a:b].copy_(self.host[k, a:b], non_blocking=True)
        return (b - a) * 4 * self.dev.shape[0]

    def job_table(self, boxes, n_mesh: int, indices=None, origins=None) -> torch.Tensor:
        """Device table of gbp_job for mocks `indices` (default all) on an n_mesh grid.

        boxes: one box size per selected mock (or a scalar); origins: (B, 3) or None.
        """
        idx = np.arange(len(self)) if indices is None else np.asarray(indices, dtype=np.int64)
        boxes = np.broadcast_to(np.asarray(boxes, dtype=np.float64), idx.shape)
        org = np.zeros((idx.size, 3)) if origins is None else np.broadcast_to(np.asarray(origins, np.float64),
                                                                               (idx.size, 3))
        arr = (_lib.Job * max(idx.size, 1))()
        base = self.dev.data_ptr()
        stride = self.dev.shape[1] * 4
        for j, i in enumerate(idx):
            off = int(self.offsets[i]) * 4
            jb = arr[j]
            jb.x, jb.y, jb.z = base + off, base + stride + off, base + 2 * stride + off
            jb.w = base + 3 * stride + off if self.weighted else None
            jb.n = int(self.counts[i])
            jb.inv_cell = float(np.float32(n_mesh / float(boxes[j])))     # as PowerSpectrum
            jb.xmin, jb.ymin, jb.zmin = (float(np.float32(v)) for v in org[j])
            jb.box_size = float(boxes[j])
        raw = np.frombuffer(bytes(arr), dtype=np.uint8).reshape(-1, _lib.JOB_BYTES)[: idx.size]
        host = torch.from_numpy(raw.copy()).pin_memory()
        return host.to(self.device, non_blocking=True)


@dataclass
class BatchResult:
    pk: torch.Tensor           # float64 [B, nb, 3]: P_0, P_2, P_4 (unrequested multipoles are 0)
    kmean: torch.Tensor | None  # float64 [B, nb] mode-averaged |k| (h/Mpc)
    nmodes: torch.Tensor       # int64 [B, nb]
    stats: torch.Tensor        # uint8 [B, sizeof(gbp_deposit_stats)]
    kedges_grid: np.ndarray    # float32 [nb + 1] in units of kF

    def deposit_stats(self) -> list:
        raw = self.stats.cpu().numpy()
        return [_lib.DepositStats.from_buffer_copy(raw[i].tobytes()) for i in range(raw.shape[0])]


class BatchRunner:
    """Lanes of one shape class; ``run`` processes a job table through them."""

    def __init__(self, n_mesh: int, *, capacity: int, mas: str = "cic", interlace: bool = True,
                 ells=(0, 2), kedges_grid=None, shot_noise: bool = True, kmean: bool = True,
                 n_lanes: int = 2, graphs: bool = True, device=None, tiles="auto"):
        if not torch.cuda.is_available():
            raise RuntimeError("gbpowspec needs a CUDA device; there is no CPU fallback")
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self.n_mesh, self.capacity = int(n_mesh), int(capacity)
        self.mas, self.interlace, self.ells = mas.lower(), bool(interlace), tuple(int(l) for l in ells)
        self.shot_noise, self.kmean = bool(shot_noise), bool(kmean)
        edges = shell_edges(self.n_mesh) if kedges_grid is None else np.asarray(kedges_grid, dtype=np.float32)
        self.kedges_grid = edges
        self.bins = _native.bins_for(edges, self.n_mesh, self.device)
        self.nb = self.bins.n_bins
        self.mask = _ells_mask(self.ells, self.kmean)
        lib = _lib.load()
        # column tile of the lanes' fused calls: "auto" = the autotuner's choice for this shape (tune.py),
        # None = the library default, or (tx, ty); the results are the same bits whatever the choice
        if tiles == "auto":
            from .tune import default_tuner
            tiles = default_tuner().best(self.n_mesh, self.mas, self.interlace, n=self.capacity,
                                         device=self.device) if _native.tile_variants(self.n_mesh) else None
        self.tiles = None if tiles is None else (int(tiles[0]), int(tiles[1]))
        flags = (_lib.LANE_GRAPH if graphs else 0) | (0 if self.tiles is None else _lib.lane_tiles_flag(*self.tiles))
        self._lanes = []
        with torch.cuda.device(self.device):
            for _ in range(int(n_lanes)):
                h = C.c_void_p()
                check(lib.gbp_lane_create(self.n_mesh, _lib.MAS[self.mas], int(self.interlace), self.mask,
                                          int(self.shot_noise), self.bins.handle, self.capacity, flags, C.byref(h)),
                      "gbp_lane_create")
                self._lanes.append(h)
        self._lane_arr = (C.c_void_p * len(self._lanes))(*[h.value for h in self._lanes])
        b = C.c_size_t(0)
        g = C.c_int(0)
        check(lib.gbp_lane_info(self._lanes[0], C.byref(b), None, C.byref(g)), "gbp_lane_info")
        self.lane_bytes, self.graphs = b.value, bool(g.value)

    @staticmethod
    def bytes_per_lane(n_mesh: int, *, capacity: int, mas: str = "cic", interlace: bool = True, ells=(0, 2),
                       kedges_grid=None, kmean: bool = True, device=None) -> int:
        dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        edges = shell_edges(n_mesh) if kedges_grid is None else np.asarray(kedges_grid, dtype=np.float32)
        bins = _native.bins_for(edges, int(n_mesh), dev)
        out = C.c_size_t(0)
        with torch.cuda.device(dev):
            check(_lib.load().gbp_lane_bytes(int(n_mesh), _lib.MAS[mas.lower()], int(interlace),
                                             _ells_mask(ells, kmean), bins.handle, int(capacity), C.byref(out)),
                  "gbp_lane_bytes")
        return out.value

    @property
    def n_lanes(self) -> int:
        return len(self._lanes)

    @property
    def device_bytes(self) -> int:
        return self.lane_bytes * len(self._lanes)

    def alloc_result(self, n_jobs: int) -> BatchResult:
        dev, nb = self.device, self.nb
        return BatchResult(pk=torch.zeros((n_jobs, nb, 3), dtype=torch.float64, device=dev),
                           kmean=torch.zeros((n_jobs, nb), dtype=torch.float64, device=dev) if self.kmean else None,
                           nmodes=torch.zeros((n_jobs, nb), dtype=torch.int64, device=dev),
                           stats=torch.zeros((n_jobs, _lib.STATS_BYTES), dtype=torch.uint8, device=dev),
                           kedges_grid=self.kedges_grid)

    def _out(self, res: BatchResult) -> _lib.LaneOut:
        return _lib.LaneOut(res.pk.data_ptr(), None if res.kmean is None else res.kmean.data_ptr(),
                            res.nmodes.data_ptr(), res.stats.data_ptr())

    def run(self, jobs: torch.Tensor, out: BatchResult | None = None, n_lanes: int | None = None) -> BatchResult:
        """Enqueue every job of the table on the current stream (lanes fork and join); no host sync."""
        n = int(jobs.shape[0])
        if jobs.dtype != torch.uint8 or jobs.device != self.device or tuple(jobs.shape[1:]) != (_lib.JOB_BYTES,):
            raise ValueError("jobs must be a device uint8 tensor [B, sizeof(gbp_job)] (ParticleArena.job_table)")
        res = self.alloc_result(n) if out is None else out
        if res.pk.shape[0] < n:
            raise ValueError("result arrays hold fewer jobs than the table")
        lanes = self.n_lanes if n_lanes is None else max(1, min(int(n_lanes), self.n_lanes))
        o = self._out(res)
        check(_lib.load().gbp_batch_run(C.cast(self._lane_arr, C.c_void_p), lanes, C.c_void_p(jobs.data_ptr()), n,
                                        C.byref(o), _native._stream_of(self.device)), "gbp_batch_run")
        return res

    def _run_rows(self, jobs: torch.Tensor, first: int, last: int, res: BatchResult, lanes: int):
        """gbp_batch_run over job rows first .. last-1, results into the same rows of `res`."""
        nb = self.nb
        o = _lib.LaneOut(res.pk.data_ptr() + first * nb * 3 * 8,
                         None if res.kmean is None else res.kmean.data_ptr() + first * nb * 8,
                         res.nmodes.data_ptr() + first * nb * 8, res.stats.data_ptr() + first * _lib.STATS_BYTES)
        check(_lib.load().gbp_batch_run(C.cast(self._lane_arr, C.c_void_p), lanes,
                                        C.c_void_p(jobs.data_ptr() + first * _lib.JOB_BYTES), last - first,
                                        C.byref(o), _native._stream_of(self.device)), "gbp_batch_run")

    def run_from_host(self, arena: "ParticleArena", jobs: torch.Tensor, out: BatchResult | None = None,
                      chunk: int | None = None) -> BatchResult:
        """Upload the arena's catalogues and process them, the copies overlapping the work: chunk c of
        mocks is copied on a copy stream while the lanes process chunk c - 1 (default chunk: the lane
        count).  Job row j must describe arena mock j (ParticleArena.job_table with the default indices).
        Same results as ``arena.upload(); run(jobs)``; no host sync."""
        n = int(jobs.shape[0])
        if n != len(arena):
            raise ValueError("run_from_host needs one job row per arena mock, in arena order")
        if jobs.dtype != torch.uint8 or jobs.device != self.device or tuple(jobs.shape[1:]) != (_lib.JOB_BYTES,):
            raise ValueError("jobs must be a device uint8 tensor [B, sizeof(gbp_job)] (ParticleArena.job_table)")
        res = self.alloc_result(n) if out is None else out
        if res.pk.shape[0] < n:
            raise ValueError("result arrays hold fewer jobs than the table")
        step = max(1, self.n_lanes if chunk is None else int(chunk))
        cur = torch.cuda.current_stream(self.device)
        if getattr(self, "_copy_stream", None) is None:
            self._copy_stream = torch.cuda.Stream(self.device)
        copy = self._copy_stream
        copy.wait_stream(cur)            # earlier work that reads the arena's device buffer comes first
        ready = []
        with torch.cuda.stream(copy):
            for a in range(0, n, step):
                arena.upload_range(a, min(n, a + step))
                ev = torch.cuda.Event()
                ev.record(copy)
                ready.append(ev)
        for ev, a in zip(ready, range(0, n, step)):
            cur.wait_event(ev)
            self._run_rows(jobs, a, min(n, a + step), res, self.n_lanes)
        return res

    def run_one(self, jobs: torch.Tensor, index: int, out: BatchResult, lane: int = 0) -> BatchResult:
        """Process job `index` of the table on one lane, on the current stream (serving)."""
        o = self._out(out)
        check(_lib.load().gbp_lane_run(self._lanes[lane], C.c_void_p(jobs.data_ptr()), int(jobs.shape[0]),
                                       int(index), int(jobs.shape[0]) + 1, C.byref(o),
                                       _native._stream_of(self.device)), "gbp_lane_run")
        return out

    def close(self):
        lib = _lib.load()
        for h in self._lanes:
            if h:
                lib.gbp_lane_destroy(h)
        self._lanes = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_mixed(work) -> list:
    """Run several (runner, jobs) pairs concurrently: each on a stream forked from the current one.

    Returns the BatchResults in order; the current stream waits for all of them.
    """
    cur = torch.cuda.current_stream()
    results = []
    streams = []
    for runner, jobs in work:
        s = torch.cuda.Stream(device=runner.device)
        s.wait_stream(cur)
        with torch.cuda.stream(s):
            results.append(runner.run(jobs))
        streams.append(s)
    for s in streams:
        cur.wait_stream(s)
    return results


def covariance(pk: np.ndarray, ells_index=(0, 1)) -> tuple[np.ndarray, np.ndarray]:
    """Mean and unbiased sample covariance of the data vector [P_l0(k) ..., P_l1(k) ...] over mocks.

    pk: [B, nb, 3] float64 (host).  Bins with NaN in any mock are dropped.
    """
    pk = np.asarray(pk, dtype=np.float64)
    if pk.shape[0] < 2:
        raise ValueError("a covariance needs at least two mocks")
    d = np.concatenate([pk[:, :, l] for l in ells_index], axis=1)
    keep = np.all(np.isfinite(d), axis=0)
    d = d[:, keep]
    mean = d.mean(axis=0)
    r = d - mean
    cov = r.T @ r / (d.shape[0] - 1)
    return mean, cov


def tune_lanes(n_mesh: int, jobs: torch.Tensor, *, capacity: int, candidates=(1, 2, 3, 4), repeats: int = 2,
               **kw) -> tuple[int, dict]:
    """Pick the lane count with the highest mocks/s on a sample job table (CUDA-event timing).

    Returns (best, {lanes: mocks/s}).  Lanes cost memory; candidates whose
    lanes do not fit in free device memory are skipped.
    """
    dev = jobs.device
    per = BatchRunner.bytes_per_lane(n_mesh, capacity=capacity, device=dev, **{k: v for k, v in kw.items()
                                                                               if k in ("mas", "interlace", "ells",
                                                                                        "kedges_grid", "kmean")})
    free, _ = torch.cuda.mem_get_info(dev)
    cand = [c for c in candidates if c * per < 0.8 * free]
    if not cand:
        raise MemoryError("not even one lane fits in free device memory")
    runner = BatchRunner(n_mesh, capacity=capacity, n_lanes=max(cand), device=dev, **kw)
    res = runner.alloc_result(int(jobs.shape[0]))
    rates = {}
    stream = torch.cuda.current_stream(dev)
    for c in cand:
        runner.run(jobs, res, n_lanes=c)                # warm
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(repeats):
            runner.run(jobs, res, n_lanes=c)
        e1.record(stream)
        e1.synchronize()
        rates[c] = repeats * int(jobs.shape[0]) / (e0.elapsed_time(e1) / 1e3)
    runner.close()
    best = max(rates, key=rates.get)
    return best, rates
