"""Serving: a continuous-batching P_l(k) request loop on one GPU (no reference counterpart).

Requests of different mesh sizes, schemes and particle counts arrive while
others run.  The server keeps, per shape class (mesh, MAS, interlacing,
multipoles, k bins), a set of resident lanes (gbp_lane: meshes, spectra,
workspaces, a captured CUDA graph), each with its own stream, particle
buffer and output buffers.  A request is admitted as soon as a lane of its
class is free; a new lane is created only while the lanes' device memory
stays within the HBM budget.  Admitted requests overlap on the device: each
runs on its lane's stream (copy particles in, write the job, replay the
lane's graph, copy P_l out), and the loop polls their completion events.

    srv = Server(budget_bytes=80e9)
    t = srv.submit(Request(x, y, z, box=1000.0, n_mesh=256, mas="cic"))
    for res in srv.drain(): ...          # Result(ticket, pk, k, nmodes, latency)

Failure handling: a request that cannot be served (too many particles for
any lane, a class whose single lane does not fit in the budget, a failing
library call) is returned as a Result with `error` set; it is not retried.
A deadline bounds drain(); requests still in flight then are reported as
timed out (their lanes stay busy until the device finishes them).

The scheduling logic is separate from the device work (`backend`), so it is
exercised on the CPU with a fake backend in the tests.
"""
from __future__ import annotations

import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

__all__ = ["Request", "Result", "Server", "percentiles", "stream_priority"]


@dataclass
class Request:
    """One P_l(k) request.  x, y, z (and w) are host arrays, ideally pinned CPU tensors."""
    x: object
    y: object
    z: object
    box: float
    n_mesh: int
    mas: str = "cic"
    interlace: bool = True
    ells: tuple = (0, 2, 4)
    w: object = None
    origin: tuple = (0.0, 0.0, 0.0)
    ticket: int = -1
    arrival: float = 0.0          # time.perf_counter() when it arrived (set by submit)

    @property
    def n(self) -> int:
        return int(len(self.x))

    def key(self) -> tuple:
        return (int(self.n_mesh), self.mas.lower(), bool(self.interlace), tuple(int(l) for l in self.ells),
                self.w is not None)


@dataclass
class Result:
    ticket: int
    pk: np.ndarray | None = None        # [nb, 3] P_0, P_2, P_4 (h^-3 Mpc^3)
    k: np.ndarray | None = None         # [nb] mode-averaged |k| (h/Mpc)
    nmodes: np.ndarray | None = None    # [nb]
    n_kept: int = 0
    latency: float = 0.0                # seconds from arrival to result on the host
    error: str | None = None


def percentiles(latencies, qs=(50, 99)) -> dict:
    a = np.asarray(latencies, dtype=np.float64)
    if a.size == 0:
        return {f"p{q}": None for q in qs}
    return {f"p{q}": float(np.percentile(a, q)) for q in qs}


@dataclass
class _Slot:
    """One lane of a class as the scheduler sees it."""
    lane: object
    bytes: int
    busy: object = None           # the Request in flight
    started: float = 0.0


@dataclass
class _Class:
    key: tuple
    slots: list = field(default_factory=list)
    failed: str | None = None     # set when even one lane cannot be created


class Server:
    """Continuous-batching request loop (see the module docstring)."""

    def __init__(self, budget_bytes: float = 80e9, lanes_per_class: int = 4, capacity: int = 10_000_000,
                 backend=None, device=None, clock=time.perf_counter):
        self.budget = int(budget_bytes)
        self.lanes_per_class = int(lanes_per_class)
        self.capacity = int(capacity)
        self.backend = backend if backend is not None else GpuBackend(device)
        self.clock = clock
        self.queue: deque = deque()
        self.classes: dict = {}
        self.used = 0
        self._next = 0
        self.done: list = []

    # ---- public API
    def submit(self, req: Request) -> int:
        req.ticket = self._next
        self._next += 1
        req.arrival = self.clock()
        if req.n > self.capacity:
            self.done.append(Result(req.ticket, error=f"{req.n} particles exceed the lane capacity "
                                                       f"{self.capacity}", latency=0.0))
            return req.ticket
        self.queue.append(req)
        self._admit()
        return req.ticket

    def poll(self) -> list:
        """Collect finished requests, admit waiting ones; returns the Results finished since the last call."""
        for cls in self.classes.values():
            for slot in cls.slots:
                if slot.busy is not None and self.backend.finished(slot.lane):
                    req = slot.busy
                    res = self.backend.result(slot.lane, req)
                    res.latency = self.clock() - req.arrival
                    self.done.append(res)
                    slot.busy = None
        self._admit()
        out, self.done = self.done, []
        return out

    def drain(self, timeout: float = 600.0, sleep: float = 0.0) -> list:
        """Poll until every submitted request has a Result (or the deadline passes)."""
        deadline = self.clock() + timeout
        results = []
        while True:
            results.extend(self.poll())
            if not self.queue and not self.in_flight():
                return results
            if self.clock() > deadline:
                for cls in self.classes.values():
                    for slot in cls.slots:
                        if slot.busy is not None:
                            results.append(Result(slot.busy.ticket, error="timed out", latency=timeout))
                while self.queue:
                    results.append(Result(self.queue.popleft().ticket, error="timed out", latency=timeout))
                return results
            if sleep:
                time.sleep(sleep)

    def in_flight(self) -> int:
        return sum(1 for c in self.classes.values() for s in c.slots if s.busy is not None)

    def close(self):
        for cls in self.classes.values():
            for slot in cls.slots:
                self.backend.destroy(slot.lane)
            cls.slots = []
        self.used = 0

    # ---- scheduling
    def _admit(self):
        """Start every queued request that has (or may get) a free lane of its class, in arrival order
        within a class; a request whose class is saturated does not block other classes."""
        waiting = deque()
        while self.queue:
            req = self.queue.popleft()
            key = req.key()
            cls = self.classes.get(key)
            if cls is None:
                cls = self.classes[key] = _Class(key)
            if cls.failed:
                self.done.append(Result(req.ticket, error=cls.failed, latency=self.clock() - req.arrival))
                continue
            slot = next((s for s in cls.slots if s.busy is None), None)
            if slot is None and len(cls.slots) < self.lanes_per_class:
                slot = self._grow(cls, req)
            if slot is None:
                waiting.append(req)
                continue
            try:
                self.backend.start(slot.lane, req)
            except Exception as e:        # a failing call: report, do not retry
                self.done.append(Result(req.ticket, error=f"start failed: {e}", latency=self.clock() - req.arrival))
                continue
            slot.busy = req
            slot.started = self.clock()
        self.queue = waiting

    def _grow(self, cls: _Class, req: Request):
        need = self.backend.lane_bytes(req, self.capacity)
        if need > self.budget:
            cls.failed = f"one lane of this class needs {need} bytes, over the budget of {self.budget}"
            return None
        if self.used + need > self.budget:
            self._evict(need, keep=cls)
        if self.used + need > self.budget:
            return None                           # wait for lanes to finish
        try:
            lane = self.backend.create(req, self.capacity)
        except Exception as e:                    # e.g. the device is out of memory: refuse, do not retry
            cls.failed = f"lane creation failed: {e}"
            return None
        # the lane may hold a little more or less than the estimate (its tuned tile shape sizes the
        # particle buckets): account what it holds
        need = int(getattr(self.backend, "lane_bytes_of", lambda _lane: need)(lane))
        self.used += need
        slot = _Slot(lane, need)
        cls.slots.append(slot)
        return slot

    def _evict(self, need: int, keep: _Class):
        """Free idle lanes of other classes (least recently started first) until `need` bytes fit."""
        idle = [(s.started, c, s) for c in self.classes.values() if c is not keep for s in c.slots if s.busy is None]
        for _, c, s in sorted(idle, key=lambda t: t[0]):
            if self.used + need <= self.budget:
                break
            self.backend.destroy(s.lane)
            c.slots.remove(s)
            self.used -= s.bytes


def stream_priority(n_mesh: int) -> int:
    """CUDA stream priority of a lane (lower is more urgent): small meshes first.

    A 128^3 request takes a fraction of a millisecond on the device and a
    512^3 one a few milliseconds; at equal priority the small request's
    kernels wait behind whole waves of the large one's blocks.  With a higher
    priority the block scheduler starts the small request's blocks as soon as
    any of the large one's retire, so short requests keep short latencies in
    a mixed stream.  (Lanes replay CUDA graphs; graph kernels take the
    priority of the stream they are launched into.)"""
    if n_mesh <= 128:
        return -2
    if n_mesh <= 256:
        return -1
    return 0


class GpuBackend:
    """Device side of the server: one native lane + stream + buffers per slot; lanes of small meshes
    run on higher-priority streams (stream_priority)."""

    def __init__(self, device=None):
        import torch
        self.torch = torch
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)

    def lane_bytes(self, req: Request, capacity: int) -> int:
        from .batch import BatchRunner
        ncol = 4 if req.w is not None else 3
        b = BatchRunner.bytes_per_lane(req.n_mesh, capacity=capacity, mas=req.mas, interlace=req.interlace,
                                       ells=req.ells, device=self.device)
        return b + ncol * 4 * capacity + 4096

    def create(self, req: Request, capacity: int):
        return _GpuLane(self, req, capacity)

    def lane_bytes_of(self, lane) -> int:
        return lane.runner.device_bytes + lane.xyz.numel() * 4 + 4096

    def destroy(self, lane):
        lane.close()

    def start(self, lane, req: Request):
        lane.start(req)

    def finished(self, lane) -> bool:
        return lane.event.query()

    def result(self, lane, req: Request) -> Result:
        return lane.result(req)


class _GpuLane:
    def __init__(self, be: GpuBackend, req: Request, capacity: int):
        import torch
        from . import _lib
        from .batch import BatchRunner
        self.torch, self.lib = torch, _lib
        dev = be.device
        self.device = dev
        self.runner = BatchRunner(req.n_mesh, capacity=capacity, mas=req.mas, interlace=req.interlace,
                                  ells=req.ells, n_lanes=1, device=dev)
        ncol = 4 if req.w is not None else 3
        self.xyz = torch.empty((ncol, capacity), dtype=torch.float32, device=dev)
        self.job_host = torch.empty((1, _lib.JOB_BYTES), dtype=torch.uint8, pin_memory=True)
        self.job_dev = torch.empty((1, _lib.JOB_BYTES), dtype=torch.uint8, device=dev)
        self.out = self.runner.alloc_result(1)
        nb = self.runner.nb
        self.pk_host = torch.empty((1, nb, 3), dtype=torch.float64, pin_memory=True)
        self.km_host = torch.empty((1, nb), dtype=torch.float64, pin_memory=True)
        self.nm_host = torch.empty((1, nb), dtype=torch.int64, pin_memory=True)
        self.st_host = torch.empty((1, _lib.STATS_BYTES), dtype=torch.uint8, pin_memory=True)
        self.stream = torch.cuda.Stream(device=dev, priority=stream_priority(req.n_mesh))
        self.event = torch.cuda.Event()
        self.event.record(self.stream)
        self.kedges = self.runner.kedges_grid

    def _pinned(self, a):
        t = a if isinstance(a, self.torch.Tensor) else self.torch.from_numpy(np.ascontiguousarray(a, np.float32))
        return t if t.is_pinned() else t.pin_memory()

    def start(self, req: Request):
        torch, _lib = self.torch, self.lib
        n = req.n
        cols = [req.x, req.y, req.z] + ([req.w] if req.w is not None else [])
        with torch.cuda.stream(self.stream):
            for k, a in enumerate(cols):
                self.xyz[k, :n].copy_(self._pinned(a).reshape(-1), non_blocking=True)
            j = _lib.Job()
            base, stride = self.xyz.data_ptr(), self.xyz.shape[1] * 4
            j.x, j.y, j.z = base, base + stride, base + 2 * stride
            j.w = base + 3 * stride if req.w is not None else None
            j.n = n
            j.inv_cell = float(np.float32(req.n_mesh / float(req.box)))
            j.xmin, j.ymin, j.zmin = (float(np.float32(v)) for v in req.origin)
            j.box_size = float(req.box)
            self.job_host.numpy()[0, :] = np.frombuffer(bytes(j), dtype=np.uint8)
            self.job_dev.copy_(self.job_host, non_blocking=True)
            self.runner.run_one(self.job_dev, 0, self.out)
            self.pk_host.copy_(self.out.pk, non_blocking=True)
            self.km_host.copy_(self.out.kmean, non_blocking=True)
            self.nm_host.copy_(self.out.nmodes, non_blocking=True)
            self.st_host.copy_(self.out.stats, non_blocking=True)
            self.event.record(self.stream)

    def result(self, req: Request) -> Result:
        st = self.lib.DepositStats.from_buffer_copy(self.st_host.numpy()[0].tobytes())
        return Result(req.ticket, pk=self.pk_host.numpy()[0].copy(), k=self.km_host.numpy()[0].copy(),
                      nmodes=self.nm_host.numpy()[0].copy(), n_kept=int(st.n_kept))

    def close(self):
        self.event.synchronize()
        self.runner.close()
