"""Autotuner for the fused path's column tile (no reference counterpart).

The deposit fused with the z pass buckets particles by column tile (tx x ty
pencils over all of z) and deposits one tile per CTA; the tile is also the
bucket of the particle sort.  Its best shape depends on the device, the
mesh, the scheme, interlacing and the particle count: small tiles replicate
more particles across tile faces (more bucket entries, more sort traffic),
large ones hold more shared memory per CTA (fewer CTAs per SM).  Every
shape gives the same P_l bit for bit (fixed-point scales per 4x4 block), so
the choice is pure speed.

``Tuner.best(N, mas, interlace, n)`` returns the shape to use.  The first
call for a (device, N, MAS, grids, n-bucket) key times every shape the
library offers (gbp_column_tile_variants) on a seeded lognormal catalogue
of n particles (CUDA events, median of a few runs after a warm-up), keeps
the fastest and writes it to a JSON cache (GBP_TUNE_CACHE, default
~/.cache/gbpowspec/tiles.json); later calls, in this process or another,
read it.  n-buckets are powers of two (round(log2 n)).  PowerSpectrum,
BatchRunner and the Server take ``tiles="auto"`` to use it.
"""
from __future__ import annotations

import json
import math
import os
import threading

__all__ = ["Tuner", "default_tuner"]


def _default_path() -> str:
    env = os.environ.get("GBP_TUNE_CACHE")
    if env:
        return env
    return os.path.join(os.path.expanduser("~"), ".cache", "gbpowspec", "tiles.json")


class Tuner:
    """Tile choices per shape, measured once and cached on disk.

    timer(N, mas, interlace, n, tiles, device) -> seconds per mock (default:
    CUDA-event timing of PowerSpectrum.run); variants(N) -> [(tx, ty), ...]
    (default: the library's list); device_name(device) -> str.  The three are
    injectable so the selection and caching logic runs without a GPU.
    """

    def __init__(self, path: str | None = None, timer=None, variants=None, device_name=None):
        self.path = path or _default_path()
        self.timer = timer or _time_tiles
        self.variants = variants or _library_variants
        self.device_name = device_name or _device_name
        self._lock = threading.Lock()
        self._cache = None
        self.timings = 0              # shapes measured by this instance

    @staticmethod
    def key(device: str, N: int, mas: str, interlace: bool, n: int) -> str:
        bucket = int(round(math.log2(max(int(n), 1))))
        return f"{device}|N{int(N)}|{mas.lower()}|G{2 if interlace else 1}|n2^{bucket}"

    def _load(self) -> dict:
        if self._cache is None:
            try:
                with open(self.path) as f:
                    self._cache = json.load(f)
            except (OSError, ValueError):
                self._cache = {}
        return self._cache

    def _save(self) -> None:
        try:
            os.makedirs(os.path.dirname(os.path.abspath(self.path)), exist_ok=True)
            tmp = f"{self.path}.{os.getpid()}.tmp"
            with open(tmp, "w") as f:
                json.dump(self._cache, f, indent=1, sort_keys=True)
            os.replace(tmp, self.path)
        except OSError:
            pass                      # a read-only home: keep the choice in memory only

    def entry(self, N: int, mas: str, interlace: bool, n: int | None = None, device=None) -> dict | None:
        """The cached record of a shape ({"tiles": [tx, ty], "ms": {...}}), or None."""
        n = _default_n(N) if n is None else int(n)
        with self._lock:
            return self._load().get(self.key(self.device_name(device), N, mas, interlace, n))

    def best(self, N: int, mas: str, interlace: bool, n: int | None = None, device=None) -> tuple:
        """(tx, ty) for this shape: cached, or measured now and cached."""
        cands = [tuple(v) for v in self.variants(int(N))]
        if not cands:
            raise ValueError(f"no fused path for {N}^3 meshes")
        if len(cands) == 1:
            return cands[0]
        n = _default_n(N) if n is None else int(n)
        key = self.key(self.device_name(device), N, mas, interlace, n)
        with self._lock:
            rec = self._load().get(key)
            if rec is not None and tuple(rec["tiles"]) in cands:
                return tuple(rec["tiles"])
            ms = {c: 1e3 * float(self.timer(int(N), mas, bool(interlace), n, c, device)) for c in cands}
            self.timings += 1
            best = min(cands, key=lambda c: (ms[c], cands.index(c)))     # ties: the library's order
            self._cache[key] = {"tiles": list(best), "ms": {f"{c[0]}x{c[1]}": round(ms[c], 5) for c in cands}}
            self._save()
            return best


def _default_n(N: int) -> int:
    """A typical catalogue for an N^3 mesh: one particle per 32 cells."""
    return max(1, N ** 3 // 32)


def _library_variants(N: int) -> list:
    from . import _native
    return _native.tile_variants(N)


def _device_name(device) -> str:
    import torch
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    return torch.cuda.get_device_name(dev).replace("|", "/")


def _time_tiles(N: int, mas: str, interlace: bool, n: int, tiles: tuple, device) -> float:
    """Seconds per mock of PowerSpectrum.run with these tiles on a seeded lognormal catalogue (median)."""
    import numpy as np
    import torch

    from .pipeline import PkConfig, PowerSpectrum
    from .synth import lognormal_catalogue_gpu
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    box = 1000.0
    x, y, z = (t.contiguous() for t in lognormal_catalogue_gpu(n, box, grid=min(int(N), 256), seed=12345,
                                                               rsd_sigma=3.0, device=dev))
    ps = PowerSpectrum(PkConfig(n_mesh=N, box_size=box, mas=mas, interlace=interlace), dev, tiles=tiles)
    ps.reserve(n)
    stream = torch.cuda.current_stream(dev)
    for _ in range(2):
        ps.run(x, y, z)
    ts = []
    for _ in range(5):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ps.run(x, y, z)
        b.record(stream)
        b.synchronize()
        ts.append(a.elapsed_time(b) / 1e3)
    return float(np.median(ts))


_default = None
_default_lock = threading.Lock()


def default_tuner() -> Tuner:
    global _default
    with _default_lock:
        if _default is None:
            _default = Tuner()
        return _default
