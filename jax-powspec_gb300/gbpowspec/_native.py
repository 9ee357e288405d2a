"""Torch-tensor wrappers over the C ABI: buffers, workspaces, plan caches.

Every function here launches CUDA work through libgbpowspec.so on the
current torch stream of the tensors' device; nothing runs on the CPU except
argument checks and the small host-side tables (bin thresholds).
"""
from __future__ import annotations

import ctypes as C
import threading
from collections import OrderedDict
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from ._lib import check

_F32 = torch.float32


def _ptr(t: torch.Tensor | None) -> C.c_void_p | None:
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream_of(device: torch.device) -> C.c_void_p:
    return C.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def as_cuda_f32(a, device: torch.device | None = None, name: str = "array") -> torch.Tensor:
    """A contiguous float32 CUDA tensor view/copy of `a` (tensor, numpy or sequence)."""
    if isinstance(a, torch.Tensor):
        t = a
    else:
        t = torch.as_tensor(np.asarray(a))
    if device is None:
        device = t.device if t.is_cuda else torch.device("cuda", torch.cuda.current_device())
    if not torch.cuda.is_available():
        raise RuntimeError("gbpowspec needs a CUDA device; there is no CPU fallback")
    t = t.to(device=device, dtype=_F32, non_blocking=True)
    if not t.is_contiguous():
        t = t.contiguous()
    return t


def workspace(nbytes: int, device: torch.device) -> torch.Tensor:
    """Scratch buffer from torch's caching allocator (cheap after the first call)."""
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)


def read_stats(stats: torch.Tensor) -> _lib.DepositStats:
    """Copy a device gbp_deposit_stats to the host (synchronises the stream)."""
    raw = stats.detach().cpu().numpy().tobytes()
    return _lib.DepositStats.from_buffer_copy(raw)


# ---------------------------------------------------------------- deposit
def deposit_workspace_size(n: int, n_mesh: int, mas: int, interlace: bool, compat: int) -> int:
    lib = _lib.load()
    out = C.c_size_t(0)
    check(lib.gbp_deposit_workspace_size(int(n), int(n_mesh), int(mas), int(interlace), int(compat),
                                         C.byref(out)), "gbp_deposit_workspace_size")
    return out.value


def deposit(x: torch.Tensor, y: torch.Tensor, z: torch.Tensor, w: torch.Tensor | None, *,
            n_mesh: int, inv_cell: float, origin=(0.0, 0.0, 0.0), mas: int = 2,
            interlace: bool = False, compat: int = 0, wrap: bool = True,
            mesh_in: torch.Tensor | None = None, out: torch.Tensor | None = None,
            stats: torch.Tensor | None = None, ws: torch.Tensor | None = None):
    """Deposit particles; returns (mesh [G,N,N,N] float32, stats uint8 tensor)."""
    lib = _lib.load()
    dev = x.device
    n = x.numel()
    for t, nm in ((x, "x"), (y, "y"), (z, "z"), (w, "w")):
        if t is None:
            continue
        if not (t.is_cuda and t.dtype == _F32 and t.is_contiguous() and t.numel() == n and t.device == dev):
            raise ValueError(f"{nm} must be a contiguous float32 CUDA tensor with {n} elements on {dev}")
    G = 2 if interlace else 1
    N = int(n_mesh)
    if out is None:
        out = torch.empty((G, N, N, N), dtype=_F32, device=dev)
    elif not (out.is_cuda and out.dtype == _F32 and out.is_contiguous() and out.numel() == G * N ** 3):
        raise ValueError("out must be a contiguous float32 CUDA tensor of G*N^3 elements")
    if mesh_in is not None and not (mesh_in.is_cuda and mesh_in.dtype == _F32 and mesh_in.is_contiguous()
                                    and mesh_in.numel() == G * N ** 3):
        raise ValueError("mesh_in must be a contiguous float32 CUDA tensor of G*N^3 elements")
    if stats is None:
        stats = torch.empty(_lib.STATS_BYTES, dtype=torch.uint8, device=dev)
    need = deposit_workspace_size(n, N, mas, interlace, compat)
    if ws is None or ws.numel() < need:
        ws = workspace(need, dev)
    check(lib.gbp_deposit(_ptr(x), _ptr(y), _ptr(z), _ptr(w), n,
                          float(np.float32(origin[0])), float(np.float32(origin[1])), float(np.float32(origin[2])),
                          float(np.float32(inv_cell)), N, int(mas), int(interlace), int(compat), int(wrap),
                          _ptr(mesh_in), _ptr(out), _ptr(stats), _ptr(ws), ws.numel(), _stream_of(dev)),
          "gbp_deposit")
    return out, stats


# ---------------------------------------------------------------- FFT plans
class FFTPlan:
    """3-D R2C plan for `grids` meshes of side n (owned; freed on close).

    `pitch` is the number of complex entries per z row of the spectrum it
    writes (the first n//2+1 are the modes); `spectrum_floats` the float32
    count of a buffer that holds all grids' spectra.
    """

    def __init__(self, n: int, grids: int, device: torch.device):
        lib = _lib.load()
        self.n, self.grids, self.device = int(n), int(grids), device
        h = C.c_void_p()
        wsb = C.c_size_t(0)
        pitch = C.c_int(0)
        with torch.cuda.device(device):
            check(lib.gbp_fft_plan_create(self.n, self.grids, C.byref(h), C.byref(wsb)), "gbp_fft_plan_create")
            check(lib.gbp_fft_plan_pitch(h, C.byref(pitch)), "gbp_fft_plan_pitch")
        self.handle, self.ws_bytes, self.pitch = h, wsb.value, pitch.value

    @property
    def spectrum_floats(self) -> int:
        return self.grids * self.n * self.n * self.pitch * 2

    def set_tiles(self, tx: int = 0, ty: int = 0) -> None:
        """Column tile (tx x ty pencils) of the fused particles path; 0, 0 = the default."""
        check(_lib.load().gbp_fft_plan_set_tiles(self.handle, int(tx), int(ty)), "gbp_fft_plan_set_tiles")

    @property
    def tiles(self) -> tuple:
        tx, ty = C.c_int(0), C.c_int(0)
        check(_lib.load().gbp_fft_plan_tiles(self.handle, C.byref(tx), C.byref(ty)), "gbp_fft_plan_tiles")
        return tx.value, ty.value

    def execute(self, mesh: torch.Tensor, spec: torch.Tensor, ws: torch.Tensor | None = None) -> torch.Tensor:
        n, G = self.n, self.grids
        if mesh.numel() != G * n ** 3 or mesh.dtype != _F32 or not mesh.is_contiguous():
            raise ValueError("mesh does not match the plan")
        if spec.numel() * spec.element_size() < self.spectrum_floats * 4:
            raise ValueError("spectrum buffer too small")
        if self.ws_bytes and (ws is None or ws.numel() < self.ws_bytes):
            ws = workspace(self.ws_bytes, mesh.device)
        check(_lib.load().gbp_fft_r2c(self.handle, _ptr(mesh), _ptr(spec), _ptr(ws),
                                      0 if ws is None else ws.numel(), _stream_of(mesh.device)), "gbp_fft_r2c")
        return spec

    def close(self):
        if self.handle:
            _lib.load().gbp_fft_plan_destroy(self.handle)
            self.handle = None


def tile_variants(n_mesh: int) -> list:
    """Column tiles [(tx, ty), ...] of the fused path for an n_mesh^3 mesh, the default first ([] when the
    mesh size has no fused path)."""
    tx, ty, cnt = (C.c_int * 8)(), (C.c_int * 8)(), C.c_int(0)
    st = _lib.load().gbp_column_tile_variants(int(n_mesh), tx, ty, 8, C.byref(cnt))
    if st == _lib.GBP_ERR_UNSUPPORTED:
        return []
    check(st, "gbp_column_tile_variants")
    return [(tx[i], ty[i]) for i in range(min(cnt.value, 8))]


_plans: dict = {}
_plans_lock = threading.Lock()


def fft_plan(n: int, grids: int, device: torch.device) -> FFTPlan:
    key = (device.index, int(n), int(grids))
    with _plans_lock:
        p = _plans.get(key)
        if p is None:
            p = _plans[key] = FFTPlan(n, grids, device)
        return p


# ---------------------------------------------------------------- bins
def bin_thresholds(kedges_grid: np.ndarray, n_mesh: int):
    """Host-only: exact integer k^2 thresholds of float32 edges (grid units)."""
    e = np.ascontiguousarray(kedges_grid, dtype=np.float32)
    thr = np.zeros(e.size, dtype=np.int32)
    last = C.c_int32(0)
    reach = C.c_int(0)
    check(_lib.load().gbp_bin_thresholds(e.ctypes.data_as(C.c_void_p), e.size, int(n_mesh),
                                         thr.ctypes.data_as(C.c_void_p), C.byref(last), C.byref(reach)),
          "gbp_bin_thresholds")
    return thr, int(last.value), int(reach.value)


class Bins:
    """Device-resident bin plan for float32 edges in fundamental-frequency units."""

    def __init__(self, kedges_grid: np.ndarray, n_mesh: int, device: torch.device):
        e = np.ascontiguousarray(kedges_grid, dtype=np.float32)
        if e.ndim != 1 or e.size < 2:
            raise ValueError("k_edges must be a 1-D array with at least two edges")
        if not np.all(np.isfinite(e)) or np.any(np.diff(e) < 0):
            raise ValueError("k_edges must be finite and monotonically increasing")
        self.edges = e
        self.n_mesh = int(n_mesh)
        self.n_bins = e.size - 1
        self.device = device
        h = C.c_void_p()
        with torch.cuda.device(device):
            check(_lib.load().gbp_bins_create(e.ctypes.data_as(C.c_void_p), e.size, self.n_mesh, C.byref(h)),
                  "gbp_bins_create")
        self.handle = h

    def close(self):
        if self.handle:
            _lib.load().gbp_bins_destroy(self.handle)
            self.handle = None


_bins: "OrderedDict[tuple, Bins]" = OrderedDict()
_BINS_MAX = 64


def bins_for(kedges_grid: np.ndarray, n_mesh: int, device: torch.device) -> Bins:
    e = np.ascontiguousarray(kedges_grid, dtype=np.float32)
    key = (device.index, int(n_mesh), e.tobytes())
    with _plans_lock:
        b = _bins.get(key)
        if b is not None:
            _bins.move_to_end(key)
            return b
    b = Bins(e, n_mesh, device)
    with _plans_lock:
        _bins[key] = b
        while len(_bins) > _BINS_MAX:
            _, old = _bins.popitem(last=False)
            old.close()
    return b


# ---------------------------------------------------------------- power
@dataclass
class PowerSums:
    sums: torch.Tensor      # float64 [nb, 3]
    nmodes: torch.Tensor    # int64 [nb]
    ksum: torch.Tensor | None


def power_workspace_size(bins: Bins, grids: int, ells: int, z_pitch: int = 0) -> int:
    out = C.c_size_t(0)
    check(_lib.load().gbp_power_workspace_size(bins.handle, int(grids), int(z_pitch), int(ells), C.byref(out)),
          "gbp_power_workspace_size")
    return out.value


def power(spec: torch.Tensor, grids: int, bins: Bins, *, mas_order: int, ells: int, z_pitch: int = 0,
          mass: torch.Tensor | None = None, ws: torch.Tensor | None = None,
          out: PowerSums | None = None) -> PowerSums:
    """Binned moments of a spectrum whose z rows are `z_pitch` complex apart (0: n//2+1)."""
    dev = spec.device
    nb = bins.n_bins
    if out is None:
        out = PowerSums(torch.empty((nb, 3), dtype=torch.float64, device=dev),
                        torch.empty(nb, dtype=torch.int64, device=dev),
                        torch.empty(nb, dtype=torch.float64, device=dev) if ells & _lib.KSUM else None)
    need = power_workspace_size(bins, grids, ells, z_pitch)
    if ws is None or ws.numel() < need:
        ws = workspace(need, dev)
    check(_lib.load().gbp_power(_ptr(spec), int(grids), int(z_pitch), bins.handle, int(mas_order), int(ells),
                                _ptr(mass), _ptr(out.sums), _ptr(out.nmodes), _ptr(out.ksum), _ptr(ws), ws.numel(),
                                _stream_of(dev)), "gbp_power")
    return out


def fft_power_workspace_size(plan: "FFTPlan", bins: Bins, ells: int) -> int | None:
    """Workspace of the fused FFT + binning, or None when the plan cannot fuse (cuFFT sizes)."""
    out = C.c_size_t(0)
    st = _lib.load().gbp_fft_power_workspace_size(plan.handle, bins.handle, int(ells), C.byref(out))
    if st == _lib.GBP_ERR_UNSUPPORTED:
        return None
    check(st, "gbp_fft_power_workspace_size")
    return out.value


def fft_power(plan: "FFTPlan", mesh: torch.Tensor, spec: torch.Tensor, bins: Bins, *, mas_order: int, ells: int,
              mass: torch.Tensor | None = None, ws: torch.Tensor | None = None, out: PowerSums | None = None) -> PowerSums:
    """3-D FFT of the meshes fused with the binning (the spectrum buffer is scratch)."""
    dev = mesh.device
    n, G = plan.n, plan.grids
    if mesh.numel() != G * n ** 3 or mesh.dtype != _F32 or not mesh.is_contiguous():
        raise ValueError("mesh does not match the plan")
    if spec.numel() * spec.element_size() < plan.spectrum_floats * 4:
        raise ValueError("spectrum buffer too small")
    need = fft_power_workspace_size(plan, bins, ells)
    if need is None:
        raise ValueError("this plan cannot fuse the FFT with the binning (cuFFT size)")
    if ws is None or ws.numel() < need:
        ws = workspace(need, dev)
    nb = bins.n_bins
    if out is None:
        out = PowerSums(torch.empty((nb, 3), dtype=torch.float64, device=dev),
                        torch.empty(nb, dtype=torch.int64, device=dev),
                        torch.empty(nb, dtype=torch.float64, device=dev) if ells & _lib.KSUM else None)
    check(_lib.load().gbp_fft_power(plan.handle, _ptr(mesh), _ptr(spec), bins.handle, int(mas_order), int(ells),
                                    _ptr(mass), _ptr(out.sums), _ptr(out.nmodes), _ptr(out.ksum), _ptr(ws),
                                    ws.numel(), _stream_of(dev)), "gbp_fft_power")
    return out


def particles_power_workspace_size(n: int, plan: "FFTPlan", bins: Bins, mas: int, ells: int) -> int | None:
    """Workspace of the fused particles -> sums path, or None when the plan cannot fuse (cuFFT sizes)."""
    out = C.c_size_t(0)
    st = _lib.load().gbp_particles_power_workspace_size(int(n), plan.handle, bins.handle, int(mas), int(ells),
                                                         C.byref(out))
    if st == _lib.GBP_ERR_UNSUPPORTED:
        return None
    check(st, "gbp_particles_power_workspace_size")
    return out.value


def particles_power(x: torch.Tensor, y: torch.Tensor, z: torch.Tensor, w: torch.Tensor | None, *, plan: "FFTPlan",
                    bins: Bins, mas: int, ells: int, inv_cell: float, origin=(0.0, 0.0, 0.0),
                    spec: torch.Tensor, stats: torch.Tensor, ws: torch.Tensor | None = None,
                    out: PowerSums | None = None) -> PowerSums:
    """Deposit fused with the z pass, y pass, x pass fused with the binning (one library call)."""
    dev = x.device
    n = x.numel()
    for t, nm in ((x, "x"), (y, "y"), (z, "z"), (w, "w")):
        if t is not None and not (t.is_cuda and t.dtype == _F32 and t.is_contiguous() and t.numel() == n
                                  and t.device == dev):
            raise ValueError(f"{nm} must be a contiguous float32 CUDA tensor with {n} elements on {dev}")
    if spec.numel() * spec.element_size() < plan.spectrum_floats * 4:
        raise ValueError("spectrum buffer too small")
    need = particles_power_workspace_size(n, plan, bins, mas, ells)
    if need is None:
        raise ValueError("this plan cannot fuse the deposit with the FFT (cuFFT size)")
    if ws is None or ws.numel() < need:
        ws = workspace(need, dev)
    nb = bins.n_bins
    if out is None:
        out = PowerSums(torch.empty((nb, 3), dtype=torch.float64, device=dev),
                        torch.empty(nb, dtype=torch.int64, device=dev),
                        torch.empty(nb, dtype=torch.float64, device=dev) if ells & _lib.KSUM else None)
    check(_lib.load().gbp_particles_power(
        _ptr(x), _ptr(y), _ptr(z), _ptr(w), n, float(np.float32(origin[0])), float(np.float32(origin[1])),
        float(np.float32(origin[2])), float(np.float32(inv_cell)), plan.handle, bins.handle, int(mas), int(ells),
        _ptr(spec), _ptr(out.sums), _ptr(out.nmodes), _ptr(out.ksum), _ptr(stats), _ptr(ws), ws.numel(),
        _stream_of(dev)), "gbp_particles_power")
    return out


def normalize(ps: PowerSums, *, n_mesh: int, box_size: float, mass: torch.Tensor | None = None,
              stats: torch.Tensor | None = None, subtract_shot: bool = False,
              pk_out: torch.Tensor | None = None, kmean_out: torch.Tensor | None = None):
    dev = ps.sums.device
    nb = ps.sums.shape[0]
    if pk_out is None:
        pk_out = torch.empty((nb, 3), dtype=torch.float64, device=dev)
    if kmean_out is None and ps.ksum is not None:
        kmean_out = torch.empty(nb, dtype=torch.float64, device=dev)
    check(_lib.load().gbp_power_normalize(_ptr(ps.sums), _ptr(ps.nmodes), _ptr(ps.ksum), nb, int(n_mesh),
                                          float(box_size), _ptr(mass), _ptr(stats), int(subtract_shot),
                                          _ptr(pk_out), _ptr(kmean_out), _stream_of(dev)), "gbp_power_normalize")
    return pk_out, kmean_out


# ---------------------------------------------------------------- tracing
def trace_enable(capacity: int = 8192) -> None:
    """Start recording CUDA events around every kernel launch of the library."""
    check(_lib.load().gbp_trace_enable(int(capacity)), "gbp_trace_enable")


def trace_collect() -> list:
    """Stop tracing; [(kernel name, ms)] in launch order (waits for the launches)."""
    lib = _lib.load()
    cap = 65536
    recs = (_lib.TraceRecord * cap)()
    n = C.c_int(0)
    check(lib.gbp_trace_collect(C.cast(recs, C.c_void_p), cap, C.byref(n)), "gbp_trace_collect")
    return [(recs[i].kernel.decode(), float(recs[i].ms)) for i in range(n.value)]

