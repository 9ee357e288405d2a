"""Fused particle -> P_l(k) pipeline (deposit -> FFT -> fused binning).

``PowerSpectrum`` keeps every buffer it needs (spectra, workspaces, the FFT
plan and the bin plan) resident on the device, so repeated calls allocate
nothing and launch only the kernels:

    bucket particles by column tile, deposit each tile
    and transform it along z in shared memory, y pass,
    x pass fused with window / interlace / |d|^2 L_l /
    binning / fold                                        -> gbp_particles_power
    (cuFFT mesh sizes: gbp_deposit, gbp_fft_r2c, gbp_power)
    normalisation, shot noise                             -> gbp_power_normalize

Unlike the reference pipeline (cic_mas_vec -> delta/mean - 1 -> powspec_vec),
the mean-density normalisation is not a pass over the mesh: the deposit sums
the mesh exactly (fixed point) and the normaliser divides by that total.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib, _native
from .correlations import default_kedges

__all__ = ["PkConfig", "PkResult", "PowerSpectrum", "power_multipoles", "algorithmic_bytes"]

_ELL_BITS = {0: _lib.ELL0, 2: _lib.ELL2, 4: _lib.ELL4}


@dataclass(frozen=True)
class PkConfig:
    n_mesh: int
    box_size: float
    mas: str = "tsc"
    interlace: bool = True
    ells: tuple = (0, 2, 4)
    shot_noise: bool = True
    k_edges: tuple | None = None          # h/Mpc; default kF .. kNyq step kF
    k_edges_kf: tuple | None = None       # edges in units of kF (exact); overrides k_edges
    origin: tuple = (0.0, 0.0, 0.0)
    kmean: bool = True

    @property
    def grids(self) -> int:
        return 2 if self.interlace else 1

    @property
    def mas_order(self) -> int:
        return _lib.MAS[self.mas.lower()]

    def edges(self) -> np.ndarray:
        if self.k_edges_kf is not None:
            return (np.asarray(self.k_edges_kf, np.float64) * (2.0 * np.pi / self.box_size)).astype(np.float32)
        if self.k_edges is None:
            return default_kedges(self.n_mesh, self.box_size)
        return np.asarray(self.k_edges, dtype=np.float32)

    def kedges_grid(self) -> np.ndarray:
        """Edges in units of kF (float32): the bins' integer thresholds come from these."""
        if self.k_edges_kf is not None:
            return np.asarray(self.k_edges_kf, dtype=np.float32)
        kf = np.float32(2.0 * np.pi / self.box_size)
        return (self.edges() / kf).astype(np.float32)

    def ells_mask(self) -> int:
        m = 0
        for l in self.ells:
            m |= _ELL_BITS[int(l)]
        if self.kmean:
            m |= _lib.KSUM
        return m


@dataclass
class PkResult:
    k_edges: np.ndarray                   # h/Mpc, float32 [nb+1]
    k_centres: torch.Tensor               # float64 [nb]
    k_mean: torch.Tensor | None           # float64 [nb] mode-averaged |k|
    pk: torch.Tensor                      # float64 [nb, 3]: P_0, P_2, P_4
    nmodes: torch.Tensor                  # int64 [nb]
    stats: torch.Tensor = field(repr=False, default=None)

    def numpy(self) -> dict:
        return {
            "k": self.k_centres.cpu().numpy(),
            "k_mean": None if self.k_mean is None else self.k_mean.cpu().numpy(),
            "pk": self.pk.cpu().numpy(),
            "nmodes": self.nmodes.cpu().numpy(),
        }


def algorithmic_bytes(n_particles: int, n_mesh: int, grids: int, weighted: bool = False) -> int:
    """Bytes a perfect implementation must move per mock: read particles once,
    write the meshes once, the FFT reads them and writes the half-complex
    spectra once, the binning reads the spectra once."""
    M = n_mesh ** 3
    Mh = n_mesh * n_mesh * (n_mesh // 2 + 1)
    return int(n_particles) * (16 if weighted else 12) + grids * (4 * M + 4 * M + 8 * Mh + 8 * Mh)


class PowerSpectrum:
    """Resident pipeline for one configuration on one device.

    Library transform sizes (power-of-two meshes 64..1024) run the fused
    path, one call to gbp_particles_power: the deposit fused with the z pass
    of the FFT, the y pass, the x pass fused with the binning; no mesh is
    stored.  Other sizes deposit a mesh (gbp_deposit), transform it with
    cuFFT (gbp_fft_r2c) and bin it (gbp_power).
    """

    def __init__(self, cfg: PkConfig, device=None, tiles=None):
        if not torch.cuda.is_available():
            raise RuntimeError("gbpowspec needs a CUDA device; there is no CPU fallback")
        self.cfg = cfg
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        N, G = cfg.n_mesh, cfg.grids
        dev = self.device
        self.stats = torch.empty(_lib.STATS_BYTES, dtype=torch.uint8, device=dev)
        # column tile of the fused path: None = the library default, "auto" = the autotuner's choice for
        # this shape (tune.py), or (tx, ty); every choice gives the same results bit for bit
        if tiles == "auto":
            from .tune import default_tuner
            tiles = default_tuner().best(N, cfg.mas, cfg.interlace, device=dev)
        if tiles is None or not _native.tile_variants(N):
            self.plan = _native.fft_plan(N, G, dev)
        else:
            self.plan = _native.FFTPlan(N, G, dev)      # a plan of its own: the tile is a plan option
            self.plan.set_tiles(*tiles)
        self.spec = torch.empty(self.plan.spectrum_floats, dtype=torch.float32, device=dev)
        self.bins = _native.bins_for(cfg.kedges_grid(), N, dev)
        self.ells = cfg.ells_mask()
        nb = self.bins.n_bins
        self.sums = _native.PowerSums(torch.empty((nb, 3), dtype=torch.float64, device=dev),
                                      torch.empty(nb, dtype=torch.int64, device=dev),
                                      torch.empty(nb, dtype=torch.float64, device=dev) if cfg.kmean else None)
        self.pk = torch.empty((nb, 3), dtype=torch.float64, device=dev)
        self.kmean = torch.empty(nb, dtype=torch.float64, device=dev) if cfg.kmean else None
        # fused path when the library's own transform serves this mesh
        self.fused = _native.particles_power_workspace_size(1, self.plan, self.bins, cfg.mas_order,
                                                            self.ells) is not None
        self.mesh = None if self.fused else torch.empty((G, N, N, N), dtype=torch.float32, device=dev)
        self.fft_ws = None if self.fused else _native.workspace(self.plan.ws_bytes, dev)
        self.pow_ws = None if self.fused else _native.workspace(
            _native.power_workspace_size(self.bins, G, self.ells, self.plan.pitch), dev)
        self.ws = None
        edges = cfg.edges()
        self.k_edges = edges
        self.k_centres = torch.from_numpy(0.5 * (edges[1:].astype(np.float64) + edges[:-1])).to(dev)

    @property
    def tiles(self):
        """The column tile (tx, ty) of the fused path, or None on the mesh path."""
        return self.plan.tiles if self.fused else None

    def _ws(self, n: int) -> torch.Tensor:
        cfg = self.cfg
        if self.fused:
            need = _native.particles_power_workspace_size(n, self.plan, self.bins, cfg.mas_order, self.ells)
        else:
            need = _native.deposit_workspace_size(n, cfg.n_mesh, cfg.mas_order, cfg.interlace, _lib.COMPAT_NONE)
        if self.ws is None or self.ws.numel() < need:
            self.ws = _native.workspace(int(need * 1.25) + 4096, self.device)
        return self.ws

    def reserve(self, n_particles: int) -> None:
        """Pre-size the workspace (so a timed or captured call allocates nothing)."""
        self._ws(int(n_particles))

    def run(self, x: torch.Tensor, y: torch.Tensor, z: torch.Tensor, w: torch.Tensor | None = None) -> PkResult:
        """Enqueue the whole pipeline on the current stream (no host synchronisation)."""
        cfg = self.cfg
        N = cfg.n_mesh
        n = x.numel()
        inv_cell = np.float32(N / cfg.box_size)
        mass = self.stats  # gbp_deposit_stats starts with double mass[2]
        if self.fused:
            _native.particles_power(x, y, z, w, plan=self.plan, bins=self.bins, mas=cfg.mas_order, ells=self.ells,
                                    inv_cell=inv_cell, origin=cfg.origin, spec=self.spec, stats=self.stats,
                                    ws=self._ws(n), out=self.sums)
        else:
            _native.deposit(x, y, z, w, n_mesh=N, inv_cell=inv_cell, origin=cfg.origin, mas=cfg.mas_order,
                            interlace=cfg.interlace, compat=_lib.COMPAT_NONE, wrap=True, out=self.mesh,
                            stats=self.stats, ws=self._ws(n))
            self.plan.execute(self.mesh, self.spec, self.fft_ws)
            _native.power(self.spec, cfg.grids, self.bins, mas_order=cfg.mas_order, ells=self.ells,
                          z_pitch=self.plan.pitch, mass=mass, ws=self.pow_ws, out=self.sums)
        _native.normalize(self.sums, n_mesh=N, box_size=cfg.box_size, mass=mass, stats=self.stats,
                          subtract_shot=cfg.shot_noise, pk_out=self.pk, kmean_out=self.kmean)
        return PkResult(self.k_edges, self.k_centres, self.kmean, self.pk, self.sums.nmodes, self.stats)

    __call__ = run


def power_multipoles(x, y, z, w=None, *, box_size: float, n_mesh: int, mas: str = "tsc", interlace: bool = True,
                     ells=(0, 2, 4), shot_noise: bool = True, k_edges=None, origin=(0.0, 0.0, 0.0),
                     device=None) -> PkResult:
    """One-shot P_l(k) of a particle catalogue in a periodic box (fresh buffers)."""
    xs = _native.as_cuda_f32(x, device).reshape(-1)
    dev = xs.device
    ys = _native.as_cuda_f32(y, dev).reshape(-1)
    zs = _native.as_cuda_f32(z, dev).reshape(-1)
    ws = None if w is None else _native.as_cuda_f32(w, dev).reshape(-1)
    cfg = PkConfig(n_mesh=int(n_mesh), box_size=float(box_size), mas=mas, interlace=bool(interlace),
                   ells=tuple(ells), shot_noise=bool(shot_noise),
                   k_edges=None if k_edges is None else tuple(np.asarray(k_edges, dtype=np.float32).tolist()),
                   origin=tuple(float(o) for o in origin))
    res = PowerSpectrum(cfg, dev).run(xs, ys, zs, ws)
    return res
