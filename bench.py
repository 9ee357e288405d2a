"""Throughput benchmark: P_0,2,4(k) mocks/s on 512^3 TSC+interlaced lognormal mocks.

Workload (the configuration the headline metric is quoted on): 4,194,304
float32 particles Poisson-like-sampled from a lognormal field on 256^3
(Gaussian P(k) = A k exp(-(k/0.3)^2), sigma_G^2 = 1), shifted along z by
N(0, 3 Mpc/h) velocities, periodic box L = 2500 Mpc/h; mesh 512^3, TSC with
interlacing, multipoles l = 0, 2, 4, k bins kF .. kNyq in steps of kF.
Synthetic, seeded data (no survey catalogue is needed or used).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = one mock through deposit -> FFT -> fused binning, particles
already resident in HBM.  Every step streams ~4.4 GB of meshes and spectra,
far more than the 129 MB L2, so no cache flush is needed between steps.
Under torchrun each rank processes its own mocks (replicas, no collective
on the data path); value = all ranks' mocks / max over ranks of the time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "jax-powspec_gb300"))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

CONFIG = dict(workload="lognormal+RSD 512^3 TSC+interlaced P_0,2,4 (4,194,304 particles, L=2500)",
              n_particles=4_194_304, n_mesh=512, box=2500.0, mas="tsc", interlace=True, ells=(0, 2, 4),
              field_grid=256, rsd_sigma=3.0)
METRIC = "mocks/sec for P_0,2,4(k) at 512^3/4M particles"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clock/throttle samples taken while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(s):
            try:
                return float(s)
            except ValueError:
                return float("nan")

        sm = np.array([num(r[1]) for r in rows])
        mx = np.array([num(r[2]) for r in rows])
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        load = sm[sm >= np.nanmax(sm) * 0.5] if np.isfinite(sm).any() else sm
        return {"sm_mhz": float(np.nanmedian(load)), "sm_max_mhz": float(np.nanmax(mx)), "reasons": reasons,
                "samples": len(rows)}


def make_catalogue(seed: int):
    from gbpowspec.synth import lognormal_catalogue
    return lognormal_catalogue(CONFIG["n_particles"], CONFIG["box"], grid=CONFIG["field_grid"], seed=seed,
                               rsd_sigma=CONFIG["rsd_sigma"])


def cpu_reference_mock(x, y, z) -> float:
    """The reference's path (cic_mas_vec -> delta/mean-1 -> powspec_vec), numpy port, one mock: seconds."""
    from oracle import reference_f32 as R
    N, box = CONFIG["n_mesh"], CONFIG["box"]
    kf = 2 * np.pi / box
    edges = np.arange(kf, np.pi * N / box, kf).astype(np.float32)
    t0 = time.perf_counter()
    d = R.cic_mas_vec(np.zeros((N, N, N), np.float32), x, y, z, None, x.size, 0.0, 0.0, 0.0, box, N, True)
    d = d / d.mean() - np.float32(1.0)
    R.powspec_vec(d, box, edges)
    return time.perf_counter() - t0


def run_reference_arm(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return
    x, y, z = make_catalogue(seed=1000)
    for _ in range(args.warmup_ref):
        cpu_reference_mock(x, y, z)
    times = [cpu_reference_mock(x, y, z) for _ in range(args.steps_ref)]
    t = float(np.median(times))
    v = 1.0 / t
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "mocks/s", "n_gpus": ws,
        "steps": len(times), "warmup": args.warmup_ref, "ms_per_step": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded lognormal mock)",
        "config": {**_cfg_json(), "implementation": "numpy port of src/mas.py cic_mas_vec + src/correlations.py "
                   "powspec_vec (CIC, no interlacing: the reference's only scheme)"},
        "cpu_baseline": {"value": v, "unit": "mocks/s", "cores": 1, "kind": "port",
                         "sample": "one full 512^3 / 4,194,304-particle mock per step"},
        "e2e": {"value": v, "unit": "mocks/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _cfg_json():
    return {"workload": CONFIG["workload"], "n_particles": CONFIG["n_particles"], "n_mesh": CONFIG["n_mesh"],
            "box_size": CONFIG["box"], "mas": CONFIG["mas"], "interlace": CONFIG["interlace"],
            "ells": list(CONFIG["ells"]), "l2_policy": "inputs larger than L2 (4.4 GB streamed per mock)",
            "parallelism": "replicas"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--steps-ref", type=int, default=2)
    ap.add_argument("--warmup-ref", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--n-mesh", type=int, default=None, help="override the mesh side (profiling cases)")
    ap.add_argument("--n-particles", type=int, default=None, help="override the particle count")
    ap.add_argument("--profile-only", action="store_true",
                    help="warm-up + timed steps only (no stage/e2e/CPU legs): a short command for ncu")
    args = ap.parse_args()
    if args.n_mesh:
        CONFIG["n_mesh"] = args.n_mesh
        CONFIG["field_grid"] = min(256, args.n_mesh)
    if args.n_particles:
        CONFIG["n_particles"] = args.n_particles
    if args.n_mesh or args.n_particles:
        CONFIG["workload"] = (f"lognormal+RSD {CONFIG['n_mesh']}^3 TSC+interlaced P_0,2,4 "
                              f"({CONFIG['n_particles']:,} particles, L={CONFIG['box']:g}) [override]")
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference_arm(args)
        return

    import torch
    import torch.distributed as dist

    from gbpowspec import PkConfig, PowerSpectrum, algorithmic_bytes
    from gbpowspec import _native

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=dev)

    x, y, z = make_catalogue(seed=1000 + rank)
    n = x.size
    host = [torch.from_numpy(a).pin_memory() for a in (x, y, z)]
    xd, yd, zd = (h.to(dev) for h in host)
    cfg = PkConfig(n_mesh=CONFIG["n_mesh"], box_size=CONFIG["box"], mas=CONFIG["mas"],
                   interlace=CONFIG["interlace"], ells=CONFIG["ells"])
    ps = PowerSpectrum(cfg, dev)
    ps.reserve(n)
    stream = torch.cuda.current_stream(dev)

    def barrier():
        if ws > 1:
            dist.barrier()

    for _ in range(args.warmup):
        ps.run(xd, yd, zd)
    torch.cuda.synchronize(dev)

    # ---- headline: device-resident inputs
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        ps.run(xd, yd, zd)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    barrier()
    t_dev = e0.elapsed_time(e1) / 1e3
    clk = clocks.stop()
    if args.profile_only:
        if rank == 0:
            print(json.dumps({"profile_only": True, "ms_per_step": t_dev / args.steps * 1e3,
                              "config": _cfg_json()}), flush=True)
        if ws > 1:
            dist.destroy_process_group()
        return

    # ---- stage breakdown (instrumented loop, events between the stages)
    N, G = cfg.n_mesh, cfg.grids
    stage_names = ["deposit", "fft", "power", "normalize"]
    acc = {s: 0.0 for s in stage_names}
    reps = max(3, min(args.steps, 10))
    import ctypes as C
    from gbpowspec import _lib
    inv = np.float32(N / cfg.box_size)
    for _ in range(reps):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
        ev[0].record(stream)
        _native.deposit(xd, yd, zd, None, n_mesh=N, inv_cell=inv, origin=cfg.origin, mas=cfg.mas_order,
                        interlace=cfg.interlace, compat=0, wrap=True, out=ps.mesh, stats=ps.stats,
                        ws=ps._dep_ws(n))
        ev[1].record(stream)
        ps.plan.execute(ps.mesh, ps.spec, ps.fft_ws)
        ev[2].record(stream)
        _native.power(ps.spec, G, ps.bins, mas_order=cfg.mas_order, ells=ps.ells, z_pitch=ps.plan.pitch,
                      mass=ps.stats, ws=ps.pow_ws,
                      out=ps.sums)
        ev[3].record(stream)
        _native.normalize(ps.sums, n_mesh=N, box_size=cfg.box_size, mass=ps.stats, stats=ps.stats,
                          subtract_shot=cfg.shot_noise, pk_out=ps.pk, kmean_out=ps.kmean)
        ev[4].record(stream)
        torch.cuda.synchronize(dev)
        for i, s in enumerate(stage_names):
            acc[s] += ev[i].elapsed_time(ev[i + 1]) / 1e3
    stage = {s: acc[s] / reps for s in stage_names}
    Mh = N * N * (N // 2 + 1)
    alg = {"deposit": n * 12 + G * 4 * N ** 3, "fft": G * (4 * N ** 3 + 8 * Mh), "power": G * 8 * Mh}
    dom = max(alg, key=lambda s: stage[s])
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = alg[dom] / stage[dom] / 1e9

    # ---- end to end: pinned host particles -> device, pipeline, P_l back to host
    pk_host = torch.empty(ps.pk.shape, dtype=ps.pk.dtype, pin_memory=True)
    nm_host = torch.empty(ps.sums.nmodes.shape, dtype=torch.int64, pin_memory=True)
    for _ in range(2):
        for h, d in zip(host, (xd, yd, zd)):
            d.copy_(h, non_blocking=True)
        ps.run(xd, yd, zd)
        pk_host.copy_(ps.pk, non_blocking=True)
    torch.cuda.synchronize(dev)
    barrier()
    e2, e3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e2.record(stream)
    for _ in range(args.steps):
        for h, d in zip(host, (xd, yd, zd)):
            d.copy_(h, non_blocking=True)
        r = ps.run(xd, yd, zd)
        pk_host.copy_(r.pk, non_blocking=True)
        nm_host.copy_(r.nmodes, non_blocking=True)
    e3.record(stream)
    torch.cuda.synchronize(dev)
    barrier()
    t_e2e = e2.elapsed_time(e3) / 1e3

    # max over ranks
    times = torch.tensor([t_dev, t_e2e], dtype=torch.float64, device=dev)
    if ws > 1:
        dist.all_reduce(times, op=dist.ReduceOp.MAX)
    t_dev, t_e2e = float(times[0]), float(times[1])

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        t_cpu = cpu_reference_mock(x, y, z)
        cpu = {"value": 1.0 / t_cpu, "unit": "mocks/s", "cores": 1, "kind": "port",
               "sample": "one full 512^3 / 4,194,304-particle mock of the reference path (CIC, no interlacing) "
                         "through the numpy port of src/mas.py + src/correlations.py"}

    mocks = ws * args.steps
    kernels_per_mock = 7   # count, scatter, tile deposit, stats, power, fold, normalize (cub scan/cuFFT excluded)
    line = {
        "metric": METRIC, "value": mocks / t_dev, "unit": "mocks/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_dev / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded lognormal+RSD mocks)",
        "config": {**_cfg_json(), "path": "plain (one mock per step, resident PowerSpectrum)"},
        "particles_per_s": mocks * n / t_dev,
        "stages_ms": {s: round(v * 1e3, 4) for s, v in stage.items()},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback 6800 GB/s",
                     "algorithmic_bytes": alg[dom]},
        "pipeline_roofline": {"algorithmic_bytes_per_mock": algorithmic_bytes(n, N, G),
                              "frac": algorithmic_bytes(n, N, G) * mocks / ws / t_dev / 1e9 / peak},
        "cpu_baseline": cpu,
        "e2e": {"value": mocks / t_e2e, "unit": "mocks/s", "h2d_bytes_per_step": 3 * 4 * n,
                "d2h_bytes_per_step": int(pk_host.numel() * 8 + nm_host.numel() * 8)},
        "gpu_launches": kernels_per_mock * args.steps,
        "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
