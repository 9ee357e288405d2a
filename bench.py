"""Throughput benchmark: P_0,2,4(k) mocks/s on 512^3 TSC+interlaced lognormal mocks, batched vs plain.

Workload (the configuration the headline metric is quoted on): 4,194,304
float32 particles Poisson-like-sampled from a lognormal field on 256^3
(Gaussian P(k) = A k exp(-(k/0.3)^2), sigma_G^2 = 1), shifted along z by
N(0, 3 Mpc/h) velocities, periodic box L = 2500 Mpc/h; mesh 512^3, TSC with
interlacing, multipoles l = 0, 2, 4, k bins kF .. kNyq in steps of kF.
Synthetic, seeded data (no survey catalogue is needed or used).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = one batch of `--batch` mocks through the batched path (lanes of
resident buffers replaying one CUDA graph per mock, several lanes on their
own streams), particles already resident in HBM; `value` is mocks/s of that
path.  The plain path (one mock at a time through PowerSpectrum.run, no
graph) is timed beside it.  Every mock streams ~4.4 GB of meshes and
spectra, far more than the 129 MB L2, so no cache flush is needed between
steps.  Per-kernel durations come from the library's CUDA-event trace of a
few plain mocks.  Under torchrun each rank processes its own mocks
(replicas, no collective on the data path); value = all ranks' mocks / max
over ranks of the time.
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
    """The reference's path for one mock (cic_mas_vec -> delta/mean - 1 -> powspec_vec), CPU stand-in
    (oracle/reference_fast: numpy, FFT on all host threads): seconds."""
    from oracle import reference_fast as F
    N, box = CONFIG["n_mesh"], CONFIG["box"]
    kf = 2 * np.pi / box
    edges = np.arange(kf, np.pi * N / box, kf).astype(np.float32)
    t0 = time.perf_counter()
    F.reference_mock(x, y, z, box, N, edges)
    return time.perf_counter() - t0


def cpu_cores() -> int:
    from oracle import reference_fast as F
    return F.threads()


CPU_SAMPLE = ("one full 512^3 / 4,194,304-particle mock per step of the reference path (cic_mas_vec with "
              "its CIC and corner bug, delta/mean - 1, powspec_vec; no interlacing: the reference's only "
              "scheme) through the numpy stand-in oracle/reference_fast (bincount scatter and histograms, "
              "scipy.fft on all host threads; deposit and binning single-threaded)")


def run_reference_arm(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return
    x, y, z = make_catalogue(seed=1000)
    steps, warm = max(1, args.steps), args.warmup    # each step is one full mock (a few seconds of CPU work)
    for _ in range(warm):
        cpu_reference_mock(x, y, z)
    times = [cpu_reference_mock(x, y, z) for _ in range(steps)]
    t = float(np.sum(times))
    v = steps / t
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "mocks/s", "n_gpus": ws,
        "steps": steps, "warmup": warm, "ms_per_step": t / steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded lognormal mock)",
        "config": {**_cfg_json(), "mas": "cic", "interlace": False, "grids": 1, "ells": [0, 2, 4],
                   "workload": CONFIG["workload"].replace("TSC+interlaced", "CIC one grid (the reference's "
                                                          "scheme) on the same catalogue"),
                   "implementation": "numpy stand-in (oracle/reference_fast) for the reference's own path: "
                   "src/mas.py cic_mas_vec (CIC with its corner-weight bug, one grid) -> delta/mean - 1 -> "
                   "src/correlations.py powspec_vec (float32 histograms); JAX is not installed on this host",
                   "differs_from_ours": "same catalogue, mesh, box and k bins; the reference implements CIC "
                   "only, without interlacing, so it deposits one grid with a 2^3 stencil where ours deposits "
                   "two with 3^3 (TSC + interlacing)"},
        "cpu_baseline": {"value": v, "unit": "mocks/s", "cores": cpu_cores(), "kind": "port", "sample": CPU_SAMPLE},
        "e2e": {"value": v, "unit": "mocks/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _cfg_json():
    return {"workload": CONFIG["workload"], "n_particles": CONFIG["n_particles"], "n_mesh": CONFIG["n_mesh"],
            "box_size": CONFIG["box"], "mas": CONFIG["mas"], "interlace": CONFIG["interlace"],
            "ells": list(CONFIG["ells"]), "l2_policy": "inputs larger than L2 (4.4 GB streamed per mock)",
            "parallelism": "replicas"}


def kernel_bytes(n: int, N: int, G: int) -> dict:
    """Algorithmic bytes per launch of each traced kernel (what the algorithm must move)."""
    M = N ** 3
    Mh = N * N * (N // 2 + 1)
    return {
        # one-pass bucketing: read x, y, z (the bucket writes are implementation traffic); its scan and
        # scatter return at once unless a bucket overflowed, so they get no byte count
        "deposit_fill": 12 * n,
        "deposit_count": 12 * n,                  # count path (small catalogues): read x, y, z
        # deposit fused with the z pass: every particle read once, the z-transformed half spectra written
        # once (the bucket entries it actually reads, 16 B per particle and touched tile, are
        # implementation traffic, as is the spectrum rows' padding)
        "deposit_fft_z": 12 * n + G * 8 * Mh,
        "deposit_tiles": 4 * G * M,               # write every cell of the G meshes once
        "fft_z": G * (4 * M + 8 * Mh),            # read the meshes, write half-spectra
        "fft_y": G * 16 * Mh,                     # read + write all grids' spectra
        "fft_x": 16 * Mh,                         # read + write one grid's spectrum
        "cufft_r2c": G * (4 * M + 8 * Mh),
        "power_bins": G * 8 * Mh,                 # read the spectra once
        "fft_x_bins": G * 8 * Mh,                 # read the z,y-transformed spectra once (x pass + binning)
    }


def trace_breakdown(ps, xd, yd, zd, reps: int, n: int) -> dict:
    """Per-kernel mean durations (CUDA events on the launching stream) over `reps` plain mocks."""
    import torch
    from gbpowspec import _native
    torch.cuda.synchronize()
    _native.trace_enable(4096)
    for _ in range(reps):
        ps.run(xd, yd, zd)
    recs = _native.trace_collect()
    per = {}
    for name, ms in recs:
        d = per.setdefault(name, [0, 0.0])
        d[0] += 1
        d[1] += ms
    N, G = ps.cfg.n_mesh, ps.cfg.grids
    alg = kernel_bytes(n, N, G)
    out = {}
    for name, (cnt, tot) in per.items():
        mean = tot / cnt
        row = {"launches_per_mock": cnt / reps, "mean_ms": round(mean, 5), "ms_per_mock": round(tot / reps, 5)}
        if name in alg:
            row["algorithmic_bytes"] = alg[name]
            row["achieved_gbs"] = round(alg[name] / (mean * 1e-3) / 1e9, 1)
        out[name] = row
    return out


def covariance_leg(dev, seed: int, n_mocks: int = 256) -> dict:
    """Batched covariance run: n_mocks lognormal mocks (device generator, a different seed each), particle
    counts log-uniform in [2e5, 2e6], half on 256^3 and half on 128^3, L = 1500, CIC + interlacing,
    l = 0, 2; both halves run concurrently; returns throughput and the covariance shapes."""
    import torch
    from gbpowspec.batch import BatchRunner, ParticleArena, covariance, run_mixed
    from gbpowspec.synth import lognormal_catalogue_gpu
    rng = np.random.default_rng(seed)
    box = 1500.0
    counts = np.exp(rng.uniform(np.log(2e5), np.log(2e6), n_mocks)).astype(np.int64)
    meshes = np.where(np.arange(n_mocks) % 2 == 0, 256, 128)
    arena = ParticleArena.empty(counts, device=dev)
    t0 = time.perf_counter()
    for i in range(n_mocks):
        lognormal_catalogue_gpu(int(counts[i]), box, grid=int(meshes[i]), seed=int(seed * 100003 + i),
                                rsd_sigma=3.0, device=dev, out=arena.views(i))
    torch.cuda.synchronize(dev)
    t_gen = time.perf_counter() - t0
    idx = {N: np.nonzero(meshes == N)[0] for N in (256, 128)}
    jobs = {N: arena.job_table(box, N, indices=idx[N]) for N in idx}
    cap = int(counts.max())
    runners = {N: BatchRunner(N, capacity=cap, mas="cic", interlace=True, ells=(0, 2), n_lanes=3, device=dev)
               for N in idx}
    run_mixed([(runners[N], jobs[N]) for N in idx])              # warm
    torch.cuda.synchronize(dev)
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    res = run_mixed([(runners[N], jobs[N]) for N in idx])
    e1.record(stream)
    torch.cuda.synchronize(dev)
    t = e0.elapsed_time(e1) / 1e3
    out = {"workload": f"{n_mocks} lognormal mocks, n log-uniform [2e5, 2e6], half 256^3 / half 128^3, L=1500, "
                       "CIC+interlacing, l=0,2 (device-generated catalogues)",
           "mocks_per_s": n_mocks / t, "particles_per_s": float(counts.sum()) / t, "ms_total": t * 1e3,
           "generation_s": t_gen, "lanes_per_mesh": 3}
    for N, r in zip(idx, res):
        mean, cov = covariance(r.pk.cpu().numpy(), ells_index=(0, 1))
        out[f"covariance_{N}"] = {"mocks": int(len(idx[N])), "data_vector": int(mean.size),
                                  "finite": bool(np.isfinite(cov).all())}
    # per mesh class: the batched path (lanes replaying one graph per mock) against the plain path
    # (PowerSpectrum.run, one mock at a time, no graph) on the same mocks
    from gbpowspec import PkConfig, PowerSpectrum
    from gbpowspec.batch import shell_edges

    def event_time(fn):
        fn()                                                     # warm
        torch.cuda.synchronize(dev)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize(dev)
        return a.elapsed_time(b) / 1e3

    for N in idx:
        ps = PowerSpectrum(PkConfig(n_mesh=N, box_size=box, mas="cic", interlace=True, ells=(0, 2),
                                    k_edges_kf=tuple(shell_edges(N).tolist())), dev)
        ps.reserve(cap)
        views = [arena.views(int(i)) for i in idx[N]]

        def plain():
            for v in views:
                ps.run(*v)

        t_b = event_time(lambda: runners[N].run(jobs[N]))
        t_p = event_time(plain)
        m = len(idx[N])
        out[f"class_{N}"] = {"mocks": m, "batched_mocks_per_s": m / t_b, "plain_mocks_per_s": m / t_p,
                             "batched_over_plain": t_p / t_b}
        del ps
    for r in runners.values():
        r.close()
    return out


def serving_leg(dev, seed: int, seconds: float = 10.0, rate: float = 200.0, lanes: int = 2) -> dict:
    """Serving stream: Poisson arrivals (mean `rate`/s) for `seconds`; mesh 128/256/512 w.p. 0.5/0.35/0.15,
    particle counts log-uniform [1e5, 1e7], MAS CIC or TSC, L from U[500, 2500]; 80 GB budget.
    Client data: a pool of 8 device-generated lognormal catalogues of 1e7 particles (one box each, drawn from
    U[500, 2500]) copied to pinned host memory; a request takes the first n particles of one of them."""
    import torch
    from gbpowspec.serve import Request, Server, percentiles
    from gbpowspec.synth import lognormal_catalogue_gpu
    rng = np.random.default_rng(seed)
    pool = []
    for i in range(8):
        box = float(rng.uniform(500.0, 2500.0))
        x, y, z = lognormal_catalogue_gpu(10_000_000, box, grid=256, seed=seed * 7919 + i, device=dev)
        pool.append((box, [t.cpu().pin_memory() for t in (x, y, z)]))
    torch.cuda.synchronize(dev)
    n_req = max(1, int(rng.poisson(rate * seconds)))
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n_req))
    reqs = []
    for i in range(n_req):
        box, (x, y, z) = pool[int(rng.integers(len(pool)))]
        n = int(np.exp(rng.uniform(np.log(1e5), np.log(1e7))))
        N = int(rng.choice([128, 256, 512], p=[0.5, 0.35, 0.15]))
        mas = str(rng.choice(["cic", "tsc"]))
        reqs.append(Request(x[:n], y[:n], z[:n], box=box, n_mesh=N, mas=mas))
    srv = Server(budget_bytes=80e9, lanes_per_class=lanes, capacity=10_000_000, device=dev)
    # warm every class once (lane creation and graph capture are not part of the stream)
    for N in (128, 256, 512):
        for mas in ("cic", "tsc"):
            box, (x, y, z) = pool[0]
            for _ in range(lanes):                               # every lane of the class
                srv.submit(Request(x[:1000], y[:1000], z[:1000], box=box, n_mesh=N, mas=mas))
    srv.drain(timeout=300)
    results = []
    mesh_of = {}
    t0 = time.perf_counter()
    for a, r in zip(arrivals, reqs):
        while time.perf_counter() - t0 < a:
            results.extend(srv.poll())
        mesh_of[srv.submit(r)] = r.n_mesh
    results.extend(srv.drain(timeout=300))
    t_end = time.perf_counter() - t0
    resident = srv.used
    srv.close()
    ok = [r for r in results if r.error is None]
    lat = [r.latency for r in ok]
    p = percentiles(lat)
    per_class = {}
    for N in (128, 256, 512):
        lc = [r.latency for r in ok if mesh_of.get(r.ticket) == N]
        pc = percentiles(lc)
        per_class[str(N)] = {"requests": len(lc), "p50_ms": None if pc["p50"] is None else pc["p50"] * 1e3,
                             "p99_ms": None if pc["p99"] is None else pc["p99"] * 1e3}
    return {"workload": f"Poisson arrivals {rate:g}/s for {seconds:g} s; mesh 128/256/512 (0.5/0.35/0.15); "
                        "n log-uniform [1e5, 1e7]; CIC/TSC; L in [500, 2500]; 80 GB budget",
            "requests": n_req, "completed": len(ok), "failed": len(results) - len(ok),
            "p50_ms": None if p["p50"] is None else p["p50"] * 1e3,
            "p99_ms": None if p["p99"] is None else p["p99"] * 1e3,
            "per_mesh": per_class,
            "throughput_rps": len(ok) / t_end, "particles_per_s": sum(r.n_kept for r in ok) / t_end,
            "lanes_per_class": lanes, "stream_priority": "128^3 lanes highest, 512^3 lowest",
            "resident_lanes_gb": resident / 1e9}


def extensions_leg(dev, seed: int, reps: int = 5) -> dict:
    """Milliseconds per call (median of `reps` after a warm call, CUDA events) of the reference's own call
    sequence through the drop-ins (cic_mas_vec -> delta/mean - 1 -> powspec_vec on the headline mock) and
    of the estimators beside P_l(k): xi_l(r) of a 256^3 contrast (xi_vec), the bispectrum of a 256^3 contrast at k1 = 0.1, k2 = 0.2,
    20 angles in [0, pi], L = 2500 (bispec; the reference's tests/bispec.py case), and P_l(k) forward +
    backward (gradients for 1,048,576 particle positions and weights, 256^3 TSC + interlacing)."""
    import torch
    from gbpowspec import bispectrum, power_multipoles_diff, xi_vec
    from gbpowspec.synth import lognormal_catalogue_gpu, lognormal_density
    stream = torch.cuda.current_stream(dev)

    def med_ms(fn):
        fn()
        torch.cuda.synchronize(dev)
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize(dev)
            ts.append(e0.elapsed_time(e1))
        return float(np.median(ts))

    box = 2500.0
    d = torch.from_numpy((lognormal_density(256, box, seed=seed) - 1.0).astype(np.float32)).to(dev)
    s_edges = np.arange(4.0, 200.0, 4.0).astype(np.float32)
    theta = np.linspace(0.0, np.pi, 20).astype(np.float32)
    x, y, z = lognormal_catalogue_gpu(1 << 20, box, grid=256, seed=seed, device=dev)
    w = torch.ones_like(x)
    pos = [t.clone().requires_grad_(True) for t in (x, y, z, w)]

    def grad_step():
        pk = power_multipoles_diff(*pos, box_size=box, n_mesh=256, mas="tsc", interlace=True)
        torch.nan_to_num(pk, nan=0.0).sum().backward()

    # the reference's own call sequence through the drop-ins on the headline mock (512^3, 4,194,304
    # particles): cic_mas_vec (its CIC, corner weight and all) -> delta / mean - 1 -> powspec_vec
    from gbpowspec import cic_mas_vec, powspec_vec
    xh, yh, zh = make_catalogue(seed=seed)
    xd_, yd_, zd_ = (torch.from_numpy(a).to(dev) for a in (xh, yh, zh))
    wd_ = torch.ones_like(xd_)
    N512, L = 512, float(CONFIG["box"])
    mesh0 = torch.zeros((N512, N512, N512), dtype=torch.float32, device=dev)
    kf = 2.0 * np.pi / L
    k_edges = np.arange(kf, np.pi * N512 / L, kf).astype(np.float32)

    def dropin():
        m = cic_mas_vec(mesh0, xd_, yd_, zd_, wd_, xd_.numel(), 0.0, 0.0, 0.0, L, N512, True)
        m = m / m.mean() - 1.0
        return powspec_vec(m, L, k_edges)

    t_dropin = med_ms(dropin)
    del mesh0
    # the reference's CPU-runnable case: 1,048,576 uniform particles, L = 1000, 128^3 CIC, monopole, k bins
    # of width kF from kF to k_Nyq, through the same drop-in sequence
    g1 = torch.Generator(device=dev).manual_seed(seed)
    u1 = [torch.rand(1 << 20, generator=g1, device=dev) * 1000.0 for _ in range(3)]
    w1 = torch.ones_like(u1[0])
    mesh1 = torch.zeros((128, 128, 128), dtype=torch.float32, device=dev)
    kf1 = 2.0 * np.pi / 1000.0
    edges1 = np.arange(kf1, np.pi * 128 / 1000.0, kf1).astype(np.float32)

    def config1():
        m = cic_mas_vec(mesh1, *u1, w1, u1[0].numel(), 0.0, 0.0, 0.0, 1000.0, 128, True)
        m = m / m.mean() - 1.0
        return powspec_vec(m, 1000.0, edges1)

    t_config1 = med_ms(config1)
    del mesh1, u1, w1
    # config 3's mesh: 1024^3, 16,777,216 lognormal particles, PCS + interlacing, P_0,2,4 (production path)
    from gbpowspec import PkConfig, PowerSpectrum
    torch.cuda.empty_cache()
    x3, y3, z3 = lognormal_catalogue_gpu(1 << 24, 2500.0, grid=256, seed=seed + 3, device=dev)
    ps3 = PowerSpectrum(PkConfig(n_mesh=1024, box_size=2500.0, mas="pcs", interlace=True), dev)
    ps3.reserve(x3.numel())
    t_config3 = med_ms(lambda: ps3.run(x3, y3, z3))
    del ps3, x3, y3, z3
    torch.cuda.empty_cache()
    return {"dropin_cic_mas_vec_powspec_vec_512_ms": t_dropin,
            "config1_uniform_1M_128_cic_dropin_ms": t_config1,
            "config3_1024_pcs_interlaced_16M_ms": t_config3,
            "xi_vec_256_ms": med_ms(lambda: xi_vec(d, box, s_edges)),
            "bispec_256_20_angles_ms": med_ms(lambda: bispectrum(d, box, 0.1, 0.2, theta)),
            "power_grad_256_tsc_interlaced_1M_particles_ms": med_ms(grad_step)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10, help="timed batches")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=16, help="mocks per batch (step)")
    ap.add_argument("--lanes", type=int, default=0, help="lanes for the batched path (0 = tune among 1..3)")
    ap.add_argument("--plain-steps", type=int, default=60)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--n-mesh", type=int, default=None, help="override the mesh side (profiling cases)")
    ap.add_argument("--n-particles", type=int, default=None, help="override the particle count")
    ap.add_argument("--no-covariance", action="store_true", help="skip the batched covariance leg")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving leg")
    ap.add_argument("--no-extensions", action="store_true", help="skip the xi / bispectrum / gradient timings")
    ap.add_argument("--serve-seconds", type=float, default=10.0)
    ap.add_argument("--serve-lanes", type=int, default=2, help="resident lanes per request class")
    ap.add_argument("--profile-only", action="store_true",
                    help="plain path only, warm-up + timed steps (no other legs): a short command for ncu")
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
    from gbpowspec.batch import BatchRunner, ParticleArena, tune_lanes

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if ws > 1:
            dist.barrier()

    x, y, z = make_catalogue(seed=1000 + rank)
    n = x.size
    host = [torch.from_numpy(a).pin_memory() for a in (x, y, z)]
    xd, yd, zd = (h.to(dev) for h in host)
    cfg = PkConfig(n_mesh=CONFIG["n_mesh"], box_size=CONFIG["box"], mas=CONFIG["mas"],
                   interlace=CONFIG["interlace"], ells=CONFIG["ells"])
    N, G = cfg.n_mesh, cfg.grids
    ps = PowerSpectrum(cfg, dev, tiles="auto")          # the autotuner's column tile for this shape
    ps.reserve(n)
    stream = torch.cuda.current_stream(dev)

    def timed(fn, steps):
        barrier()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        barrier()
        return e0.elapsed_time(e1) / 1e3

    # ---- plain path: one mock at a time, resident buffers, no graph
    for _ in range(args.warmup):
        ps.run(xd, yd, zd)
    if args.profile_only:
        t = timed(lambda: ps.run(xd, yd, zd), args.steps)
        if rank == 0:
            print(json.dumps({"profile_only": True, "ms_per_step": t / args.steps * 1e3, "config": _cfg_json()}),
                  flush=True)
        if ws > 1:
            dist.destroy_process_group()
        return
    t_plain = timed(lambda: ps.run(xd, yd, zd), args.plain_steps)

    # ---- per-kernel trace of a few plain mocks (CUDA events around every launch)
    kernels = trace_breakdown(ps, xd, yd, zd, reps=5, n=n)

    # ---- batched path: B mocks per step (two distinct catalogues, each mock its own slice of the arena)
    B = args.batch
    x2, y2, z2 = make_catalogue(seed=2000 + rank)
    cats = [(x, y, z) if i % 2 == 0 else (x2, y2, z2) for i in range(B)]
    arena = ParticleArena(cats, device=dev)
    arena.upload()
    jobs = arena.job_table(cfg.box_size, N)
    kw = dict(capacity=n, mas=cfg.mas, interlace=cfg.interlace, ells=cfg.ells, kedges_grid=cfg.kedges_grid())
    lane_rates = None
    if args.lanes > 0:
        lanes = args.lanes
    else:
        lanes, lane_rates = tune_lanes(N, jobs, candidates=(1, 2, 3), repeats=1, **kw)
    runner = BatchRunner(N, n_lanes=lanes, device=dev, **kw)
    from gbpowspec.tune import default_tuner
    tune_rec = default_tuner().entry(N, cfg.mas, cfg.interlace, n=n, device=dev)
    res = runner.alloc_result(B)
    for _ in range(args.warmup):
        runner.run(jobs, res)
    clocks = ClockSampler(local)
    clocks.start()
    t_batch = timed(lambda: runner.run(jobs, res), args.steps)
    clk = clocks.stop()

    # ---- end to end through the batched API: pinned host particles -> device, P_l back to host
    pk_host = torch.empty(res.pk.shape, dtype=res.pk.dtype, pin_memory=True)

    def e2e_step():
        runner.run_from_host(arena, jobs, res)   # pinned H2D chunk by chunk, overlapping the lanes' work
        pk_host.copy_(res.pk, non_blocking=True)

    for _ in range(2):
        e2e_step()
    clocks_e2e = ClockSampler(local)
    clocks_e2e.start()
    t_e2e = timed(e2e_step, args.steps)
    clk_e2e = clocks_e2e.stop()
    # the host-to-device link on its own (the arena's copies with nothing else running)
    t_h2d = timed(arena.upload, 3) / 3

    # the whole job ends when the slowest rank does
    from gbpowspec.replicas import max_over_ranks
    t_batch, t_e2e, t_plain = max_over_ranks([t_batch, t_e2e, t_plain])

    extra = {}
    if not args.no_covariance:
        extra["batched_covariance"] = covariance_leg(dev, seed=3000 + rank)
    if not args.no_serve:
        extra["serving"] = serving_leg(dev, seed=4000 + rank, seconds=args.serve_seconds, lanes=args.serve_lanes)
    if not args.no_extensions:
        extra["extensions"] = extensions_leg(dev, seed=5000 + rank)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        t_cpu = cpu_reference_mock(x, y, z)
        cpu = {"value": 1.0 / t_cpu, "unit": "mocks/s", "cores": cpu_cores(), "kind": "port",
               "sample": CPU_SAMPLE.replace(" per step", "")}

    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    # the dominant kernel is the one with the most time per mock; every kernel with an algorithmic
    # byte count is reported beside it
    dom = max(kernels, key=lambda k: kernels[k]["ms_per_mock"])
    if "algorithmic_bytes" not in kernels[dom]:
        raise RuntimeError(f"the dominant kernel {dom} has no algorithmic byte count")
    ach = kernels[dom]["achieved_gbs"]
    traffic = PROFILED_TRAFFIC.get((dom, N, n))
    per_kernel_roofline = {k: {"achieved_gbs": v["achieved_gbs"], "frac": v["achieved_gbs"] / peak,
                               "algorithmic_bytes": v["algorithmic_bytes"], "ms_per_mock": v["ms_per_mock"],
                               "traffic": PROFILED_TRAFFIC.get((k, N, n))}
                           for k, v in kernels.items() if "algorithmic_bytes" in v}

    mocks = ws * args.steps * B
    per_mock_launches = sum(v["launches_per_mock"] for v in kernels.values())
    line = {
        "metric": METRIC, "value": mocks / t_batch, "unit": "mocks/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_batch / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded lognormal+RSD mocks)",
        "config": {**_cfg_json(), "path": f"batched: {B} mocks per step over {lanes} lanes (one CUDA graph "
                                          "replay per mock, lanes on their own streams)",
                   "batch": B, "lanes": lanes, "lane_tuning_mocks_per_s": lane_rates,
                   "column_tile": "%dx%d" % runner.tiles if runner.tiles else None,
                   "column_tile_tuning_ms_per_mock": (tune_rec or {}).get("ms")},
        "particles_per_s": mocks * n / t_batch,
        "plain": {"value": ws * args.plain_steps / t_plain, "unit": "mocks/s", "steps": args.plain_steps,
                  "ms_per_mock": t_plain / args.plain_steps * 1e3,
                  "path": "PowerSpectrum.run, one mock at a time, no graph"},
        "batched_over_plain": (mocks / t_batch) / (ws * args.plain_steps / t_plain),
        "kernels": kernels,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": peak, "unit": "GB/s",
                     "frac": ach / peak, "traffic": traffic,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback 6800 GB/s",
                     "algorithmic_bytes": kernels[dom]["algorithmic_bytes"], "per_kernel": per_kernel_roofline},
        "pipeline_roofline": {"algorithmic_bytes_per_mock": algorithmic_bytes(n, N, G),
                              "frac": algorithmic_bytes(n, N, G) * mocks / ws / t_batch / 1e9 / peak},
        "cpu_baseline": cpu,
        "e2e": {"value": mocks / t_e2e, "unit": "mocks/s", "h2d_bytes_per_step": arena.nbytes,
                "d2h_bytes_per_step": int(pk_host.numel() * 8),
                "h2d_alone_gbs": arena.nbytes / t_h2d / 1e9, "clocks": clk_e2e,
                "path": "BatchRunner.run_from_host (pinned H2D of every mock, chunk by chunk on a copy stream "
                        "overlapping the lanes) + P_l D2H"},
        # per mock: the traced stages (the scan stage is two cub kernels) + lane_begin + lane_end; per batch
        # call: one descriptor kernel per lane
        "gpu_launches": int(round(per_mock_launches + 1 + 2)) * args.steps * B + lanes * args.steps,
        "clocks": clk,
        **extra,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


# DRAM bytes (read + write) per launch from one ncu capture of the same kernels
# (--set full, --clock-control none) on 512^3 with 1,048,576 particles,
# keyed by (kernel, mesh, particles).  The y pass and the x pass + binning
# move only spectra, so their traffic does not depend on the particle count.
# The deposit/z kernel writes the z-transformed spectra (1.048 GB, particle
# independent) and reads its bucket entries (0.037 GB at 1,048,576
# particles, in proportion to the particles): 1.047 + 4 x 0.037 GB for the
# 4,194,304-particle workload.
# The one-pass bucketing's entries are still in L2 when it ends (their DRAM
# writes fall in the deposit/z kernel's window), so it gets no figure.
PROFILED_TRAFFIC = {
    ("deposit_fft_z", 512, 4_194_304): 1_046_520_000 + 4 * 37_453_000,
    ("fft_y", 512, 4_194_304): 1_107_458_000 + 1_053_273_000,
    ("fft_x_bins", 512, 4_194_304): 1_107_381_000 + 5_776_000,
}


if __name__ == "__main__":
    main()
