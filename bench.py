"""Benchmark: batched planet generation (planets/s) on GB300.

Workload (default): 64 planets, seeds 0..63, divisions uniform in [100, 800],
octaves uniform in [4, 12], erosion iterations uniform in [0, 100]
(numpy default_rng(7), drawn in that order); fBm base frequency 1,
lacunarity 2, persistence 0.5, heights rescaled to +-8000 m, erosion from
water 1e-3 m and sediment 0.  Meshes are resident in HBM (built before the
timed region); one step = the whole batch, replayed as one CUDA graph.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  `--impl reference` times the reference's CPU
path (the oracle port: C restatement, OpenMP over the host cores) on the
same workload, each step a bounded sample of planets.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_PLANETS = 64
METRIC = "batched planets/s (64 planets, divisions 100-800, 4-12 octaves, 0-100 erosion iterations)"
UNIT = "planets/s"
SAMPLE_ALG_BYTES = 72      # erosion: algorithmic bytes per vertex-iteration (state 12+12, neighbours 24, edges 24)


def workload(name="batch64"):
    """The benchmark's planets.  `small` (8 planets, divisions 100-300, same
    draws otherwise) is the case the ncu captures use."""
    from nixis_gb300.planets import PlanetRequest
    rng = np.random.default_rng(7)
    divs = rng.integers(100, 801, N_PLANETS)
    octs = rng.integers(4, 13, N_PLANETS)
    iters = rng.integers(0, 101, N_PLANETS)
    reqs = [PlanetRequest(seed=i, divisions=int(divs[i]), octaves=int(octs[i]), erosion_iters=int(iters[i]))
            for i in range(N_PLANETS)]
    if name == "small":
        reqs = [PlanetRequest(seed=r.seed, divisions=100 + (r.divisions - 100) * 200 // 700, octaves=r.octaves,
                              erosion_iters=r.erosion_iters) for r in reqs[:8]]
    return reqs


def config(reqs):
    nv = sum(r.n_vertices for r in reqs)
    what = ("batched planets: 64 x (divisions U[100,800], octaves U[4,12], erosion iterations U[0,100]), "
            "seeds 0..63, default_rng(7)") if len(reqs) == N_PLANETS else \
        f"profiling case: {len(reqs)} planets, divisions 100-300, same draws"
    return {"workload": what,
            "planets": len(reqs), "vertices": nv,
            "vertex_octaves": sum(r.n_vertices * r.octaves for r in reqs),
            "vertex_iterations": sum(r.n_vertices * r.erosion_iters for r in reqs),
            "l2": "working set > L2 (no flush needed)", "parallelism": "replicas"}


# ---------------------------------------------------------------------------
# clocks

class ClockSampler:
    """nvidia-smi samples during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# distributed (replicas)

def dist_setup(n_gpus):
    import torch
    if n_gpus <= 1 or "RANK" not in os.environ:
        return 0, 1, None
    import torch.distributed as dist
    rank = int(os.environ["RANK"])
    world = int(os.environ["WORLD_SIZE"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    torch.cuda.set_device(local)
    dist.init_process_group("nccl")
    return rank, world, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, value):
    """Largest value over ranks (the job's wall time)."""
    if dist is None:
        return value
    import torch
    dev = "cpu" if dist.get_backend() == "gloo" else "cuda"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
# CPU reference (oracle port)

def cpu_planet(req, xyz, nbr):
    """One planet on the CPU with the reference's functions (sample_octaves,
    rescale, erosion_iteration3 x iters) restated in C, binary64.  Returns
    (noise seconds, erosion seconds)."""
    from oracle import oracle as O
    t0 = time.perf_counter()
    perm, pgi = O.init(req.seed)
    e = O.sample_octaves(xyz, None, perm, pgi, req.octaves, req.init_roughness, req.init_strength, req.roughness,
                         req.persistence, req.radius)
    h = O.rescale(e, req.elev_lo, req.elev_hi)
    t1 = time.perf_counter()
    w = np.full(len(xyz), req.water0)
    s = np.zeros(len(xyz))
    for _ in range(req.erosion_iters):
        O.erosion_iteration3(xyz, nbr, h, w, s)
    t2 = time.perf_counter()
    return t1 - t0, t2 - t1


def cpu_meshes(reqs):
    """Meshes for the CPU runs, built on the CPU (input preparation, not
    timed): the same icosphere layout and the reference's adjacency."""
    from oracle import oracle as O
    out = {}
    for r in reqs:
        if r.divisions not in out:
            out[r.divisions] = O.planet_mesh(r.divisions)
    return out


def cpu_sample(reqs, count):
    """A spread of the batch: `count` planets at equal strides (request order)."""
    step = max(1, len(reqs) // count)
    return list(range(0, len(reqs), step))[:count]


class CpuRates:
    """Seconds per vertex-octave (noise) and per vertex-iteration (erosion)
    measured on sampled planets; the full batch's CPU time is extrapolated
    from them."""

    def __init__(self):
        self.tn = self.te = 0.0
        self.vo = self.vi = 0

    def add(self, req, tn, te):
        self.tn += tn
        self.te += te
        self.vo += req.n_vertices * req.octaves
        self.vi += req.n_vertices * req.erosion_iters

    def batch_seconds(self, reqs):
        rn = self.tn / max(self.vo, 1)
        re = self.te / max(self.vi, 1)
        return sum(r.n_vertices * r.octaves for r in reqs) * rn + sum(r.n_vertices * r.erosion_iters for r in reqs) * re


def run_cpu_baseline(reqs, budget_s=15.0):
    from oracle import oracle as O
    idx = cpu_sample(reqs, 8)
    meshes = cpu_meshes([reqs[i] for i in idx])
    rates = CpuRates()
    t0 = time.perf_counter()
    done = []
    for i in idx:
        tn, te = cpu_planet(reqs[i], *meshes[reqs[i].divisions])
        rates.add(reqs[i], tn, te)
        done.append(i)
        if time.perf_counter() - t0 > budget_s:
            break
    T = rates.batch_seconds(reqs)
    return {"value": len(reqs) / T, "unit": UNIT, "cores": O.num_threads(), "kind": "port",
            "sample": f"planets {done} of the 64 run in full ({time.perf_counter() - t0:.1f} s); the batch's CPU "
                      f"time extrapolated from their seconds per vertex-octave ({1e9 * rates.tn / max(rates.vo, 1):.2f} ns)"
                      f" and per vertex-iteration ({1e9 * rates.te / max(rates.vi, 1):.2f} ns); C restatement "
                      f"(binary64, OpenMP) of sample_octaves + rescale + erosion_iteration3"}


def bench_reference(args):
    """--impl reference: the CPU path alone; each step runs 2 sampled
    planets in full and the batch rate is extrapolated per unit of work."""
    from oracle import oracle as O
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    reqs = workload()
    idx = cpu_sample(reqs, 16)
    meshes = cpu_meshes([reqs[i] for i in idx])
    for w in range(args.warmup):
        i = idx[w % len(idx)]
        cpu_planet(reqs[i], *meshes[reqs[i].divisions])
    rates = CpuRates()
    t0 = time.perf_counter()
    for s in range(args.steps):
        for q in range(2):
            i = idx[(2 * s + q) % len(idx)]
            tn, te = cpu_planet(reqs[i], *meshes[reqs[i].divisions])
            rates.add(reqs[i], tn, te)
    wall = time.perf_counter() - t0
    T = rates.batch_seconds(reqs)
    v = len(reqs) / T
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * wall / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "config": config(reqs), "impl": "reference",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": O.num_threads(), "kind": "port",
                             "sample": "each step runs 2 of 16 evenly spaced planets of the batch in full; the batch "
                                       "time is extrapolated from the measured seconds per vertex-octave "
                                       f"({1e9 * rates.tn / max(rates.vo, 1):.2f} ns) and per vertex-iteration "
                                       f"({1e9 * rates.te / max(rates.vi, 1):.2f} ns); C restatement (binary64, "
                                       "OpenMP) of the reference's functions"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# GPU

def bench_ours(args):
    import torch
    from nixis_gb300 import mesh, planets, _lib

    rank, world, dist = dist_setup(args.gpus)
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    reqs = workload(args.workload)
    npl = len(reqs)
    cache = mesh.MeshCache()
    for r in reqs:
        cache.get(r.divisions)
    torch.cuda.synchronize()
    batch = planets.PlanetBatch(reqs, cache)
    if args.profile:
        # one eager run of the batch (what the ncu captures record), then exit
        batch.launch()
        torch.cuda.synchronize()
        if rank == 0:
            print(json.dumps({"profile_run": args.workload, "kernels": batch.kernels_per_run(),
                              "erosion_launches": batch.max_iters, "config": config(reqs)}))
        return
    if args.eager:
        batch.launch()
    else:
        batch.capture()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()

    # warm-up, then K timed steps bracketed by barrier + sync
    for _ in range(args.warmup):
        batch.run()
    torch.cuda.synchronize()
    barrier(dist)
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        batch.run()
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier(dist)
    ms = e0.elapsed_time(e1)
    ms = max_over_ranks(dist, ms)
    value = world * npl * args.steps / (ms / 1e3)

    # erosion stage alone (the dominant kernel): algorithmic bytes / time
    peak, peak_kind = measured_peak()
    import ctypes
    from nixis_gb300 import _dev
    s = _dev.stream_handle()
    np_ = len(reqs)
    batch.launch()
    torch.cuda.synchronize()
    call = _lib.call
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    batch.minmax.copy_(batch.minmax0)
    ev[0].record(stream)
    call("nx_fbm_batch", _dev.ptr(batch.fb_dev), ctypes.cast(batch.fb_host, ctypes.c_void_p), np_, None, s)
    ev[1].record(stream)
    call("nx_erosion_init_batch", _dev.ptr(batch.er_dev), ctypes.cast(batch.er_host, ctypes.c_void_p), np_,
         _dev.ptr(batch.raw), _dev.ptr(batch.minmax), ctypes.c_float(-8000.0), ctypes.c_float(8000.0),
         ctypes.c_float(1e-3), _dev.ptr(batch.st), _dev.ptr(batch.st_tmp), s)
    call("nx_erosion_ctl_init", _dev.ptr(batch.ws), batch.ws.numel(), np_, s)
    ev[2].record(stream)
    call("nx_erosion_batch", _dev.ptr(batch.er_dev), ctypes.cast(batch.er_host, ctypes.c_void_p), np_,
         _dev.ptr(batch.st), _dev.ptr(batch.st_tmp), None, _dev.ptr(batch.ws), batch.ws.numel(), s)
    ev[3].record(stream)
    torch.cuda.synchronize()
    ero_ms = ev[2].elapsed_time(ev[3])
    fbm_ms = ev[0].elapsed_time(ev[1])
    vit = sum(r.n_vertices * r.erosion_iters for r in reqs)
    alg = vit * SAMPLE_ALG_BYTES
    achieved = alg / (ero_ms / 1e3) / 1e9
    n_launch = batch.erosion_launches()
    blocked = any(batch.er_host[j].tiling for j in range(np_))
    ero_kernel = "erosion_tb_kernel" if blocked else "erosion_step_kernel"
    roofline = {"bound": "hbm", "kernel": ero_kernel, "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                "alg_bytes_per_vertex_iteration": SAMPLE_ALG_BYTES, "launches": n_launch,
                "alg_bytes_per_launch": alg / max(n_launch, 1), "avg_launch_ms": ero_ms / max(n_launch, 1),
                "traffic": None, "fbm_ms": fbm_ms, "erosion_ms": ero_ms}
    prof = os.path.join(ROOT, "profiles", "erosion_traffic.json")
    if os.path.exists(prof):
        try:
            with open(prof) as f:
                tr = json.load(f)
            roofline["traffic"] = tr["bytes_per_vertex_iteration"] * vit / max(n_launch, 1)
            roofline["traffic_source"] = tr.get("source")
        except (OSError, KeyError, ValueError):
            pass

    # plain per-planet path on the same planets
    torch.cuda.synchronize()
    for r in reqs[:2]:
        planets.generate_plain(r, cache)
    t0 = time.perf_counter()
    for r in reqs:
        planets.generate_plain(r, cache)
    torch.cuda.synchronize()
    plain_s = time.perf_counter() - t0
    plain = {"value": npl / plain_s, "unit": UNIT,
             "what": "one planet at a time, one launch per octave and per erosion iteration, synchronised per planet"}

    # end to end: per step, request tables host->device, batch, heights device->host (pinned)
    host_tab = torch.empty_like(batch.tables, device="cpu").pin_memory()
    host_tab.copy_(batch.tables)
    host_out = torch.empty(batch.heights.numel(), dtype=torch.float32).pin_memory()
    for _ in range(2):
        batch.tables.copy_(host_tab, non_blocking=True)
        batch.run()
        host_out.copy_(batch.heights, non_blocking=True)
    torch.cuda.synchronize()
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        batch.tables.copy_(host_tab, non_blocking=True)
        batch.run()
        host_out.copy_(batch.heights, non_blocking=True)
        torch.cuda.synchronize()
    e2e_s = max_over_ranks(dist, time.perf_counter() - t0)
    e2e = {"value": world * npl * args.steps / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": int(batch.tables.numel() * 4), "d2h_bytes_per_step": int(batch.heights.numel() * 4),
           "note": "request tables in, all heights out to pinned host memory, per step"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = run_cpu_baseline(reqs, budget_s=args.cpu_budget)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config(reqs),
                "plain_per_planet": plain, "ratio_vs_plain": value / (plain["value"] * world),
                "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clk,
                "gpu_launches": batch.kernels_per_run() * args.steps}
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--workload", choices=["batch64", "small"], default="batch64")
    ap.add_argument("--eager", action="store_true", help="launch without a CUDA graph (for profilers)")
    ap.add_argument("--profile", action="store_true", help="build the batch, run it once eagerly, exit (ncu)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        bench_reference(args)
    else:
        bench_ours(args)


if __name__ == "__main__":
    main()
