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
SAMPLE_ALG_BYTES = 72      # erosion: algorithmic bytes per vertex-iteration, the binary32 model (state 12 in +
                           # 12 out, neighbour ids 24, edge lengths 24); the pair state and edge lengths used
                           # here would count 120


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
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
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
    # blocked-erosion setting: autotuned on this device (before anything is timed)
    from nixis_gb300 import autotune
    tune_t0 = time.perf_counter()
    if args.tb or args.profile:
        # profiler runs launch nothing but the batch: a given or the default setting
        tb = autotune.parse(args.tb) if args.tb else autotune.DEFAULT
        autotune.use(tb)
        tune_info = {"setting": tb.label, "source": "given" if args.tb else "default"}
    else:
        tb, timings = autotune.tune(save=False)
        tune_info = {"setting": tb.label, "source": "autotuned",
                     "candidates_ms": timings, "seconds": round(time.perf_counter() - tune_t0, 2)}
    if args.tune_only:
        if rank == 0:
            print(json.dumps({"autotune": tune_info}))
        return
    cache = mesh.MeshCache()
    for r in reqs:
        cache.get(r.divisions)
    torch.cuda.synchronize()
    batch = planets.PlanetBatch(reqs, cache, blocked=not args.no_blocked)
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
    call("nx_erosion_ctl_init", _dev.ptr(batch.ws), batch.ws.numel(), np_, s)
    ev[2].record(stream)
    # the erosion stage as the batch runs it: the blocked passes with the
    # rescale fused into each planet's first pass and the heights into its last
    r0 = reqs[0]
    call("nx_erosion_run_batch", _dev.ptr(batch.er_dev), ctypes.cast(batch.er_host, ctypes.c_void_p), np_,
         _dev.ptr(batch.raw), _dev.ptr(batch.minmax), float(r0.elev_lo), float(r0.elev_hi), float(r0.water0),
         _dev.ptr(batch.st), _dev.ptr(batch.st_tmp), _dev.ptr(batch.heights), _dev.ptr(batch.ws),
         batch.ws.numel(), s)
    ev[3].record(stream)
    # the heights kernel that ends the stage, alone (the same launch again)
    hev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    hev[0].record(stream)
    call("nx_erosion_heights_batch", _dev.ptr(batch.er_dev), ctypes.cast(batch.er_host, ctypes.c_void_p), np_,
         _dev.ptr(batch.st), _dev.ptr(batch.ws), _dev.ptr(batch.heights), s)
    hev[1].record(stream)
    torch.cuda.synchronize()
    ero_ms = ev[2].elapsed_time(ev[3])
    heights_ms = hev[0].elapsed_time(hev[1])
    fbm_ms = ev[0].elapsed_time(ev[1])
    vit = sum(r.n_vertices * r.erosion_iters for r in reqs)
    alg = vit * SAMPLE_ALG_BYTES
    # the erosion passes: the stage less its closing heights kernel
    passes_ms = ero_ms - heights_ms
    achieved = alg / (passes_ms / 1e3) / 1e9
    n_launch = batch.erosion_launches()
    blocked = any(batch.er_host[j].tiling for j in range(np_))
    ero_kernel = "erosion_tb_kernel" if blocked else "erosion_step_kernel"
    roofline = {"bound": "hbm", "kernel": ero_kernel, "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                "alg_bytes_per_vertex_iteration": SAMPLE_ALG_BYTES, "launches": n_launch,
                "alg_bytes_per_launch": alg / max(n_launch, 1), "avg_launch_ms": passes_ms / max(n_launch, 1),
                "traffic": None, "fbm_ms": fbm_ms, "erosion_ms": ero_ms, "erosion_passes_ms": passes_ms,
                "heights_ms": heights_ms,
                "stage_note": "erosion_ms: the rescale (fused into each planet's first pass), the passes and the "
                              "heights kernel; the roofline divides by the passes alone (erosion_ms - heights_ms)"}
    # every kernel of the path against its own roofline
    sm_mhz = clk.get("sm_mhz") or 2070.0
    fp32_fma = fp32_peak_tflops(sm_mhz)
    vo = sum(r.n_vertices * r.octaves for r in reqs)
    fbm_tf = vo * FBM_ALG_FLOP / (fbm_ms / 1e3) / 1e12
    kernels = {
        ero_kernel: {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "model": f"{SAMPLE_ALG_BYTES} B per vertex-iteration x {vit} vertex-iterations"},
        "fbm_batch_kernel": {"bound": "fp32", "achieved": fbm_tf, "peak": fp32_fma, "unit": "TFLOP/s",
                             "frac": fbm_tf / fp32_fma, "ms": fbm_ms,
                             "model": f"{FBM_ALG_FLOP} FLOP per vertex-octave (the reference's binary64 operations) x "
                                      f"{vo} vertex-octaves; peak = 152 SMs x 128 lanes x 2 x {sm_mhz:.0f} MHz (derived)",
                             "note": "evaluated in float-float pairs (~2.4x the binary32 kernel's instructions) to stay "
                                     "within 1e-13 of binary64, which the erosion's flow choices need"}}
    issue = os.path.join(ROOT, "profiles", "fbm_issue.json")
    if os.path.exists(issue):
        # executed instructions against the issue peak (152 SMs x 4
        # schedulers x 32 lanes per clock): what the pair arithmetic costs
        try:
            with open(issue) as f:
                ipv = float(json.load(f)["thread_instructions_per_vertex_octave"])
            rate = vo * ipv / (fbm_ms / 1e3)
            kernels["fbm_batch_kernel"]["executed"] = {
                "thread_instructions_per_vertex_octave": ipv, "tinst_per_s": rate,
                "issue_frac": rate / (152 * 4 * 32 * sm_mhz * 1e6),
                "source": "instruction count from the ncu capture in profiles/fbm_batch_small.md"}
        except (OSError, KeyError, ValueError):
            pass
    inso = measure_insolation(sm_mhz)
    if inso:
        kernels["insolation_kernel"] = inso
    roofline["kernels"] = kernels
    prof = os.path.join(ROOT, "profiles", "erosion_traffic.json")
    if os.path.exists(prof):
        try:
            with open(prof) as f:
                tr = json.load(f)
            roofline["traffic"] = tr["bytes_per_vertex_iteration"] * vit / max(n_launch, 1)
            roofline["traffic_source"] = tr.get("source")
        except (OSError, KeyError, ValueError):
            pass

    # plain per-planet paths on the same planets: one launch per erosion
    # iteration (the comparator), and one per blocked pass (the same erosion
    # kernel as the batch, so the ratio isolates batching)
    plains = {}
    for key, blocked in (("plain", False), ("plain_blocked", True)):
        torch.cuda.synchronize()
        for r in reqs[:2]:
            planets.generate_plain(r, cache, blocked=blocked)
        t0 = time.perf_counter()
        for r in reqs:
            planets.generate_plain(r, cache, blocked=blocked)
        torch.cuda.synchronize()
        plains[key] = npl / (time.perf_counter() - t0)
    plain = {"value": plains["plain"], "unit": UNIT,
             "what": "one planet at a time, one launch per octave and per erosion iteration, synchronised per planet"}
    plain_blocked = {"value": plains["plain_blocked"], "unit": UNIT,
                     "what": "one planet at a time, one launch per octave and per blocked erosion pass (the batch's "
                             "erosion kernel), synchronised per planet"}
    # (outside the timed regions) every batched planet equals the planet generated alone
    res = batch.results()
    plain["batch_equals_plain"] = bool(all(torch.equal(a.heights, planets.generate_plain(r, cache).heights)
                                           for r, a in zip(reqs, res)))
    del res
    errors = errors_vs_binary64(batch, reqs, cache) if (rank == 0 and not args.no_cpu) else None

    # end to end: per step, request tables host->device, batch, heights device->host (pinned)
    host_tab = torch.empty_like(batch.tables, device="cpu").pin_memory()
    host_tab.copy_(batch.tables)
    host_out = torch.empty(batch.heights.numel(), dtype=torch.float64).pin_memory()
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
    serial_s = max_over_ranks(dist, time.perf_counter() - t0)
    # the same copies pipelined through the public API: a step's heights go to
    # the host on a side stream while the next step runs (PlanetBatch.run_to_host)
    for _ in range(2):
        batch.tables.copy_(host_tab, non_blocking=True)
        batch.run_to_host(host_out)
    batch.wait_host()
    torch.cuda.synchronize()
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        batch.tables.copy_(host_tab, non_blocking=True)
        batch.run_to_host(host_out)
    batch.wait_host()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(dist, time.perf_counter() - t0)
    e2e = {"value": world * npl * args.steps / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": int(batch.tables.numel() * 4), "d2h_bytes_per_step": int(batch.heights.numel() * 8),
           "note": "request tables in, all heights out to pinned host memory, every step; each step's heights are "
                   "copied on a side stream while the next step runs (PlanetBatch.run_to_host), all copies complete "
                   "inside the timed region",
           "serial_value": world * npl * args.steps / serial_s,
           "serial_note": "the same with a host synchronisation after every step's copy (no overlap)"}

    launches = batch.kernels_per_run() * args.steps
    serving = None
    if rank == 0 and world == 1 and args.serve_requests > 0:
        # the serving leg starts from an empty device: the batch's state and
        # its 59 resident meshes (tens of GB) are released first
        del batch, cache, host_out, host_tab
        import gc
        gc.collect()
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        serving = run_serving(args.serve_requests)

    # single-planet configurations with per-field errors against binary64
    # (divisions 250 / 8 octaves; divisions 1000 / 12 octaves + 50 erosion
    # iterations), outside every timed region
    singles = None
    if rank == 0 and world == 1 and not args.no_cpu and not args.no_single:
        import gc
        gc.collect()
        torch.cuda.empty_cache()
        singles = {c: single_planet(c) for c in ("c1", "c2")}

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = run_cpu_baseline(reqs, budget_s=args.cpu_budget)

    if rank == 0:
        if "candidates_ms" in tune_info:          # the five fastest settings
            best = sorted(tune_info["candidates_ms"].items(), key=lambda kv: kv[1])[:5]
            tune_info = dict(tune_info, candidates_ms=dict(best), candidates=len(tune_info["candidates_ms"]))
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config(reqs),
                "gpu_launches": launches, "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clk,
                "blocked_erosion": tune_info, "serving": serving,
                "plain_per_planet": plain, "plain_blocked_per_planet": plain_blocked,
                "ratio_vs_plain": value / (plain["value"] * world),
                "ratio_vs_plain_blocked": value / (plain_blocked["value"] * world),
                "errors_vs_fp64": errors, "single_planets": singles}
        # the figures a reader needs first, last on the line and compact
        line["summary"] = summary(line)
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def summary(line):
    """Compact digest of the line's comparisons: batch vs the plain paths,
    serving (p50/p99, planets/s, results equal), errors against binary64,
    every kernel's roofline fraction."""
    g = lambda x, n=4: None if x is None else float(f"{x:.{n}g}")
    out = {"planets_per_s": g(line["value"]), "e2e": g(line["e2e"]["value"]),
           "plain": g(line["plain_per_planet"]["value"]), "plain_blocked": g(line["plain_blocked_per_planet"]["value"]),
           "ratio_vs_plain": g(line["ratio_vs_plain"], 3), "ratio_vs_plain_blocked": g(line["ratio_vs_plain_blocked"], 3),
           "batch_equals_plain": line["plain_per_planet"].get("batch_equals_plain")}
    rf = line.get("roofline") or {}
    ks = rf.get("kernels") or {}
    out["roofline_frac"] = {k: g(v.get("frac"), 3) for k, v in ks.items()}
    # what the compute-bound kernels issue against the issue peak
    issue = {k: g((v.get("executed") or {}).get("issue_frac"), 3) for k, v in ks.items()
             if (v.get("executed") or {}).get("issue_frac") is not None}
    issue.update({k: g(v.get("frac"), 3) for k, v in ks.items() if v.get("bound") == "issue"})
    if issue:
        out["issue_frac"] = issue
    sv = line.get("serving")
    if sv:
        out["serving"] = {"requests": sv["requests"]}
        for mode in ("arrivals", "all_at_once"):
            m = sv[mode]
            out["serving"][mode] = {p: [g(m[p]["p50_ms"]), g(m[p]["p99_ms"]), g(m[p]["planets_per_s"])]
                                    for p in ("engine", "plain")}
            out["serving"][mode]["equal"] = m["results_equal_plain"]
        out["serving"]["fields"] = "[p50 ms, p99 ms, planets/s]"
    er = line.get("errors_vs_fp64")
    if er:
        out["batch_vs_fp64_max_rel_h"] = g(er["max_rel_h"], 3)
    sp = line.get("single_planets")
    if sp:
        c1, c2 = sp.get("c1") or {}, sp.get("c2") or {}
        out["c1_elevation_max_err_m"] = g(c1.get("elevation_max_err_m"), 3)
        e50 = (c2.get("erosion_errors") or {}).get(50)
        if e50:
            out["c2_50_iters_vs_fp64"] = {f: [g(e50[f]["max_abs_over_max"], 3), g(e50[f]["rms_over_max"], 3)]
                                          for f in "hws"}
            out["c2_50_iters_vs_fp64"]["fields"] = "[max, rms] / max|field|"
            out["c2_flow_choice_flips"] = e50.get("flow_choice_flips")
    return out


def fp32_peak_tflops(sm_mhz, fma=True):
    """GB300 binary32 peak from its shape: 152 SMs x 128 lanes x (2 FLOP per
    fused multiply-add | 1 op) per clock, at the sampled SM clock."""
    return 152 * 128 * (2 if fma else 1) * sm_mhz * 1e6 / 1e12


FBM_ALG_FLOP = 160      # fBm: FLOP per vertex-octave of the reference's noise3d (binary64 operation count)


def measure_insolation(sm_mhz):
    """The insolation kernel on its own (the 64-planet batch has none): a
    year of hourly sun positions (365 x 24) over a divisions-1000 sphere
    (10,000,002 vertices), CUDA events, best of 3.  The kernel sums each
    vertex's year by breakpoints (the schedule's days sorted once per block,
    twelve searches per vertex), so it performs no per-term operations: its
    bound is instruction issue, reported from the instruction count of the
    ncu capture of the same launch (profiles/insolation_issue.json) against
    152 SMs x 4 schedulers x the clock; beside it the HBM traffic the kernel
    needs (24 B of coordinates in, 4 B out per vertex) and the reference's
    work model (6 FLOP per vertex x sun position), which an exact algebraic
    reduction of the sum exceeds."""
    import torch
    from nixis_gb300 import mesh, climate, _dev, _lib
    try:
        m = mesh.PlanetMesh(1000)
        out = torch.empty(m.n, dtype=torch.float32, device="cuda")
        # the schedule planned once (host tables, one copy), then the kernel
        # launches alone inside the timed region
        rot, tilts = climate.annual_schedule(23.44, 365, 365, 24)
        tab, nre, pairs = climate._plan(rot, tilts)
        tdev = torch.from_numpy(tab).cuda()
        s = _dev.stream_handle()
        ms = _time(lambda: _lib.call("nx_insolation", _dev.ptr(m.xyz), m.n, 1.0, _dev.ptr(tdev), nre, pairs,
                                     len(tilts), _dev.ptr(out), 0, s))
        ref = climate.annual_insolation(m.xyz, 1.0)
        if not torch.equal(ref, out):
            raise RuntimeError("timed launch differs from annual_insolation")
    except Exception as e:       # reported, not fatal: the headline is the batch
        return {"error": str(e)[:200]}
    n = m.n
    del m, out, ref
    terms = n * 365 * 24
    res = {"ms": ms, "terms_per_s": terms / (ms / 1e3),
           "hbm": {"bytes_per_vertex": 28, "achieved_gbs": n * 28 / (ms / 1e3) / 1e9},
           "reference_model": {"flop_per_term": 6, "equivalent_tflops": terms * 6 / (ms / 1e3) / 1e12,
                               "fp32_peak_tflops": fp32_peak_tflops(sm_mhz),
                               "note": "6 FLOP per vertex x sun position, the reduced form of the reference's term; "
                                       "the kernel reaches the same sums without per-term work (exact algebra, within "
                                       "1e-5 of binary64 in tests)"}}
    peak_issue = 152 * 4 * sm_mhz * 1e6
    issue = os.path.join(ROOT, "profiles", "insolation_issue.json")
    try:
        with open(issue) as f:
            wpv = float(json.load(f)["warp_instructions_per_vertex"])
        rate = n * wpv / (ms / 1e3)
        res.update({"bound": "issue", "achieved": rate / 1e12, "peak": peak_issue / 1e12,
                    "unit": "T warp instructions/s", "frac": rate / peak_issue,
                    "model": f"{wpv:.2f} warp instructions per vertex (ncu capture of the same launch) x {n} vertices; "
                             "peak = 152 SMs x 4 schedulers x clock"})
    except (OSError, KeyError, ValueError):
        pk, _ = measured_peak()
        res.update({"bound": "hbm", "achieved": res["hbm"]["achieved_gbs"], "peak": pk, "unit": "GB/s",
                    "frac": res["hbm"]["achieved_gbs"] / pk})
    return res


# planets of the 64-planet workload checked against binary64 outside the
# timed region: 22 (divisions 339, 12 octaves, 85 iterations), 9 (310, 7, 97),
# 0 (762, 12, 56)
ERROR_SAMPLE = (22, 9, 0)


def errors_vs_binary64(batch, reqs, cache):
    """Per-field error of sampled batched planets against the oracle's
    binary64 run of the reference's functions (sample_octaves, rescale,
    erosion_iteration3): max |err| / max |ref| and RMS / max |ref| for
    height, water and sediment."""
    from oracle import oracle as O
    out = {}
    worst = 0.0
    for i in ERROR_SAMPLE:
        r = reqs[i]
        m = cache.get(r.divisions)
        pts, adj = m.xyz.cpu().numpy(), m.nbr.cpu().numpy()
        perm, pgi = O.init(r.seed)
        h = O.rescale(O.sample_octaves(pts, None, perm, pgi, r.octaves, 1.0, 1.0, 2.0, 0.5, 1.0), -8000.0, 8000.0)
        w, s = np.full(len(pts), 1e-3), np.zeros(len(pts))
        for _ in range(r.erosion_iters):
            O.erosion_iteration3(pts, adj, h, w, s)
        got = [t.cpu().numpy() for t in batch.fields(i)]
        fields = {}
        for name, g, ref in zip("hws", got, (h, w, s)):
            sc = float(np.abs(ref).max()) or 1.0
            err = g - ref
            fields[name] = {"max_rel": float(np.abs(err).max() / sc), "rms_rel": float(np.sqrt(np.mean(err ** 2)) / sc)}
        worst = max(worst, fields["h"]["max_rel"])
        out[f"planet{i}"] = dict(divisions=r.divisions, octaves=r.octaves, iters=r.erosion_iters, **fields)
    out["max_rel_h"] = worst
    out["bar"] = 1e-5
    return out


# ---------------------------------------------------------------------------
# serving: continuous batching against the plain per-planet path

def run_serving(n_requests, hbm_budget=120 * 2**30):
    """The first n requests of the serving stream (Poisson arrivals at 20
    req/s, seed 11, divisions log-uniform in [50, 2000], octaves U[4,12],
    erosion iterations U[0,100], insolation for half), served (a) as they
    arrive and (b) all at once, by the engine and by the plain per-planet
    path; every engine result is checked bit for bit against the plain
    path's.  Meshes are built on demand by both (resident, LRU under each
    path's budget); both paths keep theirs from the arrivals run for the
    all-at-once run."""
    import hashlib
    from concurrent.futures import ThreadPoolExecutor
    import torch
    from nixis_gb300 import serve
    stream = serve.poisson_stream(2000)[:n_requests]
    # results are compared through 16-byte BLAKE2b digests of their bytes,
    # taken on a pool of their own (hashlib releases the GIL), so that
    # neither path holds 2,000 results (~100 GB) and neither waits on them
    pool = ThreadPoolExecutor(max_workers=8, thread_name_prefix="digest")

    def fingerprint(a):
        return None if a is None else hashlib.blake2b(memoryview(np.ascontiguousarray(a)), digest_size=16).digest()

    def digest_pair(h, i):
        return pool.submit(lambda: (fingerprint(h), fingerprint(i)))

    def engine_sink(t):
        t.digest = digest_pair(t.heights, t.insolation)
        t.heights = t.insolation = None

    def plain_sink(h, i):
        return digest_pair(h.numpy(), None if i is None else i.numpy())
    out = {"requests": len(stream), "arrival_rate_per_s": 20.0, "hbm_budget_gb": hbm_budget / 2**30,
           "meshes": "built on demand; each path keeps its meshes from the arrivals run for the all-at-once run "
                     "within its HBM budget (LRU), so meshes evicted since are rebuilt"}
    eng_meshes = None
    pm = serve.ResidentMeshes(hbm_budget // 2)
    # both paths load their kernels on two tiny requests before timing
    from nixis_gb300.planets import PlanetRequest
    serve.serve_plain([(0.0, PlanetRequest(seed=0, divisions=2, octaves=2, erosion_iters=3, insolation=True,
                                           days=2, hours=24))], realtime=False)
    for mode, realtime in (("arrivals", True), ("all_at_once", False)):
        eng = serve.ServeEngine(hbm_budget=hbm_budget).warmup()
        eng.result_sink = engine_sink
        if eng_meshes is not None:
            eng.meshes = eng_meshes          # meshes stay resident between the two runs
            eng.meshes.tb = eng.tb
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        tk = eng.run(stream, realtime=realtime, t0=t0)
        span = time.perf_counter() - t0
        eng_meshes = eng.meshes
        eng.close()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        plain = serve.serve_plain(stream, meshes=pm, realtime=realtime, t0=t1, sink=plain_sink)
        span_p = time.perf_counter() - t1
        same = all(t.digest.result() == p[2].result() for t, p in zip(tk, plain))
        lat_e = serve.latency_stats([t.latency for t in tk])
        lat_p = serve.latency_stats([f - a for a, f, _ in plain])
        r3 = lambda d: {k: round(v, 2) for k, v in d.items()}
        out[mode] = {"engine": r3(dict(lat_e, planets_per_s=len(tk) / span, seconds=span)),
                     "plain": r3(dict(lat_p, planets_per_s=len(plain) / span_p, seconds=span_p)),
                     "p99_ratio_plain_over_engine": round(lat_p["p99_ms"] / lat_e["p99_ms"], 3),
                     "results_equal_plain": bool(same)}
        del eng
    pool.shutdown(wait=True)
    return out


def profile_extras():
    """One run of each kernel outside the batch on a mid-size sphere
    (divisions 500, 2,500,002 vertices): mesh and tiling build (the default
    blocked setting's tile side and rings), the height
    shaping sequence, the latitude-table year, an equirectangular map of
    1024 x 512 pixels.  The case the ncu summaries of those kernels use."""
    import torch
    from oracle import oracle as O
    from nixis_gb300 import mesh, terrain, util, climate
    from nixis_gb300 import autotune
    m = mesh.PlanetMesh(500)
    m.tiling(autotune.DEFAULT.tile_side, autotune.DEFAULT.rings).maxnl
    perm, pgi = O.init(3)
    h = terrain.sample_octaves(m.xyz, None, perm, pgi, 8, 1.0, 1.0, 2.0, 0.5, 1.0)
    shaped, _, _ = util.shape_heights(h)
    climate.calc_yearly_insolation(m.xyz, None, 1.0, 23.44)
    colors = util.rescale(shaped, 0, 255)
    util.equirect_map(m.xyz, m.nbr, 500, colors, 1024, 512, 1.0)
    torch.cuda.synchronize()
    print(json.dumps({"profile_run": "extras", "vertices": m.n}))


def profile_insolation():
    """One insolation launch (365 days x 24 hours) over divisions 1000
    (10,000,002 vertices, the case measure_insolation times): the case the
    ncu capture of the kernel uses."""
    import torch
    from nixis_gb300 import mesh, climate
    m = mesh.PlanetMesh(1000)
    climate.annual_insolation(m.xyz, 1.0)
    torch.cuda.synchronize()
    print(json.dumps({"profile_run": "insolation", "vertices": m.n, "sun_positions": 365 * 24}))


def bench_serve(args):
    from nixis_gb300 import autotune
    import torch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    if args.tb:
        tb = autotune.parse(args.tb)
        autotune.use(tb)
    else:
        tb, _ = autotune.tune(save=False)
    res = run_serving(args.serve)
    res["blocked_erosion"] = tb.label
    print(json.dumps({"serving": res}))


# ---------------------------------------------------------------------------
# single-planet configurations (supplementary lines)

def _events():
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def _time(fn, reps=3):
    import torch
    fn()
    torch.cuda.synchronize()
    best = None
    for _ in range(reps):
        a, b = _events()
        a.record()
        fn()
        b.record()
        torch.cuda.synchronize()
        ms = a.elapsed_time(b)
        best = ms if best is None else min(best, ms)
    return best


def bench_single(name):
    """Print the single-planet line of `name` (see single_planet)."""
    print(json.dumps(single_planet(name)))


def single_planet(name):
    """c1: divisions 250, 8 octaves, seed 0, metres (float64);
    c2: divisions 1000, 12 octaves, seed 1, then 50 erosion iterations from
        water 1e-3, sediment 0 (errors per field vs binary64 at 1/10/50);
    c3: divisions 2500, 12 octaves, seed 2, 200 erosion iterations, and
        mean annual insolation over 365 days x 24 hours.
    Returns the configuration's figures as a dict."""
    import torch
    from oracle import oracle as O
    from nixis_gb300 import mesh, terrain, erosion, climate, planets
    k, octs, seed = {"c1": (250, 8, 0), "c2": (1000, 12, 1), "c3": (2500, 12, 2)}[name]
    m = mesh.PlanetMesh(k)
    n = m.n
    perm, pgi = O.init(seed)
    sc, st = terrain._octave_args(octs, 1.0, 1.0, 2.0, 0.5, 1.0)
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    out32 = torch.empty(n, dtype=torch.float32, device="cuda")
    fbm_ms = _time(lambda: terrain.fbm(m.xyz, perm, pgi, sc, st, 1.0, out=out))          # pair precision
    fbm32_ms = _time(lambda: terrain.fbm(m.xyz, perm, pgi, sc, st, 1.0, out=out32))      # binary32
    _, nfb = terrain.fbm(m.xyz, perm, pgi, sc, st, 1.0, out=out, count_fallbacks=True)
    h = out.cpu().numpy()
    h32 = out32.double().cpu().numpy()
    del out32
    line = {"config": name, "divisions": k, "vertices": n, "octaves": octs, "seed": seed,
            "fbm_ms": fbm_ms, "fbm_precision": "pair (float-float)", "vertex_octaves_per_s": n * octs / (fbm_ms / 1e3),
            "fbm_tflops_at_160": n * octs * 160 / (fbm_ms / 1e3) / 1e12,
            "fbm_binary32_ms": fbm32_ms, "binary64_decision_rate": nfb / (n * octs)}
    pts = m.xyz.cpu().numpy()
    t0 = time.perf_counter()
    ref = O.sample_octaves(pts, None, perm, pgi, octs, 1.0, 1.0, 2.0, 0.5, 1.0)
    line["cpu_fbm_s"] = time.perf_counter() - t0
    r = ref.max() - ref.min()
    line["fbm_max_err_over_range"] = float(np.abs(h - ref).max() / r)
    line["fbm_rms_err_over_range"] = float(np.sqrt(np.mean((h - ref) ** 2)) / r)
    line["fbm_binary32_max_err_over_range"] = float(np.abs(h32 - ref).max() / r)
    hm = O.rescale(ref, -8000.0, 8000.0)
    hg = O.rescale(h, -8000.0, 8000.0)
    line["elevation_max_err_m"] = float(np.abs(hg - hm).max())
    if name == "c1":
        return line
    iters = 50 if name == "c2" else 200
    nbr = m.nbr.cpu().numpy()
    hm_t = torch.from_numpy(hm).cuda()
    w0 = torch.full((n,), 1e-3, dtype=torch.float64, device="cuda")
    run = erosion.ErosionRun(m.xyz, m.nbr, m.edge)
    checkpoints = [1, 10, 50] if name == "c2" else [1, 10, 50, 100, 140, 150, 200]
    # binary32-pair state vs binary64 reference, per field, at checkpoints
    errs = {}
    if name == "c2":
        run.load(hm_t, w0)
        hw, ww, sw = hm.copy(), np.full(n, 1e-3), np.zeros(n)
        done = 0
        hd = torch.empty(n, dtype=torch.float64, device="cuda")
        wd, sd = torch.empty_like(hd), torch.empty_like(hd)
        for cp in checkpoints:
            run.steps(cp - done)
            for _ in range(cp - done):
                O.erosion_iteration3(pts, nbr, hw, ww, sw)
            done = cp
            run.store(hd, wd, sd)
            g = [hd.cpu().numpy(), wd.cpu().numpy(), sd.cpu().numpy()]
            errs[cp] = {f: {"max_abs_over_max": float(np.abs(a - b).max() / np.abs(b).max()),
                            "rms_over_max": float(np.sqrt(np.mean((a - b) ** 2)) / np.abs(b).max())}
                        for f, a, b in zip("hws", g, (hw, ww, sw))}
            # flow choices (sign of h_n - h_i per slot) that differ from binary64's
            jj = np.where(nbr < 0, np.arange(n)[:, None], nbr)
            errs[cp]["flow_choice_flips"] = int((np.sign(g[0][jj] - g[0][:, None]) !=
                                                 np.sign(hw[jj] - hw[:, None])).sum())
        line["erosion_errors"] = errs
    # timing: one planet's erosion, blocked (batch of one) and iteration at a time (CUDA graph)
    req = planets.PlanetRequest(seed=seed, divisions=k, octaves=octs, erosion_iters=iters)
    cache = mesh.MeshCache()
    cache._m[k] = m
    cache._order.append(k)
    for blocked in (True, False):
        bt = planets.PlanetBatch([req], cache, blocked=blocked)
        bt.capture()
        ms = _time(lambda: bt.run())
        ero = ms - fbm_ms
        line["planet_ms_blocked" if blocked else "planet_ms_iteration_kernel"] = ms
        line["erosion_gvi_per_s_blocked" if blocked else "erosion_gvi_per_s_iteration_kernel"] = n * iters / (ero / 1e3) / 1e9
        res = bt.results()[0]
        line["scale_exponent"] = res.scale_exponent
        del bt
    # mass sums (compensated, per iteration) and where plain binary32 would overflow
    run.load(hm_t, w0)
    mass, _ = run.steps(iters, mass=True)
    ms_ = mass.cpu().numpy()
    # sum(h + s) is invariant under the update; its drift relative to the
    # size of the sums (which grow ~2x per iteration)
    inv0, inv1 = ms_[0, 0] + ms_[0, 2], ms_[-1, 0] + ms_[-1, 2]
    line["mass_h_plus_s_drift_rel"] = float(abs(inv1 - inv0) / max(abs(ms_[-1, 0]), abs(ms_[-1, 2]), abs(inv0)))
    line["scale_exponent_after"] = run.scale_exponent()
    over = [i + 1 for i in range(iters) if abs(ms_[i, 1]) / n > 3.4e38]
    line["first_iteration_mean_water_above_binary32_max"] = over[0] if over else None
    if name == "c3":
        xs = m.xyz
        ins_ms = _time(lambda: climate.annual_insolation(xs, 1.0), reps=2)
        samples = n * 365 * 24
        line["insolation_ms"] = ins_ms
        line["insolation_samples_per_s"] = samples / (ins_ms / 1e3)
        line["insolation_tflops_at_6"] = samples * 6 / (ins_ms / 1e3) / 1e12
        rng = np.random.default_rng(0)
        idx = rng.choice(n, 100000, replace=False)
        got = climate.annual_insolation(xs, 1.0).cpu().numpy()[idx]
        ref_i = O.annual_insolation(pts[idx], 1.0)
        line["insolation_max_err_over_max"] = float(np.abs(got - ref_i).max() / np.abs(ref_i).max())
        line["mean_toa_wm2_range"] = [float(1361 * got.min() / 8760), float(1361 * got.max() / 8760)]
    return line


def bench_mesh_prep(args):
    """Mesh preparation of the workload (supplementary line): the distinct
    divisions' meshes (icosphere, adjacency, edge lengths) and then their
    blocked-erosion tilings, each phase timed with CUDA events, twice after
    a warm-up build (the batch keeps them resident, so this is not part of
    its step)."""
    import torch
    from nixis_gb300 import autotune, mesh
    cfg = autotune.DEFAULT
    divs = sorted({r.divisions for r in workload(args.workload)})
    m = mesh.PlanetMesh(20)
    m.tiling(cfg.tile_side, cfg.rings)
    torch.cuda.synchronize()
    del m
    reps = []
    for _ in range(2):
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        torch.cuda.synchronize()
        e0.record()
        meshes = [mesh.PlanetMesh(k, defer_checks=True) for k in divs]
        e1.record()
        tilings = [x.tiling(cfg.tile_side, cfg.rings) for x in meshes]
        e2.record()
        torch.cuda.synchronize()
        for x in meshes:
            x.check()
        reps.append((e0.elapsed_time(e1), e1.elapsed_time(e2)))
        nv = sum(x.n for x in meshes)
        del meshes, tilings
    print(json.dumps({"mesh_prep": args.workload, "meshes": len(divs), "vertices": nv,
                      "tiling": f"{cfg.tile_side}/{cfg.rings}",
                      "mesh_ms": [round(a, 2) for a, _ in reps], "tiling_ms": [round(b, 2) for _, b in reps]}))


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
    ap.add_argument("--single", choices=["c1", "c2", "c3"], help="a single-planet configuration (supplementary line)")
    ap.add_argument("--tb", help="blocked-erosion setting side/rings/threads[variant letter] instead of autotuning "
                                 "(e.g. 40/4/512, 40/4/384p with prefetch, 32/4/384d with 3 blocks per SM)")
    ap.add_argument("--tune-only", action="store_true", help="run the autotuner, print its table, exit")
    ap.add_argument("--profile-insolation", action="store_true",
                    help="one annual insolation launch on a 2,246,762-vertex sphere (ncu), exit")
    ap.add_argument("--profile-extras", action="store_true",
                    help="one run of the mesh, shaping, latitude-table and map kernels (ncu), exit")
    ap.add_argument("--no-blocked", action="store_true",
                    help="with --profile: one launch per erosion iteration instead of blocked passes")
    ap.add_argument("--serve", type=int, default=0, help="serving comparison on the first N stream requests, exit")
    ap.add_argument("--serve-requests", type=int, default=2000, help="stream requests in the default line's serving leg")
    ap.add_argument("--no-single", action="store_true",
                    help="skip the single-planet error block (c1, c2 against binary64) of the default line")
    ap.add_argument("--mesh-prep", action="store_true",
                    help="time the workload's mesh and tiling builds (CUDA events), print one line, exit")
    args = ap.parse_args()
    if args.mesh_prep:
        bench_mesh_prep(args)
        return
    if args.single:
        bench_single(args.single)
        return
    if args.serve:
        bench_serve(args)
        return
    if args.profile_insolation:
        profile_insolation()
        return
    if args.profile_extras:
        profile_extras()
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        bench_reference(args)
    else:
        bench_ours(args)


if __name__ == "__main__":
    main()
