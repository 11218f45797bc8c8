"""Benchmark of the SPH step on GB300: particle-steps/s on the 2,097,152-particle
dam-break block (128^3 jittered lattice, spacing 0.05 m, box 16 x 8 x 8 m,
h = 0.1, FP32), one JSON line on rank 0.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl sphx|reference]

* value: K device-resident steps timed with CUDA events on the scene's
  stream (barrier + synchronize on both sides, max over ranks); each rank
  advances its own replica (a single scene does not shard: "replicas").
* roofline: per-phase CUDA events recorded inside the same timed region;
  density + force kernels against the measured HBM copy bandwidth.
* e2e: the same metric through the C-ABI with host buffers — every step
  uploads the state from pinned host memory, steps, and reads positions and
  velocities back.
* cpu_baseline: the oracle restatement of the reference's multithreaded CPU
  update (oracle/sph_oracle.cpp) on this host's cores, on a bounded sample.
* --impl reference: that CPU implementation alone, as the reference arm.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "sph-fluid-simulator_gb300"))

METRIC = "particle-steps/s @2.1M"
UNIT = "particle-steps/s"
SIDE = 128  # 128^3 = 2,097,152 particles
ALGO_BYTES = 80  # density 24 B + force 56 B per particle-step (compulsory FP32 SoA)
# FP32 operations of the walk kernels: an r^2 test is 3 sub + 3 mul + 2 add;
# an accepted pair costs the density 1 sub + 1 mul + 1 fused multiply-add
# (the cube added to its row's sum) and the force 41 (distance 8, rsqrt, r
# and h - r 2, two coefficients 6, three components 3 x 4, compensated adds
# 12)
OPS_PER_TEST = 8
OPS_PER_PAIR_DENSITY = 4
OPS_PER_PAIR_FORCE = 41
WORKLOAD = ("dam-break block 128^3 = 2,097,152 particles, jittered cubic lattice spacing 0.05 m "
            "(+-5%), box 16 x 8 x 8 m (walls at bound +- h, floor y=0, no ceiling), h=0.1, "
            "rho0=1000, m=0.125, k=20, mu=1, g=-9.8, dt=0.002, damping 0.5")


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def max_over_ranks(x):
    """Max of a float over all ranks (identity when not distributed).  Uses a
    CUDA tensor under NCCL and a CPU tensor under gloo."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def profiled_traffic(n):
    """DRAM bytes (read + write) of one k_density and one k_force launch on this
    workload, from the committed ncu capture summary (profiles/), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "dram_traffic.json")) as f:
            d = json.load(f)
        if int(d["particles"]) != n:
            return None
        return float(d["k_density"]) + float(d["k_force"])
    except Exception:
        return None


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


class ClockSampler:
    """nvidia-smi SM clock / throttle-reason sampling during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if len(r) > 4 + i and r[4 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def workload():
    import sphx
    pos, box = sphx.dambreak(SIDE)
    return pos, box, sphx.config_settings()


def cpu_baseline(pos, box, s, budget_s=15.0, max_steps=20):
    """The oracle restatement of the reference CPU update on this host."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    pyoracle.build()
    port = pyoracle.Port()
    import sphx
    args = sphx.args_array(s)
    t0 = time.perf_counter()
    port.run(pos, None, args, sphx.DT, 0, box=box.as_array())  # load/unload only
    t_io = time.perf_counter() - t0
    t0 = time.perf_counter()
    port.run(pos, None, args, sphx.DT, 1, box=box.as_array())
    t1 = max(time.perf_counter() - t0 - t_io, 1e-6)
    steps = int(max(1, min(max_steps, budget_s // t1)))
    t0 = time.perf_counter()
    port.run(pos, None, args, sphx.DT, steps, box=box.as_array())
    t = max(time.perf_counter() - t0 - t_io, 1e-6)
    return {"value": len(pos) * steps / t, "unit": UNIT, "cores": port.hw_threads(), "kind": "port",
            "sample": "%d steps of the %d-particle workload from its initial state "
                      "(oracle restatement of updateParticlesCPU, std::thread x %d)"
                      % (steps, len(pos), port.hw_threads())}


def batch_compare(scenes, steps, warmup, device, cache_path=None):
    """Scenes/s of the batched form against the same scenes one at a time
    through the plain single-scene path, each arm end to end: upload, `steps`
    steps of dt, readout of every scene (the batched arm's autotuning is a
    one-off, cached, and not timed)."""
    import torch
    import sphx
    opts = sphx.default_options(device=device)
    with sphx.Scene.batch(scenes, opts) as b:
        tune = b.autotune(sphx.DT, trial_steps=3, cache_path=cache_path)
    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    with sphx.Scene.batch(scenes, opts) as b:
        b.set_tuning(tune.density_threads, tune.force_threads, tune.reorder_interval)
        stream = torch.cuda.ExternalStream(b.device_view().stream, device=device)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.step(sphx.DT, steps)
        e1.record(stream)
        out = b.read()  # every scene, scene after scene, each in id order
        ranges = [b.scene_range(k) for k in range(len(scenes))]
        per_scene = [out["pos"][first:first + count] for first, count in ranges]
    t_batch = time.perf_counter() - t0
    steps_ms = e0.elapsed_time(e1)
    assert len(per_scene) == len(scenes)
    t0 = time.perf_counter()
    for s, pos, box in scenes:
        with sphx.Scene(s, box, pos, None, opts) as one:
            one.step(sphx.DT, steps)
            one.read()
    t_seq = time.perf_counter() - t0
    n = sum(len(p) for _, p, _ in scenes)
    return {"scenes": len(scenes), "particles": n, "steps": steps,
            "batched_scenes_per_s": len(scenes) / t_batch,
            "sequential_scenes_per_s": len(scenes) / t_seq,
            "speedup": t_seq / t_batch,
            "batched_particle_steps_per_s": n * steps / t_batch,
            "batched_device_particle_steps_per_s": n * steps / (steps_ms / 1e3),
            "tuning": {"density_threads": tune.density_threads, "force_threads": tune.force_threads,
                       "reorder_interval": tune.reorder_interval},
            "note": "end to end per arm: upload, steps, readout of every scene (the batch in one "
                    "read); results bit-identical per scene; device rate: the steps alone, CUDA events"}


def run_batch(a):
    import torch
    import sphx
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    scenes = sphx.batch_scenes(512, seed=0)
    res = batch_compare(scenes, a.steps, a.warmup, local,
                        cache_path=os.environ.get("SPHX_TUNE_CACHE"))
    line = {"metric": "scenes/s (512 scenes, batched vs one at a time)", "value": res["batched_scenes_per_s"],
            "unit": "scenes/s", "n_gpus": 1, "steps": a.steps, "warmup": a.warmup,
            "higher_is_better": True, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": "512 dam-break scenes, N log-uniform [1000, 65536], aspect U[0.5,2], "
                                   "k U[10,40], mu U[0.5,3], box 2.5/1.25/1.25 x block"},
            "batched": res}
    print(json.dumps(line), flush=True)


def serve_requests(count, seed=1):
    """The served workload's request stream: dam-break blocks with N
    log-uniform in [2000, 500000], step counts uniform in [100, 2000], k and mu
    drawn as in the batched workload."""
    import math
    import sphx
    rng = np.random.default_rng(seed)
    reqs = []
    for k in range(count):
        target = math.exp(rng.uniform(math.log(2000), math.log(500000)))
        aspect = rng.uniform(0.5, 2.0, 3)
        c = (target / aspect.prod()) ** (1.0 / 3.0)
        nx, ny, nz = (max(2, int(round(c * x))) for x in aspect)
        s = sphx.config_settings(gas_const=float(rng.uniform(10, 40)),
                                 viscosity=float(rng.uniform(0.5, 3)))
        pos, box = sphx.dambreak(nx, ny, nz, seed=seed * 7919 + k)
        reqs.append((s, pos, box, int(rng.integers(100, 2001))))
    return reqs


def serve_sweep(sphx, count, rates, tick, device):
    """Poisson arrivals at each rate: p50/p95/p99 completion latency and
    scenes/s of the continuous-batching server, against the same stream
    served one request at a time through the plain path (FIFO: each request
    starts when both it has arrived and the previous one has finished, with
    its measured service time, each request measured alone once)."""
    reqs = serve_requests(count, seed=1)
    service = []
    for s, pos, box, nsteps in reqs:
        t0 = time.perf_counter()
        with sphx.Scene(s, box, pos, None, sphx.default_options(device=device)) as one:
            one.step(sphx.DT, nsteps)
            one.read()
        service.append(time.perf_counter() - t0)
    results = []
    rng = np.random.default_rng(2)
    q = lambda x, p: float(np.percentile(x, p))
    for lam in rates:
        arrivals = np.cumsum(rng.exponential(1.0 / lam, len(reqs)))
        arrivals -= arrivals[0]
        end = 0.0
        lat_seq = []
        for t_arr, svc in zip(arrivals, service):
            start = max(t_arr, end)
            end = start + svc
            lat_seq.append(end - t_arr)
        span_seq = end - arrivals[0]
        with sphx.Server(budget_bytes=150e9, steps_per_tick=tick, device=device) as srv:
            t0 = time.perf_counter()
            tickets = []
            for (s, pos, box, nsteps), t_arr in zip(reqs, arrivals):
                delay = t_arr - (time.perf_counter() - t0)
                if delay > 0:
                    time.sleep(delay)
                tickets.append(srv.submit(s, box, pos, nsteps))
            for t in tickets:
                srv.wait(t, timeout=1200)
            sts = [srv.status(t) for t in tickets]
            for t in tickets:
                srv.result(t)
            st = srv.stats()
        lat = np.array([x.done_s - x.submit_s for x in sts])
        span = max(x.done_s for x in sts) - min(x.submit_s for x in sts)
        results.append({"rate_per_s": lam, "span_s": span,
                        "served": {"scenes_per_s": len(reqs) / span, "p50_s": q(lat, 50),
                                   "p95_s": q(lat, 95), "p99_s": q(lat, 99),
                                   "relayouts": int(st.relayouts), "ticks": int(st.ticks),
                                   "worker_s": {"layout": st.layout_s, "step": st.step_s,
                                                "readout": st.readout_s}},
                        "sequential": {"scenes_per_s": len(reqs) / span_seq, "p50_s": q(lat_seq, 50),
                                       "p95_s": q(lat_seq, 95), "p99_s": q(lat_seq, 99)},
                        "speedup": span_seq / span})
    n_ps = sum(len(p) * k for _, p, _, k in reqs)
    return {"requests": len(reqs), "particle_steps": n_ps, "steps_per_tick": tick,
            "hbm_budget_gb": 150, "rates": results,
            # no schedule can finish the stream before its longest request
            # finishes alone: the served span's floor
            "requests_n": [int(len(p)) for _, p, _, _ in reqs],
            "requests_steps": [int(k) for _, _, _, k in reqs],
            "service_s": [round(float(x), 4) for x in service],
            "longest_request_alone_s": float(max(service)),
            "sequential_total_s": float(sum(service)),
            "speedup_bound": float(sum(service)) / float(max(service)),
            "workload": "requests: N log-uniform [2000, 500000], steps U[100, 2000], k U[10,40], "
                        "mu U[0.5,3], dam-break blocks; sequential arm: each request alone through "
                        "the plain path (create, steps, readout), FIFO over the same arrivals"}


def run_serve(a):
    import torch
    import sphx
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    res = serve_sweep(sphx, a.requests, [float(x) for x in a.rates.split(",")], a.tick, local)
    line = {"metric": "served scenes/s and completion latency", "unit": "scenes/s",
            "value": res["rates"][-1]["served"]["scenes_per_s"], "higher_is_better": True,
            "n_gpus": 1, "dtype": "f32", "data": "synthetic (seeded Poisson stream)",
            "config": {"workload": res["workload"], "steps_per_tick": a.tick}, "served": res}
    print(json.dumps(line), flush=True)


def run_steps_only(a):
    """Profiling driver: the headline scene (or a --side^3 block, or with
    --scenes the batched workload's first N scenes as one batch), W + K steps
    as plain launches (no graph, no events), one summary line."""
    import torch
    import sphx
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    opt = sphx.default_options(device=local, use_graph=0)
    if a.scenes:
        scenes = sphx.batch_scenes(a.scenes, seed=0)
        n = sum(len(p) for _, p, _ in scenes)
        with sphx.Scene.batch(scenes, opt) as b:
            b.step(sphx.DT, a.warmup + a.steps)
            b.synchronize()
    else:
        pos, box = sphx.dambreak(a.side)
        n = len(pos)
        with sphx.Scene(sphx.config_settings(), box, pos, None, opt) as sc:
            sc.step(sphx.DT, a.warmup + a.steps)
            sc.synchronize()
    print(json.dumps({"workload": "steps", "scenes": a.scenes or 1, "particles": n,
                      "steps": a.warmup + a.steps}))


def run_reference(a):
    """The reference arm: the CPU restatement alone, on the same workload.
    Its inputs come from the oracle's numpy generators (bit-identical to the
    product's), so this arm loads nothing of the product."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    pyoracle.build()
    port = pyoracle.Port()
    pos, box = pyoracle.dambreak(SIDE)
    args = pyoracle.config_args()
    p, v = pos, None
    for _ in range(a.warmup):
        p, v, _, _ = port.run(p, v, args, pyoracle.DT, 1, box=box)
    # each step is one full-workload step; the loop stops early once the
    # budget is spent so that a large --steps still ends within minutes
    t0 = time.perf_counter()
    done = 0
    while done < max(1, a.steps) and (done == 0 or time.perf_counter() - t0 < a.ref_budget):
        p, v, _, _ = port.run(p, v, args, pyoracle.DT, 1, box=box)
        done += 1
    t = time.perf_counter() - t0
    val = len(pos) * done / t
    line = {"metric": METRIC, "value": val, "unit": UNIT, "n_gpus": 0, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": 1e3 * t / done, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "impl": "reference",
            "data": "synthetic (seeded SplitMix64 lattice)",
            "config": {"workload": WORKLOAD, "reorder_interval": None, "parallelism": "host threads"},
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": port.hw_threads(), "kind": "port",
                             "sample": "%d timed steps (after %d warm-up) of the full workload; "
                                       "the reference's own build cannot run on this host "
                                       "(compiled x86-64 only), so its restatement runs"
                                       % (done, a.warmup)},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


SIDE_8M = 200  # 200^3 = 8,000,000 particles
REORDER_SWEEP = (1, 4, 16, 64)


def copy_ceiling(torch, nbytes, reps=10):
    """Single-copy rates (GB/s) between pinned host memory and the device, each
    direction alone, for copies of nbytes."""
    h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    out = {}
    for kind in ("h2d", "d2h"):
        for _ in range(2):
            (d.copy_(h, non_blocking=True) if kind == "h2d" else h.copy_(d, non_blocking=True))
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            (d.copy_(h, non_blocking=True) if kind == "h2d" else h.copy_(d, non_blocking=True))
        e1.record()
        torch.cuda.synchronize()
        out[kind + "_gbs"] = nbytes * reps / (e0.elapsed_time(e1) / 1e3) / 1e9
    out["bytes"] = nbytes
    return out


def configured_run(sphx, torch, s, box, pos, device, steps, reorder, phases, peak):
    """`steps` steps from the initial lattice as CUDA-graph replays, timed with
    CUDA events on the scene's stream.  With `phases`, the same run again as
    plain launches with per-phase events (sort, density, force) for the
    roofline of the whole run."""
    n = len(pos)
    out = {"steps": steps, "reorder_interval": reorder}
    with sphx.Scene(s, box, pos, None, sphx.default_options(device=device, use_graph=1,
                                                           reorder_interval=reorder)) as sc:
        stream = torch.cuda.ExternalStream(sc.device_view().stream, device=device)
        c0 = torch.cuda.Event(enable_timing=True)
        c1 = torch.cuda.Event(enable_timing=True)
        c0.record(stream)
        sc.step(sphx.DT, steps)
        c1.record(stream)
        sc.synchronize()
        ms = max_over_ranks(c0.elapsed_time(c1))
    out["ms_per_step"] = ms / steps
    out["particle_steps_per_s"] = n * steps / (ms / 1e3)
    if phases:
        with sphx.Scene(s, box, pos, None, sphx.default_options(device=device, use_graph=0,
                                                               reorder_interval=reorder)) as sc:
            sc.set_profiling(True)
            sc.kernel_times()
            sc.step(sphx.DT, steps)
            kt = sc.kernel_times()
        d, f = kt.density_ms / max(kt.steps, 1), kt.force_ms / max(kt.steps, 1)
        achieved = ALGO_BYTES * n / ((d + f) / 1e3) / 1e9
        out["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                           "frac": achieved / peak, "kernels": "k_density + k_force",
                           "per_step_ms": {"sort": kt.sort_ms / max(kt.steps, 1), "density": d,
                                           "force": f},
                           "note": "mean over the whole run, plain launches with per-phase events"}
    out["note"] = "whole configured run from the initial lattice, CUDA graph replay"
    return out


def run_sphx(a):
    import torch
    import sphx
    rank, world, local = dist_env()
    device = local
    torch.cuda.set_device(device)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", device))
    pos, box, s = workload()
    n = len(pos)
    opts = sphx.default_options(device=device, reorder_interval=a.reorder, use_graph=0)
    sc = sphx.Scene(s, box, pos, None, opts)
    view = sc.device_view()
    stream = torch.cuda.ExternalStream(view.stream, device=device)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    # warm-up, then the timed region with per-phase events recorded inside it
    sc.step(sphx.DT, a.warmup)
    sc.synchronize()
    st0 = sc.read()  # the window's first state: the e2e leg below starts from it
    walk0 = sc.walk_stats()  # (r^2 tests, accepted pairs) of the window's first step
    sc.set_profiling(True)
    sc.kernel_times()  # reset accumulators
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize(device)
    with ClockSampler(device) as clk:
        e0.record(stream)
        for _ in range(a.steps):
            sc.step(sphx.DT, 1)
        e1.record(stream)
        sc.synchronize()
        torch.cuda.synchronize(device)
    barrier()
    ms = max_over_ranks(e0.elapsed_time(e1))
    kt = sc.kernel_times()
    value = n * a.steps * world / (ms / 1e3)

    walk1 = sc.walk_stats()  # ... and of the state after its last step
    peak, peak_kind = peaks()
    dens_ms = kt.density_ms / max(kt.steps, 1)
    force_ms = kt.force_ms / max(kt.steps, 1)
    achieved = ALGO_BYTES * n / ((dens_ms + force_ms) / 1e3) / 1e9
    tests = 0.5 * (walk0[0] + walk1[0])
    pairs = 0.5 * (walk0[1] + walk1[1])
    ops = tests * OPS_PER_TEST + pairs * (OPS_PER_PAIR_DENSITY + OPS_PER_PAIR_FORCE)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_kind": peak_kind,
                "traffic": a.traffic if a.traffic is not None else profiled_traffic(n),
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, one launch of each "
                                  "kernel (profiles/dram_traffic.json)",
                "kernels": "k_density + k_force",
                "per_step_ms": {"sort": kt.sort_ms / max(kt.steps, 1), "density": dens_ms,
                                "force": force_ms},
                # the walk kernels are issue-bound, not bandwidth-bound: their work rates
                "r2_tests_per_step": tests, "accepted_pairs_per_step": pairs,
                "r2_tests_per_s": tests / (dens_ms / 1e3),
                "fp32_ops_per_s": ops / ((dens_ms + force_ms) / 1e3),
                "work_note": "mean of the window's first and last state (sphx_walk_stats); FP32 ops "
                             "= %d per r^2 test + %d per accepted pair (density %d, force %d)"
                             % (OPS_PER_TEST, OPS_PER_PAIR_DENSITY + OPS_PER_PAIR_FORCE,
                                OPS_PER_PAIR_DENSITY, OPS_PER_PAIR_FORCE)}
    sc.set_profiling(False)

    # e2e through the C-ABI with pinned host buffers: every step uploads the
    # state, steps (graph replay, as a user's handle does) and reads
    # positions and velocities back, from the timed window's first state.
    pin_pos = torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy()
    pin_vel = torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy()
    pin_pos[:] = st0["pos"]
    pin_vel[:] = st0["vel"]
    sc.close()
    sc = sphx.Scene(s, box, pin_pos, pin_vel,
                    sphx.default_options(device=device, reorder_interval=a.reorder, use_graph=1))
    e2e_steps = max(1, min(a.steps, 10))
    lib = sphx.lib()

    e2e_stream = torch.cuda.ExternalStream(sc.device_view().stream, device=device)

    def e2e_iteration():
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        t0 = time.perf_counter()
        sc.set_state(pin_pos, pin_vel)
        t1 = time.perf_counter()
        ev[0].record(e2e_stream)
        sc.step(sphx.DT, 1)
        ev[1].record(e2e_stream)
        sphx._check(lib.sphx_read_state(sc.h, sphx._ptr(pin_pos), sphx._ptr(pin_vel), None, None,
                                        None))
        return t1 - t0, time.perf_counter() - t1, ev[0].elapsed_time(ev[1])

    for _ in range(3):
        e2e_iteration()
    barrier()
    t0 = time.perf_counter()
    parts = [e2e_iteration() for _ in range(e2e_steps)]
    t_e2e = time.perf_counter() - t0
    barrier()
    t_e2e = max_over_ranks(t_e2e)
    sc.close()
    ceil = copy_ceiling(torch, 24 * n)
    step_ms = float(np.mean([p[2] for p in parts]))  # device time of the e2e steps themselves
    copy_ms = 1e3 * 24 * n * (1.0 / ceil["h2d_gbs"] + 1.0 / ceil["d2h_gbs"]) / 1e9
    e2e = {"value": n * e2e_steps * world / t_e2e, "unit": UNIT,
           "h2d_bytes_per_step": 24 * n, "d2h_bytes_per_step": 24 * n,
           "ms_per_step": 1e3 * t_e2e / e2e_steps,
           "upload_ms": 1e3 * float(np.mean([p[0] for p in parts])),
           "step_and_readout_ms": 1e3 * float(np.mean([p[1] for p in parts])),
           "device_step_ms": step_ms,
           "copy_ceiling": ceil,
           "bound_ms": step_ms + copy_ms,
           "bound_note": "device time of the e2e steps (CUDA events on the handle's stream) + 24 "
                         "B/particle each way at the measured single-copy pinned rates",
           "path": "sphx_set_state + sphx_step (graph replay) + sphx_read_state (pinned host buffers)"}

    # The configured runs (200 steps from the initial lattice): the fluid
    # clumps as it falls (the reference's physics at these constants), so
    # later steps cost more than the timed window above.  The headline block
    # and the 8M block, each at reorder intervals 1, 4, 16 and 64.
    peak_hbm = peaks()[0]
    config_run, sweep_8m, reorder_sweep = None, None, []
    if a.config_steps > 0:
        t_sec = time.perf_counter()
        for side in (SIDE, SIDE_8M):
            if side == SIDE:
                p_s, b_s = pos, box
            else:
                p_s, b_s = sphx.dambreak(side)
            for R in REORDER_SWEEP:
                r = configured_run(sphx, torch, s, b_s, p_s, device, a.config_steps, R,
                                   phases=(R == 1), peak=peak_hbm)
                r["particles"] = len(p_s)
                reorder_sweep.append({k: r[k] for k in ("particles", "reorder_interval", "ms_per_step",
                                                       "particle_steps_per_s")})
                if R == 1 and side == SIDE:
                    config_run = r
                if R == 1 and side == SIDE_8M:
                    sweep_8m = r
            del p_s, b_s
        sweep_s = time.perf_counter() - t_sec

    if rank != 0:
        return
    section_s = {"sweeps": round(sweep_s, 1) if a.config_steps > 0 else 0.0}
    t_sec = time.perf_counter()
    cpu = cpu_baseline(pos, box, s) if world == 1 and not a.no_cpu else None
    section_s["cpu_baseline"] = round(time.perf_counter() - t_sec, 1)
    batched = None
    if world == 1 and a.batch_steps > 0:
        t_sec = time.perf_counter()
        batched = batch_compare(sphx.batch_scenes(512, seed=0), a.batch_steps, 0, device)
        section_s["batched"] = round(time.perf_counter() - t_sec, 1)
    served = None
    if world == 1 and a.requests > 0 and a.served_rates:
        t_sec = time.perf_counter()
        served = serve_sweep(sphx, a.requests, [float(x) for x in a.served_rates.split(",")],
                             a.tick, device)
        section_s["served"] = round(time.perf_counter() - t_sec, 1)
    # state, ids, density, sort scratch, neighbour records and the list entries in use
    ws_mb = (n * (16 * 4 + 4 * 2 + 16 + 12 + 8 + 32) + 4 * pairs) / 1e6
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded SplitMix64 jittered lattice)",
            "config": {"workload": WORKLOAD, "reorder_interval": a.reorder,
                       "timed_window": "steps %d..%d of the run from the initial lattice" % (a.warmup, a.warmup + a.steps),
                       "l2": "inputs larger than L2: per-step working set %.0f MB > 129 MB, no flush" % ws_mb,
                       "parallelism": "replicas" if world > 1 else "single"},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "clocks": clk.summary(), "gpu_launches": int(kt.launches), "batched": batched,
            "config_run": config_run, "sweep_8m": sweep_8m, "reorder_sweep": reorder_sweep,
            "served": served, "section_s": section_s}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="sphx", choices=["sphx", "reference"])
    ap.add_argument("--workload", default="plain", choices=["plain", "batch", "serve", "steps"])
    ap.add_argument("--side", type=int, default=SIDE, help="block side of --workload steps")
    ap.add_argument("--scenes", type=int, default=0,
                    help="--workload steps: step the batched workload's first N scenes instead")
    ap.add_argument("--batch-steps", type=int, default=200,
                    help="steps of the batched-vs-sequential comparison in the plain run (0: skip)")
    ap.add_argument("--requests", type=int, default=64,
                    help="requests of the served comparison (0: skip it in the plain run)")
    ap.add_argument("--served-rates", default="50,200,1000,2000",
                    help="arrival rates of the served comparison in the plain run ('': skip)")
    ap.add_argument("--config-steps", type=int, default=200,
                    help="steps of the whole-configuration run reported as config_run (0: skip)")
    ap.add_argument("--rates", default="50,100,200,500,1000,2000")
    ap.add_argument("--tick", type=int, default=10)
    ap.add_argument("--reorder", type=int, default=1)
    ap.add_argument("--traffic", type=float, default=None,
                    help="ncu dram bytes per density+force step, if captured")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--ref-budget", type=float, default=120.0,
                    help="seconds after which the reference arm stops timing more steps")
    a = ap.parse_args()
    if a.impl == "reference":
        run_reference(a)
    elif a.workload == "batch":
        run_batch(a)
    elif a.workload == "serve":
        run_serve(a)
    elif a.workload == "steps":
        run_steps_only(a)
    else:
        run_sphx(a)


if __name__ == "__main__":
    main()
