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
                 "--format=csv,noheader,nounits", "-lms", "100"],
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


def run_reference(a):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    pos, box, s = workload()
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    pyoracle.build()
    port = pyoracle.Port()
    import sphx
    args = sphx.args_array(s)
    p, v = pos, None
    for _ in range(a.warmup):
        p, v, _, _ = port.run(p, v, args, sphx.DT, 1, box=box.as_array())
    # each step is one full-workload step; the loop stops early once the
    # budget is spent so that a large --steps still ends within minutes
    t0 = time.perf_counter()
    done = 0
    while done < a.steps and (done == 0 or time.perf_counter() - t0 < a.ref_budget):
        p, v, _, _ = port.run(p, v, args, sphx.DT, 1, box=box.as_array())
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
    ms = e0.elapsed_time(e1)
    kt = sc.kernel_times()
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = n * a.steps * world / (ms / 1e3)

    peak, peak_kind = peaks()
    dens_ms = kt.density_ms / max(kt.steps, 1)
    force_ms = kt.force_ms / max(kt.steps, 1)
    achieved = ALGO_BYTES * n / ((dens_ms + force_ms) / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_kind": peak_kind,
                "traffic": a.traffic, "kernels": "k_density + k_force",
                "per_step_ms": {"sort": kt.sort_ms / max(kt.steps, 1), "density": dens_ms,
                                "force": force_ms}}
    sc.set_profiling(False)

    # e2e through the C-ABI with pinned host buffers
    pin_pos = torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy()
    pin_vel = torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy()
    st = sc.read()
    pin_pos[:] = st["pos"]
    pin_vel[:] = st["vel"]
    e2e_steps = max(1, min(a.steps, 10))
    for _ in range(2):
        sc.set_state(pin_pos, pin_vel)
        sc.step(sphx.DT, 1)
        sphx._check(sphx.lib().sphx_read_state(sc.h, sphx._ptr(pin_pos), sphx._ptr(pin_vel),
                                               None, None, None))
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        sc.set_state(pin_pos, pin_vel)
        sc.step(sphx.DT, 1)
        sphx._check(sphx.lib().sphx_read_state(sc.h, sphx._ptr(pin_pos), sphx._ptr(pin_vel),
                                               None, None, None))
    t_e2e = time.perf_counter() - t0
    barrier()
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([t_e2e], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_e2e = float(t.item())
    e2e = {"value": n * e2e_steps * world / t_e2e, "unit": UNIT,
           "h2d_bytes_per_step": 24 * n, "d2h_bytes_per_step": 24 * n,
           "path": "sphx_set_state + sphx_step + sphx_read_state (pinned host buffers)"}
    sc.close()

    if rank != 0:
        return
    cpu = cpu_baseline(pos, box, s) if world == 1 and not a.no_cpu else None
    ws_mb = n * (16 * 4 + 4 * 2 + 8 + 16 + 12) / 1e6
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded SplitMix64 jittered lattice)",
            "config": {"workload": WORKLOAD, "reorder_interval": a.reorder,
                       "l2": "inputs larger than L2: per-step working set %.0f MB > 129 MB, no flush" % ws_mb,
                       "parallelism": "replicas" if world > 1 else "single"},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "clocks": clk.summary(), "gpu_launches": int(kt.launches)}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="sphx", choices=["sphx", "reference"])
    ap.add_argument("--reorder", type=int, default=1)
    ap.add_argument("--traffic", type=float, default=None,
                    help="ncu dram bytes per density+force step, if captured")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--ref-budget", type=float, default=120.0,
                    help="seconds after which the reference arm stops timing more steps")
    a = ap.parse_args()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_sphx(a)


if __name__ == "__main__":
    main()
