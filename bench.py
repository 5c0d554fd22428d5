#!/usr/bin/env python
"""Benchmark: particle-updates/s of the gravity + SPH force evaluation at 1M particles.

Workload (default): 1,000,000 particles (500,000 gas + 500,000 dark matter), the seeded
synthetic disk + 1/r halo snapshot (galaxy_formation_gb300.synthetic, seed 3). One step =
one full force evaluation of every particle: Barnes-Hut tree build + group walk (theta 0.7,
eps 0.4 kpc, monopole, the reference's float32 arithmetic), full 48-candidate neighbour
search of the gas, smoothing lengths, SPH density + pressure/viscosity forces (float64)
and the time-step glue (simulation.py:61-95). One particle-update = one particle receiving
a freshly computed total acceleration.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

`value` is timed on the device with CUDA events around each step, inputs resident in HBM,
L2 flushed (256 MB write) between steps; `e2e` is the same metric through the C ABI with
host (pageable NumPy) buffers, copies in and out included. `--impl reference` times the
reference's CPU algorithm on this host's cores (the oracle restatement of cpp/nbody.cpp +
the reference's scipy cKDTree call + the restated SPH forces) on the same workload.
Multi-GPU (torchrun): independent replicas, one per GPU, no collective on the data path.
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

METRIC = "particle-updates/s at 1M (BH+SPH), mixed+learned vs plain GPU, p99 acc err≤1e-3"
UNIT = "particle-updates/s"
CONFIG_IDX = 2
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--scale", type=float, default=1.0, help="shrink the workload (testing only)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    return ap.parse_args()


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def allmax(world, x):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload(scale):
    from galaxy_formation_gb300 import synthetic

    return synthetic.make_config(CONFIG_IDX, seed=3, scale=scale)


def workload_name(n_gas, n_dm):
    return f"disk+halo snapshot, {n_gas:,} gas + {n_dm:,} DM, one full force evaluation"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.gpu)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_force_step(fo, d):
    fo.accelerations(d["pos"], d["vel"], d["mass"], d["kind"], d["u"], None, True, True, True)


def time_cpu(d, reps, warm):
    """The reference's algorithm on this host's CPU cores; returns seconds per step."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from force_ref import ForceOracle

    from galaxy_formation_gb300 import params

    oracle.build()
    fo = ForceOracle(len(d["mass"]), params.THETA, params.EPS)
    for _ in range(warm):
        cpu_force_step(fo, d)
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        cpu_force_step(fo, d)
        ts.append(time.perf_counter() - t0)
    return statistics.median(ts), oracle.num_threads()


def run_reference(args, world, rank):
    if rank != 0:
        return
    d = workload(args.scale)
    n = len(d["mass"])
    n_gas = int((d["kind"] == 0).sum())
    steps = max(1, min(args.steps, 5))
    warm = min(args.warmup, 1)
    sec, cores = time_cpu(d, steps, warm)
    v = n / sec
    sample = (f"{steps} full force evaluations of the {n:,}-particle workload (median), "
              f"{warm} warm-up; oracle restatement of cpp/nbody.cpp (OpenMP) + scipy cKDTree "
              f"(workers=-1) + restated sph_forces (OpenMP), numba absent")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": steps, "warmup": warm, "ms_per_step": sec * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32", "data": "synthetic",
        "config": {"workload": workload_name(n_gas, n - n_gas), "particles": n, "gas": n_gas,
                   "theta": 0.7, "eps_kpc": 0.4, "host_cores": os.cpu_count()},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def load_traffic():
    p = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


def run_gpu(args, world, rank, local):
    import torch

    from galaxy_formation_gb300 import _lib, build, params
    from galaxy_formation_gb300.engine import Engine

    build.build()
    lib = _lib.load()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    d = workload(args.scale)
    n = len(d["mass"])
    n_gas = int((d["kind"] == 0).sum())
    T = {k: torch.from_numpy(np.ascontiguousarray(d[k])).to(dev) for k in ("pos", "vel", "mass", "kind", "u")}
    acc = torch.empty((n, 3), dtype=torch.float64, device=dev)
    dt_ind = torch.empty(n, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > L2

    def step():
        st = lib.gf_accelerations_dev(n, T["pos"].data_ptr(), T["vel"].data_ptr(), T["mass"].data_ptr(),
                                      T["kind"].data_ptr(), T["u"].data_ptr(), params.THETA, params.EPS,
                                      params.GAMMA, params.ALPHA, params.BETA, None, 1, 1, 1,
                                      acc.data_ptr(), dt_ind.data_ptr(), stream.cuda_stream)
        if st:
            _lib.check(st)

    for _ in range(args.warmup):
        step()
        flush.zero_()
    torch.cuda.synchronize()
    barrier(world)

    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    gpu_index = vis.split(",")[local] if vis else str(local)
    clocks = ClockSampler(gpu_index)
    lib.gf_profile(1)
    launches0 = lib.gf_launch_count()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    torch.cuda.synchronize()
    clocks.start()
    for e0, e1 in evs:
        e0.record(stream)
        step()
        e1.record(stream)
        flush.zero_()
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier(world)
    launches = lib.gf_launch_count() - launches0
    times = [e0.elapsed_time(e1) for e0, e1 in evs]
    total_ms = allmax(world, sum(times))
    ms_per_step = total_ms / args.steps
    value = world * n / (ms_per_step * 1e-3)

    import ctypes

    stages = {}
    for i, name in enumerate(_lib.STAGES):
        ms, cnt = ctypes.c_double(), ctypes.c_int()
        lib.gf_profile_stage(i, ctypes.byref(ms), ctypes.byref(cnt))
        if cnt.value:
            stages[name] = {"ms_per_launch": ms.value / cnt.value, "launches": cnt.value}
    lib.gf_profile(0)
    pairs = lib.gf_walk_pairs()
    info = [ctypes.c_int(), ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()]
    lib.gf_force_info(*[ctypes.byref(x) for x in info])

    if rank != 0:
        return

    # roofline of the dominant kernel
    peaks = json.load(open(PEAKS)) if os.path.exists(PEAKS) else {}
    hbm = peaks.get("hbm_gbs", 6800.0)
    hbm_src = "measured (MEASURED_PEAKS.json)" if "hbm_gbs" in peaks else "fallback"
    fp32 = ctypes.c_double()
    lib.gf_fp32_peak(ctypes.byref(fp32))
    kernel_stages = {k: v for k, v in stages.items() if k in ("walk", "knn", "sph_density", "sph_force", "verlet")}
    dom = max(kernel_stages, key=lambda k: kernel_stages[k]["ms_per_launch"] * kernel_stages[k]["launches"])
    t_launch = kernel_stages[dom]["ms_per_launch"] * 1e-3
    # algorithmic work per launch (unit figures are stated in the design doc)
    bytes_per_gas = {"knn": 24 + 48 * 4 + 8, "sph_density": 32 * 4 + 24 + 8 + 8 + 8,
                     "sph_force": 32 * 4 + 24 + 24 + 8 + 8 + 8 + 8 + 8 + 24 + 8 + 8, "verlet": 48 * 4 + 24 + 32 * 4 + 8}
    traffic_db = load_traffic()
    traffic = traffic_db.get(dom, {}).get("bytes_per_launch") if traffic_db.get("particles") == n else None
    if dom == "walk":
        work = 20.0 * pairs
        achieved = work / t_launch / 1e12
        roof = {"kernel": "k_walk_mono", "bound": "fp32", "achieved": achieved, "peak": fp32.value,
                "unit": "TFLOP/s", "frac": achieved / fp32.value, "traffic": traffic,
                "peak_source": "measured float32 FFMA throughput of this GPU (gf_fp32_peak)",
                "work_per_launch": {"pair_interactions": pairs, "flops_per_pair": 20}}
    else:
        work = bytes_per_gas[dom] * n_gas
        achieved = work / t_launch / 1e9
        roof = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "traffic": traffic, "peak_source": hbm_src,
                "work_per_launch": {"bytes": work, "bytes_per_gas_particle": bytes_per_gas[dom]}}

    # accuracy of the gravity against the float64 direct sum (2000 random targets)
    eng = Engine()
    agrav = np.zeros_like(d["pos"])
    eng.gravity(d["pos"], d["mass"], agrav, params.THETA, params.EPS)
    tgt = np.random.default_rng(11).choice(n, 2000, replace=False)
    exact = eng.gravity_direct_targets(d["pos"], d["mass"], tgt, params.EPS)
    err = np.linalg.norm(agrav[tgt] - exact, axis=1) / np.linalg.norm(exact, axis=1)

    e2e = None
    if not args.no_e2e:
        host = {k: np.ascontiguousarray(d[k]) for k in ("pos", "vel", "mass", "kind", "u")}
        a_h = np.empty((n, 3))
        dt_h = np.empty(n)

        def host_step():
            st = lib.gf_accelerations(n, host["pos"], host["vel"], host["mass"], host["kind"], host["u"],
                                      params.THETA, params.EPS, params.GAMMA, params.ALPHA, params.BETA,
                                      None, 1, 1, 1, a_h, dt_h)
            if st:
                _lib.check(st)

        host_step()
        ts = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            host_step()
            ts.append(time.perf_counter() - t0)
        e2e = {"value": world * n / statistics.mean(ts), "unit": UNIT,
               "h2d_bytes_per_step": n * (24 + 24 + 8 + 1 + 8), "d2h_bytes_per_step": n * (24 + 8),
               "ms_per_step": statistics.mean(ts) * 1e3}

    cpu = None
    if world == 1 and not args.no_cpu:
        sec, cores = time_cpu(d, 3, 1)
        cpu = {"value": n / sec, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"3 full force evaluations of the {n:,}-particle workload (median) after 1 "
                         "warm-up: oracle restatement of cpp/nbody.cpp (OpenMP) + scipy cKDTree "
                         "(workers=-1) + restated sph_forces (OpenMP)"}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 gravity + f64 SPH", "data": "synthetic",
        "config": {"workload": workload_name(n_gas, n - n_gas), "particles": n, "gas": n_gas,
                   "theta": params.THETA, "eps_kpc": params.EPS_KPC, "form": "plain (reference arithmetic)",
                   "l2": "flushed between steps (256 MB write)", "parallelism": f"replicas x{world}"},
        "roofline": roof,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clk,
        "stages_ms": {k: round(v["ms_per_launch"], 4) for k, v in stages.items()},
        "accuracy": {"grav_p99_rel_err_vs_f64_direct": float(np.percentile(err, 99)),
                     "grav_median": float(np.median(err)), "targets": 2000},
        "knn_iterations_per_gas": info[3].value / max(1, info[0].value),
        "walk": {"pair_interactions": pairs,
                 "tflops": 20.0 * pairs / (stages["walk"]["ms_per_launch"] * 1e-3) / 1e12
                 if "walk" in stages else None, "fp32_peak_tflops": fp32.value},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_gpu(args, world, rank, local)


if __name__ == "__main__":
    main()
