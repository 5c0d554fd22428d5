#!/usr/bin/env python
"""Benchmark: particle-updates/s of the gravity + SPH force evaluation at 1M particles.

Workload: 1,000,000 particles (500,000 gas + 500,000 dark matter), the seeded synthetic disk +
1/r halo snapshot (galaxy_formation_gb300.synthetic, seed 3), eps 0.4 kpc. One step = one full
force evaluation of every particle: Barnes-Hut tree build + group walk, full 48-candidate
neighbour search of the gas, smoothing lengths, SPH density + pressure/viscosity forces and
the time-step glue (simulation.py:61-95). One particle-update = one particle receiving a
freshly computed total acceleration.

Forms measured (same snapshot, same evaluation):
  plain          the reference's arithmetic: float32 monopole walk at theta 0.7 (its
                 default), float64 SPH, search radius from the previous h;
  plain_matched  the same arithmetic at the opening angle whose gravity error against the
                 float64 direct sum meets p99 <= 1e-3 (theta 0.15);
  mixed_learned  the headline: float32 walk with Kahan tile sums and quadrupole nodes under the
                 relative opening criterion (alpha 4e-3, a geometric floor at theta 1; accepted
                 nodes whose quadrupole term is below 1.5e-4 a_min taken as monopoles; walk items
                 merged from sibling groups up to 40 particles), p99 <= 1e-3 against the float64
                 direct sum; float32 + Kahan SPH; search radius from 2.5 x the previous h, and
                 from the learned MLP guess (trained first on pairs the simulator produced, on
                 the GPU) for searches without a previous h;
plus the batched form (block time steps, CUDA-graph replay, autotuned) as particle-updates/s
over a 64-sub-step block.

`value` = mixed_learned, timed on the device with CUDA events on the launching stream around
each step, inputs resident in HBM, L2 flushed (256 MB write) between steps; `e2e` = the same
form through the C ABI with pinned host buffers (copies in and out included); `parity` = the
GPU forms against the oracle's evaluation of the same snapshot (computed by the cpu_baseline
leg, which runs the oracle anyway). `--impl reference`
times the reference's CPU algorithm on this host's cores (the oracle restatement of
cpp/nbody.cpp + scipy cKDTree + the restated sph_forces) on the same workload.
Multi-GPU (torchrun): independent replicas, one per GPU, no collective on the data path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]
"""

import argparse
import ctypes
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

# theta, quadrupole gravity, float32 SPH, h guess (0 previous h, 2 learned), relative opening
# tolerance (0: geometric criterion at theta; > 0: the relative criterion once every particle
# has a previous gravity, with theta used for the first evaluation), walk items merged from
# sibling groups up to this many particles (0: the reference's groups), monopole tolerance of
# accepted nodes (0: every accepted node to quadrupole order)
FORMS = {
    "plain": (0.7, 0, 0, 0, 0.0, 0, 0.0),
    "plain_matched": (0.15, 0, 0, 0, 0.0, 0, 0.0),
    "mixed_learned": (0.55, 1, 1, 2, 4e-3, 40, 1.5e-4),
}
# flops per interaction (an FMA counting 2): monopole pair (cpp/nbody.cpp:398-402 in float32)
# and the softened quadrupole node term of the mixed walk
FLOPS_MONO, FLOPS_QUAD = 20, 57


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--scale", type=float, default=1.0, help="shrink the workload (testing only)")
    ap.add_argument("--forms", default="plain,plain_matched,mixed_learned",
                    help="comma list of forms to time (the last one given is the headline)")
    ap.add_argument("--blocks", type=int, default=3, help="64-sub-step blocks of the batched form (0: skip)")
    ap.add_argument("--workload", default="force", choices=["force", "drift", "learned"],
                    help="force: the headline (one full evaluation, 1M disk+halo); drift: 4M cloud, "
                         "plain step loop vs batched mixed+learned blocks over the same simulated time, "
                         "energy and angular-momentum drift; learned: 1M gas with clumps, search "
                         "iterations with and without the learned guess")
    ap.add_argument("--no-configs", dest="configs", action="store_false",
                    help="skip the shortened config 3 (clumped snapshot) and config 4 (4M drift) measurements")
    ap.add_argument("--drift-steps", type=int, default=10, help="long steps of the plain loop in the 4M drift run")
    ap.add_argument("--block-config", default="",
                    help="walk item code per bin and rebuild cadence of the batched form, e.g. "
                         "'104,180,0,0,0,0:8', instead of the autotuner's choice (for profiles)")
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


def workload(scale, idx=CONFIG_IDX):
    from galaxy_formation_gb300 import synthetic

    return synthetic.make_config(idx, seed=3, scale=scale)


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
    """The reference's algorithm on this host's CPU cores; returns seconds per step, the
    threads used and the oracle holding the last evaluation (the checker of the GPU forms)."""
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
    return statistics.median(ts), oracle.num_threads(), fo


def parity_vs_oracle(G, fo, head):
    """The GPU forms against the oracle's evaluation of the same snapshot (the CPU leg's last
    step): the plain form's gravity against the oracle's Barnes-Hut at theta 0.7 (per-particle
    relative error), and the headline form's SPH against the oracle's float64 SPH — neighbour
    sets, h, density, Courant step, SPH acceleration and du/dt (the last two also relative to
    the sum of |pair terms|, the scale that bounds the rounding of a cancelling sum)."""
    import sph_ref

    torch, lib, L, params = G.torch, G.lib, G._lib, G.params
    out = {"oracle": "ForceOracle: restated cpp/nbody.cpp Barnes-Hut at theta 0.7 + scipy cKDTree 48-candidate "
                     "search + restated sph_forces (float64), same snapshot"}
    theta = G.set_form("plain")
    G.step(theta, kind=torch_full_like(torch, G.T["kind"], 2))
    e = np.linalg.norm(G.acc.cpu().numpy() - fo.acc_grav, axis=1) / np.linalg.norm(fo.acc_grav, axis=1)
    out["plain_gravity_vs_oracle_bh"] = {"p99_rel_err": float(np.percentile(e, 99)), "max_rel_err": float(e.max()),
                                         "median_rel_err": float(np.median(e)), "bar_p99": 1e-4}
    theta = G.set_form(head)
    G.step(theta)
    G.step(theta)  # the relative criterion's error scale is the previous evaluation's gravity
    torch.cuda.synchronize()
    gs = L.read_gas(lib)
    g = fo.gas_idx
    p, v, m, u = (np.ascontiguousarray(G.d[k][g]) for k in ("pos", "vel", "mass", "u"))
    sa, sd = np.empty(g.size), np.empty(g.size)
    for s0 in range(0, g.size, 100_000):
        rows = np.arange(s0, min(g.size, s0 + 100_000))
        _, _, _, sa[rows], sd[rows] = sph_ref.forces(p, v, m, fo.nb, fo.h, u, fo.rho, rows, params.GAMMA,
                                                     params.ALPHA, params.BETA)
    a, b = np.sort(gs["nb"].astype(np.int64), axis=1), np.sort(fo.nb, axis=1)
    bad = np.flatnonzero(np.any(a != b, axis=1))
    edge = 0
    for i in bad:
        diff = np.setxor1d(a[i], b[i])
        r = np.linalg.norm(p[diff] - p[i], axis=1)
        edge += int(np.all(np.abs(r - 2 * fo.h[i]) <= 1e-6 * fo.h[i]))
    dti = fo.dt_courant[g]
    a_sph = fo.acc_sph[g]
    err = np.linalg.norm(gs["acc_sph"] - a_sph, axis=1)
    out["headline_sph_vs_oracle_f64"] = {
        "form": head, "gas": int(g.size),
        "gas_index_identical": bool(np.array_equal(gs["gidx"], g)),
        "neighbour_rows_differing": int(bad.size), "of_which_at_support_edge": edge,
        "h_max_rel_diff": float(np.max(np.abs(gs["h"] - fo.h) / fo.h)),
        "rho_max_rel_err": float(np.max(np.abs(gs["rho"] - fo.rho) / fo.rho)),
        "dt_max_rel_err": float(np.max(np.abs(gs["dt_i"] - dti) / dti)),
        "acc_sph_p99_rel_err": float(np.percentile(err / np.linalg.norm(a_sph, axis=1), 99)),
        "acc_sph_max_err_over_term_sum": float(np.max(err / sa)),
        "dudt_max_err_over_term_sum": float(np.max(np.abs(gs["dudt"] - fo.dudt) / sd)),
        "bar": 1e-5}
    return out


def run_reference(args, world, rank):
    if rank != 0:
        return
    d = workload(args.scale)
    n = len(d["mass"])
    n_gas = int((d["kind"] == 0).sum())
    steps = max(1, args.steps)
    warm = args.warmup
    sec, cores, _ = time_cpu(d, steps, warm)
    v = n / sec
    sample = (f"{steps} full force evaluations of the {n:,}-particle workload (median), "
              f"{warm} warm-up; oracle restatement of cpp/nbody.cpp (OpenMP) + scipy cKDTree "
              f"(workers=-1) + restated sph_forces (OpenMP), numba absent")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": steps, "warmup": warm, "ms_per_step": sec * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32", "data": "synthetic",
        "config": {"workload": workload_name(n_gas, n - n_gas), "particles": n, "gas": n_gas,
                   "theta": 0.7, "eps_kpc": 0.4, "host_cores": os.cpu_count(),
                   "note": "the reference's method: geometric opening at theta 0.7 (float32 monopole walk) and "
                           "float64 SPH; the GPU headline runs the relative opening criterion with quadrupoles "
                           "(p99 <= 1e-3 against the float64 direct sum, which theta 0.7 misses) and float32 + "
                           "Kahan SPH, so the two arms compute the same evaluation by different methods"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def load_traffic():
    p = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


class Gpu:
    """The workload resident on one GPU and the library's entry points around it."""

    def __init__(self, args, local, config_idx=CONFIG_IDX, ic="host"):
        import torch

        from galaxy_formation_gb300 import _lib, build, params, synthetic

        build.build()
        self.torch, self._lib, self.params = torch, _lib, params
        self.lib = _lib.load()
        torch.cuda.set_device(local)
        self.dev = torch.device("cuda", local)
        t0 = time.perf_counter()
        if ic == "device":  # drawn on the GPU (gf_ic_generate), copied to the host once
            self.d = synthetic.make_config_device(config_idx, seed=3, scale=args.scale, lib=self.lib)
        else:
            self.d = workload(args.scale, config_idx)
        self.ic = {"generator": ic, "seconds": time.perf_counter() - t0}
        self.n = len(self.d["mass"])
        self.n_gas = int((self.d["kind"] == 0).sum())
        self.T = {k: torch.from_numpy(np.ascontiguousarray(self.d[k])).to(self.dev)
                  for k in ("pos", "vel", "mass", "kind", "u")}
        self.acc = torch.empty((self.n, 3), dtype=torch.float64, device=self.dev)
        self.dt = torch.empty(self.n, dtype=torch.float64, device=self.dev)
        # a stream of its own: the library orders its work on the handle it is given, and the
        # CUDA events bracketing a step are recorded on the same stream
        self.stream = torch.cuda.Stream(self.dev)
        torch.cuda.set_stream(self.stream)
        self.flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=self.dev)  # 256 MB > L2

    def set_form(self, form):
        theta, quad, sph32, hguess, rel, merge, relq = FORMS[form]
        L, lib = self._lib, self.lib
        tuned = getattr(self, "tuned", {}).get(form)
        if tuned:  # the walk autotuner's choice for this form (time_form)
            merge = tuned["walk_merge"]
        lib.gf_set_option(L.OPT_WALK_SHAPE, tuned["walk_shape"] if tuned else 0)
        lib.gf_set_option(L.OPT_GRAVITY_QUAD, quad)
        lib.gf_set_option(L.OPT_SPH_FLOAT32, sph32)
        lib.gf_set_option(L.OPT_HGUESS, hguess)
        lib.gf_set_option(L.OPT_GRAVITY_REL, rel)  # the next evaluation sets the error scale
        lib.gf_set_option(L.OPT_WALK_MERGE, merge)
        lib.gf_set_option(L.OPT_GRAVITY_REL_MONO, relq)
        return theta

    def step(self, theta, pos=None, kind=None, sph=1):
        T, p = self.T, self.params
        st = self.lib.gf_accelerations_dev(
            self.n, (pos if pos is not None else T["pos"]).data_ptr(), T["vel"].data_ptr(), T["mass"].data_ptr(),
            (kind if kind is not None else T["kind"]).data_ptr(), T["u"].data_ptr(), theta, p.EPS, p.GAMMA,
            p.ALPHA, p.BETA, None, 1, sph, 1, self.acc.data_ptr(), self.dt.data_ptr(), self.stream.cuda_stream)
        if st:
            self._lib.check(st)

    def knn_iters(self):
        info = [ctypes.c_int(), ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()]
        self.lib.gf_force_info(*[ctypes.byref(x) for x in info])
        return info[3].value / max(1, info[0].value)

    def time_form(self, form, steps, warmup):
        """Device time of `steps` evaluations (CUDA events on the launching stream, L2 flushed
        between steps), stages, launches, walk interactions."""
        torch, lib, L = self.torch, self.lib, self._lib
        theta = self.set_form(form)
        for _ in range(warmup):
            self.step(theta)
            self.flush.zero_()
        torch.cuda.synchronize()
        tuned = None
        if FORMS[form][1]:  # mixed walk: item size and launch shape chosen by the autotuner
            mg, sh, wms = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
            L.check(lib.gf_force_autotune(self.params.EPS, ctypes.byref(mg), ctypes.byref(sh), ctypes.byref(wms)))
            tuned = {"walk_merge": mg.value, "walk_shape": sh.value, "walk_ms": wms.value}
            if not hasattr(self, "tuned"):
                self.tuned = {}
            self.tuned[form] = tuned
            self.step(theta)
            torch.cuda.synchronize()
        lib.gf_profile(1)
        launches0 = lib.gf_launch_count()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        torch.cuda.synchronize()
        for e0, e1 in evs:
            e0.record(self.stream)
            self.step(theta)
            e1.record(self.stream)
            self.flush.zero_()
        torch.cuda.synchronize()
        launches = lib.gf_launch_count() - launches0
        times = [e0.elapsed_time(e1) for e0, e1 in evs]
        stages = {}
        for i, name in enumerate(L.STAGES):
            ms, cnt = ctypes.c_double(), ctypes.c_int()
            lib.gf_profile_stage(i, ctypes.byref(ms), ctypes.byref(cnt))
            if cnt.value:
                stages[name] = {"ms_per_launch": ms.value / cnt.value, "launches": cnt.value}
        # the gravity chain alone (no hydro stream beside it): what its stages cost without the
        # contention of the neighbour search for the SMs (the step's stage times include it)
        lib.gf_profile(1)
        for _ in range(3):
            self.step(theta, sph=0)
            self.flush.zero_()
        torch.cuda.synchronize()
        alone = {}
        for name in ("tree_build", "tree_sort", "tree_emit", "tree_moments", "group_prep", "walk"):
            ms, cnt = ctypes.c_double(), ctypes.c_int()
            lib.gf_profile_stage(L.STAGES.index(name), ctypes.byref(ms), ctypes.byref(cnt))
            if cnt.value:
                alone[name] = ms.value / cnt.value
        lib.gf_profile(0)
        st = np.zeros(9)
        lib.gf_force_stats(st, 9)
        return {"theta": theta, "times_ms": times, "launches": launches, "stages": stages, "gravity_alone": alone,
                "pairs": lib.gf_walk_pairs(), "qpairs": lib.gf_walk_quad_pairs(), "knn_iters": self.knn_iters(),
                "nodes": int(st[8]), "autotune": tuned}

    def gravity_error(self, form, targets, exact):
        """p99 / median relative error of the form's gravity against the float64 direct sum:
        the fused evaluation with every particle flagged dark matter (no hydro term)."""
        theta = self.set_form(form)
        dm = torch_full_like(self.torch, self.T["kind"], 2)
        # twice: the relative criterion takes its error scale from the previous evaluation,
        # as in every timed step
        self.step(theta, kind=dm)
        self.step(theta, kind=dm)
        a = self.acc.cpu().numpy()[targets]
        e = np.linalg.norm(a - exact, axis=1) / np.linalg.norm(exact, axis=1)
        return float(np.percentile(e, 99)), float(np.median(e))

    def collect_pairs(self, rows, collect_steps=4, start=True):
        """(features, log distance of the 48th nearest) pairs from the plain method's own evaluations of drifting
        copies of the snapshot (the collection buffer is cleared when start)."""
        torch, lib, L = self.torch, self.lib, self._lib
        theta = self.set_form("plain")
        lib.gf_set_option(L.OPT_HGUESS, 0)
        pos = self.T["pos"].clone()
        self.step(theta, pos=pos)
        if start:
            lib.gf_set_option(L.OPT_COLLECT, rows)
        for _ in range(collect_steps):
            pos += 0.5 * self.dt[:, None] * self.T["vel"]
            self.step(theta, pos=pos)
        torch.cuda.synchronize()
        return pos

    def train_hguess(self, rows=2_000_000, collect_steps=4, collected=False):
        """Learned smoothing-length guess: pairs collected from the simulator (unless already
        collected), then Adam on the GPU; iteration counts on a drifted snapshot."""
        torch, lib, L = self.torch, self.lib, self._lib
        theta = self.set_form("plain")
        pos = self.T["pos"].clone() if collected else self.collect_pairs(rows, collect_steps)
        m = lib.gf_mlp_collected(None, None, 0)
        X = np.zeros((m, 4), np.float32)
        Y = np.zeros(m, np.float32)
        lib.gf_mlp_collected(X.ctypes.data, Y.ctypes.data, m)
        L.check(lib.gf_mlp_init(7))
        mu, sd = X.mean(0), X.std(0) + 1e-6
        L.check(lib.gf_mlp_set_norm(mu.astype(np.float32), sd.astype(np.float32), float(Y.mean()), float(Y.std())))
        loss0, loss1 = ctypes.c_double(), ctypes.c_double()
        t0 = time.perf_counter()
        L.check(lib.gf_mlp_train(1, 4096, 1e-3, ctypes.byref(loss0)))
        L.check(lib.gf_mlp_train(2000, 4096, 2e-3, ctypes.byref(loss1)))
        train_s = time.perf_counter() - t0
        lib.gf_set_option(L.OPT_COLLECT, 0)  # stop collecting (clears the pairs)
        # the first search of a snapshot (no previous h): cell density vs the learned guess;
        # with a previous h (the snapshot drifted by 1, 4, 16 half steps since it was taken)
        # the start is 2.5 h in both modes; the converged neighbours are the same in all
        cold = {name: self.search_without_h(theta, pos, mode) for mode, name in ((1, "cell_density"),
                                                                                  (2, "learned"))}
        by_drift = {f"{halves}_half_steps": {"previous_h": self.search_after_drift(theta, pos, halves, 0)}
                    for halves in (1, 4, 16)}
        lib.gf_set_option(L.OPT_HGUESS, 0)
        return {"training_rows": int(m), "loss_start": loss0.value, "loss_end": loss1.value,
                "train_s": train_s, "adam_steps": 2000, "batch": 4096,
                "first_search_without_previous_h": cold,
                "search_with_previous_h_after_drift": by_drift,
                "note": "the learned guess starts searches without a previous h; where one exists, 2.5 h "
                        "starts them (fewer iterations than the network's guess: 1.04 against 1.11)"}

    def search_without_h(self, theta, pos, mode):
        """Radius iterations and neighbour-search time of a full search that has no previous h,
        started from h guess `mode` (1 the cell density, 2 the learned guess)."""
        torch, lib, L = self.torch, self.lib, self._lib
        lib.gf_set_option(L.OPT_HGUESS, mode)
        lib.gf_set_option(L.OPT_FORGET_H, 1)
        lib.gf_profile(1)
        self.step(theta, pos=pos)
        torch.cuda.synchronize()
        ms, cnt = ctypes.c_double(), ctypes.c_int()
        lib.gf_profile_stage(L.STAGES.index("knn"), ctypes.byref(ms), ctypes.byref(cnt))
        lib.gf_profile(0)
        return {"iterations_per_gas": self.knn_iters(), "knn_ms": ms.value}

    def search_after_drift(self, theta, pos, halves, mode):
        """Radius iterations and neighbour-search time of a full search on the snapshot drifted by
        `halves` half time steps (dt of each particle's last evaluation), starting from h guess
        `mode`, with the previous h from an evaluation before the drift."""
        torch, lib, L = self.torch, self.lib, self._lib
        lib.gf_set_option(L.OPT_HGUESS, 0)
        self.step(theta, pos=pos)
        nxt = pos + (0.5 * halves) * self.dt[:, None] * self.T["vel"]
        lib.gf_set_option(L.OPT_HGUESS, mode)
        lib.gf_profile(1)
        self.step(theta, pos=nxt)
        torch.cuda.synchronize()
        ms, cnt = ctypes.c_double(), ctypes.c_int()
        lib.gf_profile_stage(L.STAGES.index("knn"), ctypes.byref(ms), ctypes.byref(cnt))
        lib.gf_profile(0)
        return {"iterations_per_gas": self.knn_iters(), "knn_ms": ms.value}

    def step_loop(self, form, steps):
        """The reference's step loop (gf_sim_step) in `form` for `steps` long steps from the
        snapshot: particle-updates/s and the simulated time covered."""
        torch, lib, L, p = self.torch, self.lib, self._lib, self.params
        theta = self.set_form(form)
        d = self.d
        L.check(lib.gf_sim_init(self.n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], theta, p.EPS,
                                p.GAMMA, p.ALPHA, p.BETA))
        s = torch.cuda.ExternalStream(lib.gf_stream())
        tk, sub = ctypes.c_double(), ctypes.c_int()
        L.check(lib.gf_sim_step(1e30, ctypes.byref(tk), ctypes.byref(sub)))  # warm-up
        t0 = ctypes.c_double()
        L.check(lib.gf_sim_read(None, None, None, None, ctypes.byref(t0)))
        tk0 = t0.value
        upd, subs = 0.0, 0
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(steps):
            L.check(lib.gf_sim_step(1e30, ctypes.byref(tk), ctypes.byref(sub)))
            upd += lib.gf_sim_updates()
            subs += sub.value
        e1.record(s)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        t1 = ctypes.c_double()
        L.check(lib.gf_sim_read(None, None, None, None, ctypes.byref(t1)))
        return {"value": upd / (ms * 1e-3), "unit": UNIT, "form": form, "steps": steps, "substeps": subs,
                "updates": upd, "ms": ms, "simulated_time": t1.value - tk0,
                "simulated_time_per_wall_second": (t1.value - tk0) / (ms * 1e-3),
                "note": "simulation.py:114-149 on the GPU: per sub-step the gravity of the fast particles on a "
                        "refitted tree and the SPH of all the gas"}

    def batched(self, blocks, nlev=7, form="mixed_learned", plain_steps=10, config=""):
        """Block time steps at the mixed + learned form: autotune (or the given configuration:
        'codes:rebuild_every'), one warm block, then `blocks` blocks timed with CUDA events on
        the library's stream."""
        torch, lib, L, p = self.torch, self.lib, self._lib, self.params
        theta = self.set_form(form)
        d = self.d
        L.check(lib.gf_sim_init(self.n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], theta, p.EPS,
                                p.GAMMA, p.ALPHA, p.BETA))
        chunk = np.zeros(nlev - 1, np.int32)
        every, gms = ctypes.c_int(), ctypes.c_double()
        t0 = time.perf_counter()
        if config:
            codes, _, reb = config.partition(":")
            chunk[:] = [int(x) for x in codes.split(",")]
            every.value = int(reb or 8)
            L.check(lib.gf_sim_block_config(chunk.ctypes.data, len(chunk), every.value))
        else:
            L.check(lib.gf_sim_block_autotune(nlev, chunk.ctypes.data, ctypes.byref(every), ctypes.byref(gms)))
        tune_s = time.perf_counter() - t0
        upd = ctypes.c_double()
        L.check(lib.gf_sim_blocks(1, nlev, ctypes.byref(upd)))
        frac = np.zeros(nlev)
        L.check(lib.gf_sim_levels(nlev, frac))
        s = torch.cuda.ExternalStream(lib.gf_stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        launches0 = lib.gf_launch_count()
        tb0 = ctypes.c_double()
        L.check(lib.gf_sim_read(None, None, None, None, ctypes.byref(tb0)))
        torch.cuda.nvtx.range_push("blocks")  # for profilers: the timed blocks only
        e0.record(s)
        L.check(lib.gf_sim_blocks(blocks, nlev, ctypes.byref(upd)))
        e1.record(s)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        ms = e0.elapsed_time(e1)
        launches = lib.gf_launch_count() - launches0
        tb1 = ctypes.c_double()
        L.check(lib.gf_sim_read(None, None, None, None, ctypes.byref(tb1)))
        sim_rate = (tb1.value - tb0.value) / (ms * 1e-3)
        # the full neighbour search of a block end (the previous h of the coarse levels' gas is
        # a block old there): one more block with the stage profiler on
        lib.gf_profile(1)
        L.check(lib.gf_sim_blocks(1, nlev, ctypes.byref(ctypes.c_double())))
        torch.cuda.synchronize()
        kms, kcnt = ctypes.c_double(), ctypes.c_int()
        lib.gf_profile_stage(L.STAGES.index("knn"), ctypes.byref(kms), ctypes.byref(kcnt))
        lib.gf_profile(0)
        block_end = {"knn_ms": kms.value / max(1, kcnt.value), "iterations_per_gas": self.knn_iters(),
                     "h_guess": ["previous h", "cell density", "previous h (learned MLP without one)"][FORMS[form][3]]}
        # the plain GPU form of the same hierarchical time stepping: the reference's step loop
        # (simulation.py:114-149: gravity of the fast particles on a refitted tree and SPH of all
        # the gas at every sub-step) with the reference's arithmetic, from the same snapshot
        plain = self.step_loop("plain", plain_steps)
        self.set_form(form)
        value = upd.value / (ms * 1e-3)
        return {"value": value, "unit": UNIT, "blocks": blocks, "substeps_per_block": 1 << (nlev - 1),
                "levels": nlev, "level_fractions": [round(float(x), 5) for x in frac],
                "updates": upd.value, "ms": ms, "ms_per_block": ms / blocks,
                "autotune": {"chunk_per_bin": chunk.tolist(), "rebuild_every": every.value, "seconds": tune_s,
                             "given": bool(config)},
                "launches_outside_graphs": launches, "block_end_search": block_end, "form": form,
                "simulated_time_per_wall_second": sim_rate,
                "plain_step_loop": plain, "ratio_vs_plain_step_loop": value / plain["value"],
                "time_to_solution_ratio_vs_plain_step_loop": sim_rate / plain["simulated_time_per_wall_second"],
                "note": "an update = a particle given a freshly computed force at one of its own steps; "
                        "each block = 63 sub-steps replayed as one CUDA graph + a full evaluation"}


# Algorithmic bytes of the HBM-bound passes (the per-unit figures of the scope table's
# measurement row): the radix sort reads the 8 B keys once for its digit counts and moves 12 B
# (key + index) in and out per digit pass; node
# emission reads the 8 B sorted key per particle and writes a 64 B node; the moments pass reads
# a 16 B float32 particle record and reads + writes 64 B per node; the SPH passes per gas
# particle with float32 storage (int32 neighbour rows): density 152 B, force 188 B, and with the
# reference's float64 storage 176 B and 256 B.
SORT_PASSES = 8


def pass_bytes(stage, n, n_gas, nodes, sph32):
    if stage == "tree_sort":
        return 8 * n + 2 * 12 * SORT_PASSES * n
    if stage == "tree_emit":
        return 8 * n + 64 * nodes
    if stage == "tree_moments":
        return 16 * n + 64 * nodes
    if stage == "sph_density":
        return (152 if sph32 else 176) * n_gas
    if stage == "sph_force":
        return (188 if sph32 else 256) * n_gas
    return None


def hbm_passes(res, forms, head, n, n_gas, peak, peak_src, traffic_db):
    """HBM roofline of the sort, build and SPH passes: algorithmic bytes per launch / the
    pass's CUDA-event time per launch inside the timed steps, against the measured copy
    bandwidth; ncu DRAM bytes of one launch where profiles/roofline_traffic.json has them."""
    out = {}
    for f in forms:
        if f not in (head, "plain"):
            continue
        r = res[f]
        sph32 = FORMS[f][2] == 1
        for stage in ("tree_sort", "tree_emit", "tree_moments", "sph_density", "sph_force"):
            st = r["stages"].get(stage)
            b = pass_bytes(stage, n, n_gas, r["nodes"], sph32)
            if not st or b is None:
                continue
            t = st["ms_per_launch"] * 1e-3
            tkey = f"{f}:{stage}"
            tr = traffic_db.get(tkey, {}).get("bytes_per_launch") if traffic_db.get("particles") == n else None
            out[tkey] = {"bound": "hbm", "achieved": b / t / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": b / t / 1e9 / peak, "bytes_per_launch": b, "ms_per_launch": st["ms_per_launch"],
                         "traffic": tr, "peak_source": peak_src}
    return out


def torch_full_like(torch, t, v):
    return torch.full_like(t, v)


def run_gpu(args, world, rank, local):
    G = Gpu(args, local)
    torch, lib, L, params = G.torch, G.lib, G._lib, G.params
    n, n_gas = G.n, G.n_gas
    forms = [f for f in args.forms.split(",") if f]
    head = forms[-1]

    learned = None
    if any(FORMS[f][3] == 2 for f in forms):
        learned = G.train_hguess()

    barrier(world)
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    gpu_index = vis.split(",")[local] if vis else str(local)
    res = {}
    clk = None
    for f in forms:
        steps = args.steps if FORMS[f][0] >= 0.3 else max(3, args.steps // 5)
        if f == head:
            clocks = ClockSampler(gpu_index)
            clocks.start()
        res[f] = G.time_form(f, steps, args.warmup)
        if f == head:
            clk = clocks.stop()
    barrier(world)
    for f in forms:
        r = res[f]
        r["ms_per_step"] = allmax(world, sum(r["times_ms"])) / len(r["times_ms"])
        r["value"] = world * n / (r["ms_per_step"] * 1e-3)

    if rank != 0:
        return

    # accuracy of each form's gravity against the float64 direct sum (2000 random targets)
    tgt = np.random.default_rng(11).choice(n, 2000, replace=False)
    exact = np.zeros((len(tgt), 3))
    L.check(lib.gf_accel_direct_targets(n, G.d["pos"], G.d["mass"], len(tgt), tgt.astype(np.int64), exact,
                                        params.EPS))
    for f in forms:
        res[f]["p99"], res[f]["median"] = G.gravity_error(f, tgt, exact)

    batched = G.batched(args.blocks, config=args.block_config) if args.blocks > 0 else None

    H = res[head]
    # roofline of the dominant kernel of the headline form
    peaks = json.load(open(PEAKS)) if os.path.exists(PEAKS) else {}
    hbm = peaks.get("hbm_gbs", 6800.0)
    hbm_src = "measured (MEASURED_PEAKS.json)" if "hbm_gbs" in peaks else "fallback"
    fp32 = ctypes.c_double()
    lib.gf_fp32_peak(ctypes.byref(fp32))
    stages = H["stages"]
    kernel_stages = {k: v for k, v in stages.items() if k in ("walk", "knn", "sph_density", "sph_force", "verlet")}
    dom = max(kernel_stages, key=lambda k: kernel_stages[k]["ms_per_launch"] * kernel_stages[k]["launches"])
    t_launch = kernel_stages[dom]["ms_per_launch"] * 1e-3
    traffic_db = load_traffic()
    tkey = f"{head}:{dom}"
    traffic = traffic_db.get(tkey, {}).get("bytes_per_launch") if traffic_db.get("particles") == n else None
    quad = FORMS[head][1] == 1
    if dom == "walk":
        mono = H["pairs"] - H["qpairs"]
        flops = FLOPS_MONO * mono + FLOPS_QUAD * H["qpairs"]
        achieved = flops / t_launch / 1e12
        roof = {"kernel": "k_walk<QUAD>" if quad else "k_walk<mono>", "bound": "fp32", "achieved": achieved,
                "peak": fp32.value, "unit": "TFLOP/s", "frac": achieved / fp32.value, "traffic": traffic,
                "peak_source": "measured float32 FFMA throughput of this GPU (gf_fp32_peak)",
                "work_per_launch": {"monopole_interactions": mono, "quadrupole_interactions": H["qpairs"],
                                    "flops_per_monopole": FLOPS_MONO, "flops_per_quadrupole": FLOPS_QUAD}}
        t_alone = H["gravity_alone"].get("walk")
        if t_alone:  # the same launch without the neighbour search beside it
            roof["achieved_alone"] = flops / (t_alone * 1e-3) / 1e12
            roof["frac_alone"] = roof["achieved_alone"] / fp32.value
    else:
        bytes_per_gas = {"knn": 24 + 48 * 4 + 8, "sph_density": 32 * 4 + 24 + 8 + 8 + 8,
                         "sph_force": 32 * 4 + 24 + 24 + 8 + 8 + 8 + 8 + 8 + 24 + 8 + 8,
                         "verlet": 48 * 4 + 24 + 32 * 4 + 8}
        work = bytes_per_gas[dom] * n_gas
        achieved = work / t_launch / 1e9
        roof = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "traffic": traffic, "peak_source": hbm_src,
                "work_per_launch": {"bytes": work, "bytes_per_gas_particle": bytes_per_gas[dom]}}

    passes = hbm_passes(res, forms, head, n, n_gas, hbm, hbm_src, traffic_db)

    e2e = None
    if not args.no_e2e:
        theta = G.set_form(head)

        def pinned(a):  # page-locked host copy (numpy view of a pinned torch tensor)
            t = G.torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
            return t.numpy()

        host = {k: pinned(G.d[k]) for k in ("pos", "vel", "mass", "kind", "u")}
        a_h = pinned(np.empty((n, 3)))
        dt_h = pinned(np.empty(n))

        def host_step():
            st = lib.gf_accelerations(n, host["pos"], host["vel"], host["mass"], host["kind"], host["u"],
                                      theta, params.EPS, params.GAMMA, params.ALPHA, params.BETA,
                                      None, 1, 1, 1, a_h, dt_h)
            if st:
                L.check(st)

        host_step()
        ts = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            host_step()
            ts.append(time.perf_counter() - t0)
        e2e = {"value": world * n / statistics.mean(ts), "unit": UNIT,
               "h2d_bytes_per_step": n * (24 + 24 + 8 + 1 + 8), "d2h_bytes_per_step": n * (24 + 8),
               "ms_per_step": statistics.mean(ts) * 1e3, "form": head,
               "host_buffers": "pinned (page-locked); copies in and out inside each timed call"}

    cpu = None
    parity = None
    if world == 1 and not args.no_cpu:
        sec, cores, fo = time_cpu(G.d, 3, 1)
        cpu = {"value": n / sec, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"3 full force evaluations of the {n:,}-particle workload (median) after 1 "
                         "warm-up: oracle restatement of cpp/nbody.cpp (OpenMP) + scipy cKDTree "
                         "(workers=-1) + restated sph_forces (OpenMP), theta 0.7"}
        parity = parity_vs_oracle(G, fo, head)

    # configs 3 and 4 at bench time, after every measurement of the headline snapshot
    # (shortened: the first search of the clumped snapshot, and 10 long steps of the 4M cloud
    # against block steps over the same simulated time)
    configs = {}
    if args.configs and learned is not None:
        configs["learned_clumps_1M"] = measure_learned_clumps(args, local)
        D = Gpu(args, local, 4, ic="device")
        configs["drift_4M"] = measure_drift(D, args.drift_steps)
        del D
        torch.cuda.set_stream(G.stream)
        torch.cuda.empty_cache()

    def summary(f):
        r = res[f]
        th, quad_f, sph32, hg, rel, merge, relq = FORMS[f]
        out = {"value": r["value"], "ms_per_step": r["ms_per_step"], "theta": th,
               "gravity": "quadrupole float32 + Kahan" if quad_f else "monopole float32 (reference)",
               "opening": (f"relative, alpha {rel:g} with a geometric floor at theta 1 (error scale: the "
                           f"previous evaluation's gravity; theta {th} before it); accepted nodes with a "
                           f"quadrupole term below {relq:g} a_min as monopoles") if rel else
                          f"geometric, theta {th} (cpp/nbody.cpp:104-106)",
               "walk_items": (f"runs of sibling groups of <= {merge} particles, own spheres" if merge else
                              "the reference's groups (cpp/nbody.cpp:235-243)"),
               "sph": "float32 + Kahan" if sph32 else "float64 (reference)",
               "h_guess": ["previous h (cell density without one)", "cell density",
                           "previous h (learned MLP without one)"][hg],
               "grav_p99_rel_err_vs_f64_direct": r["p99"], "grav_median_rel_err": r["median"],
               "stages_ms": {k: round(v["ms_per_launch"], 4) for k, v in r["stages"].items()},
               "gravity_chain_alone_ms": {k: round(v, 4) for k, v in r["gravity_alone"].items()},
               "knn_iterations_per_gas": r["knn_iters"], "walk_interactions": r["pairs"],
               "walk_quadrupole_interactions": r["qpairs"], "steps": len(r["times_ms"])}
        if r.get("autotune"):
            out["walk_autotune"] = r["autotune"]
            out["walk_items"] = (f"runs of sibling groups of <= {r['autotune']['walk_merge']} particles, own spheres"
                                 if r["autotune"]["walk_merge"] else "the reference's groups")
        return out

    line = {
        "metric": METRIC, "value": H["value"], "unit": UNIT, "n_gpus": world, "steps": len(H["times_ms"]),
        "warmup": args.warmup, "ms_per_step": H["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (Kahan) gravity + f32 (Kahan) SPH, f64 positions" if FORMS[head][2] else "f32 gravity + f64 SPH",
        "data": "synthetic",
        "config": {"workload": workload_name(n_gas, n - n_gas), "particles": n, "gas": n_gas,
                   "form": head, "theta": FORMS[head][0], "relative_opening_alpha": FORMS[head][4],
                   "walk_merge": (H.get("autotune") or {}).get("walk_merge", FORMS[head][5]),
                   "walk_shape": (H.get("autotune") or {}).get("walk_shape", 0),
                   "monopole_alpha": FORMS[head][6],
                   "eps_kpc": params.EPS_KPC,
                   "l2": "flushed between steps (256 MB write)", "parallelism": f"replicas x{world}"},
        "roofline": roof,
        "hbm_passes": passes,
        "cpu_baseline": cpu,
        "parity": parity,
        "e2e": e2e,
        "gpu_launches": H["launches"],
        "clocks": clk,
        "forms": {f: summary(f) for f in forms},
        "speedup_vs_plain": {f"{head}/{f}": H["value"] / res[f]["value"] for f in forms if f != head},
        "batched": batched,
        "learned_h": learned,
        "configs": configs or None,
    }
    print(json.dumps(line), flush=True)


def run_learned(args, world, rank, local):
    """Learned smoothing-length guess on 1M gas with 200 Plummer clumps: trained on pairs that
    the plain method produces on the 200k and 1M disk+halo snapshots; search iterations and
    time with the learned guess, with the cell-density start it replaces, and with the
    previous h, on a drifted snapshot; the converged neighbours (hence accelerations) must be
    identical."""
    if rank != 0:
        return
    G1 = Gpu(args, local, 1)
    G1.collect_pairs(5_000_000, collect_steps=6, start=True)
    G2 = Gpu(args, local, 2)
    G2.collect_pairs(5_000_000, collect_steps=4, start=False)
    G = Gpu(args, local, 3)
    tr = G.train_hguess(collected=True)
    torch, lib, L = G.torch, G.lib, G._lib
    theta = G.set_form("mixed_learned")
    # the geometric opening criterion here: the relative one takes its error scale from the
    # previous evaluation, which differs between the three runs compared bit for bit below
    lib.gf_set_option(L.OPT_GRAVITY_REL, 0)
    # the first search of this snapshot (the network never saw it): without a previous h the
    # start is the cell density or the learned guess; then, with a previous h, 2.5 h
    res = {}
    pos = G.T["pos"].clone()
    for mode, name in ((1, "cell_density"), (2, "learned")):
        r = G.search_without_h(theta, pos, mode)
        res[name] = {**r, "acc": G.acc.clone(), "dt": G.dt.clone()}
    lib.gf_set_option(L.OPT_HGUESS, 0)
    res["previous_h"] = G.search_after_drift(theta, pos, 1, 0)
    res["previous_h"].update({"acc": res["learned"]["acc"], "dt": res["learned"]["dt"]})
    same = all(torch.equal(res[k]["acc"], res["cell_density"]["acc"]) and
               torch.equal(res[k]["dt"], res["cell_density"]["dt"]) for k in ("learned",))
    print(json.dumps({
        "workload": "learned smoothing-length guess: 1,000,000 gas, disk + 200 Plummer clumps (seed 3)",
        "training": {k: v for k, v in tr.items() if k in ("training_rows", "loss_start", "loss_end", "train_s")},
        "training_pairs_from": "plain-method evaluations of the 200k and 1M disk+halo snapshots",
        "first_search": {k: {"iterations_per_gas": v["iterations_per_gas"], "knn_ms": v["knn_ms"]}
                         for k, v in res.items() if k != "previous_h"},
        "search_with_previous_h_after_half_step": {"iterations_per_gas": res["previous_h"]["iterations_per_gas"],
                                                   "knn_ms": res["previous_h"]["knn_ms"]},
        "converged_results_identical": bool(same),
        "speedup_learned_vs_cell_density": res["cell_density"]["knn_ms"] / res["learned"]["knn_ms"],
    }), flush=True)


def measure_drift(G, steps, nlev=7):
    """Config 4: the plain form with the reference's step loop against the mixed + batched +
    learned form (block time steps) over the same simulated time, on G's particle set (the
    learned guess must be trained already); updates/s, time to solution and the float64 energy /
    angular-momentum drift of each."""
    torch, lib, L, p = G.torch, G.lib, G._lib, G.params
    d, n = G.d, G.n
    s = torch.cuda.ExternalStream(lib.gf_stream())
    out = {}

    def diag():
        q = np.zeros(8)
        L.check(lib.gf_sim_diagnostics(0.5, q))
        return q

    def drift(q0, q1):
        return {"dE_over_E": abs(q1[3] - q0[3]) / abs(q0[3]),
                "dL_over_L": float(np.linalg.norm(q1[4:7] - q0[4:7]) / np.linalg.norm(q0[4:7])),
                "E0": q0[3], "E1": q1[3]}

    # both forms integrate u with the explicit compression / shock-heating update of
    # _thermodynamics (no cooling, which would radiate energy away), so the total energy
    # kinetic + potential + thermal is the conserved quantity
    units = np.array(p.THERMO_UNITS)
    theta = G.set_form("plain")
    L.check(lib.gf_sim_init(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], theta, p.EPS, p.GAMMA, p.ALPHA,
                            p.BETA))
    L.check(lib.gf_sim_thermo(1, units.ctypes.data))
    q0 = diag()
    tk, sub = ctypes.c_double(), ctypes.c_int()
    upd, subs = 0.0, 0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(steps):
        L.check(lib.gf_sim_step(1e30, ctypes.byref(tk), ctypes.byref(sub)))
        upd += lib.gf_sim_updates()
        subs += sub.value
    e1.record(s)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    q1 = diag()
    t_end = q1[7]
    out["plain_step_loop"] = {"value": upd / (ms * 1e-3), "unit": UNIT, "steps": steps, "substeps": subs,
                              "updates": upd, "ms": ms, "simulated_time": t_end, **drift(q0, q1),
                              "form": "plain: reference step loop (simulation.py:114-149), theta 0.7, "
                                      "float32 monopole walk, float64 SPH"}

    theta = G.set_form("mixed_learned")
    L.check(lib.gf_sim_init(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], theta, p.EPS, p.GAMMA, p.ALPHA,
                            p.BETA))
    L.check(lib.gf_sim_thermo(1, units.ctypes.data))
    chunk = np.zeros(nlev - 1, np.int32)
    every, gms = ctypes.c_int(), ctypes.c_double()
    L.check(lib.gf_sim_block_autotune(nlev, chunk.ctypes.data, ctypes.byref(every), ctypes.byref(gms)))
    q0 = diag()
    upd_b = ctypes.c_double()
    upd, blocks = 0.0, 0
    e0.record(s)
    while True:
        L.check(lib.gf_sim_blocks(1, nlev, ctypes.byref(upd_b)))
        upd += upd_b.value
        blocks += 1
        t = ctypes.c_double()
        L.check(lib.gf_sim_read(None, None, None, None, ctypes.byref(t)))
        if t.value >= t_end or blocks >= 10 * steps:
            break
    e1.record(s)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    q1 = diag()
    out["mixed_batched_learned"] = {"value": upd / (ms * 1e-3), "unit": UNIT, "blocks": blocks,
                                    "substeps": blocks * (1 << (nlev - 1)), "updates": upd, "ms": ms,
                                    "simulated_time": q1[7], **drift(q0, q1),
                                    "autotune": {"chunk_per_bin": chunk.tolist(), "rebuild_every": every.value},
                                    "form": "quadrupole float32 + Kahan walk (relative opening criterion, alpha "
                                            f"{FORMS['mixed_learned'][4]:g}; merged walk items), float32 + Kahan SPH, "
                                            "learned h guess, block time steps (7 levels) replayed as CUDA graphs"}
    lib.gf_sim_thermo(0, None)
    r = out["mixed_batched_learned"]["simulated_time"] / out["mixed_batched_learned"]["ms"]
    r0 = out["plain_step_loop"]["simulated_time"] / out["plain_step_loop"]["ms"]
    return {
        "workload": f"rotating 1/r cloud, {int((d['kind'] == 0).sum()):,} gas + {int((d['kind'] != 0).sum()):,} DM "
                    "(seed 3, drawn on the GPU), the same simulated time for both forms",
        "forms": out,
        "simulated_time_per_wall_second_ratio": r / r0,
        "diagnostics": "gf_sim_diagnostics: float64 sums; potential from a monopole walk at theta 0.5",
        "thermal_update": "u += dt du/dt at every (sub-)step, floored at 1e4 K (simulation.py:97-102); no cooling",
        "initial_conditions": G.ic,
    }


def run_drift(args, world, rank, local):
    """4M rotating cloud: the plain form with the reference's step loop against the mixed +
    batched + learned form (block time steps), over the same simulated time; updates/s and the
    float64 energy / angular-momentum drift of each."""
    if rank != 0:
        return
    G = Gpu(args, local, 4, ic="device")
    G.collect_pairs(2_000_000, collect_steps=2, start=True)
    G.train_hguess(collected=True)
    print(json.dumps(measure_drift(G, args.steps)), flush=True)


def measure_learned_clumps(args, local):
    """Config 3: the first search (no previous h) of 1M gas in a disk with 200 Plummer clumps,
    densities over 6 decades, with the trained network (this process trained it on pairs from
    the disk+halo snapshots, which hold no clumps) against the cell-density start; the
    converged neighbours, hence accelerations and time steps, must be identical."""
    G = Gpu(args, local, 3)
    torch, lib, L = G.torch, G.lib, G._lib
    theta = G.set_form("mixed_learned")
    # the geometric opening criterion: the relative one takes its error scale from the previous
    # evaluation, which differs between the runs compared bit for bit
    lib.gf_set_option(L.OPT_GRAVITY_REL, 0)
    pos = G.T["pos"].clone()
    res = {}
    for mode, name in ((1, "cell_density"), (2, "learned")):
        r = G.search_without_h(theta, pos, mode)
        res[name] = {**r, "acc": G.acc.clone(), "dt": G.dt.clone()}
    lib.gf_set_option(L.OPT_HGUESS, 0)
    same = torch.equal(res["learned"]["acc"], res["cell_density"]["acc"]) and \
        torch.equal(res["learned"]["dt"], res["cell_density"]["dt"])
    out = {"workload": f"{G.n_gas:,} gas + {G.n - G.n_gas:,} DM, disk + 200 Plummer clumps (seed 3)",
           "first_search": {k: {"iterations_per_gas": v["iterations_per_gas"], "knn_ms": v["knn_ms"]}
                            for k, v in res.items()},
           "converged_results_identical": bool(same),
           "speedup_learned_vs_cell_density": res["cell_density"]["knn_ms"] / res["learned"]["knn_ms"]}
    del G
    torch.cuda.empty_cache()
    return out


def main():
    args = parse()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.workload == "drift":
        run_drift(args, world, rank, local)
    elif args.workload == "learned":
        run_learned(args, world, rank, local)
    else:
        run_gpu(args, world, rank, local)


if __name__ == "__main__":
    main()
