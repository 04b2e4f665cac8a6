#!/usr/bin/env python
"""Benchmark of the GB300 Metropolis hot path (flip attempts/s).

Default workload: parallel tempering on a random PUBO -- N=4096 binary
variables, 20000 terms of order {1,2,3,4} w.p. {.1,.5,.3,.1}, weights N(0,1)
FP64, 32 replicas on a geometric temperature ladder 0.05 -> 3.0, 500 sweeps
with a replica swap after every sweep, 16 restarts (16 independent ladders).
One step = one complete solve (init + 500 sweeps + 500 swap phases of all 512
walkers) = 1.05e9 flip attempts.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload pt_pubo|sa_ising|pa_square|batch_cubic|batch_pubo|serving|serving_1e5|
                              pf_sa|tabu_ising|ssmc_ising|qmc_ising|qmc_ising_counter]

Without --workload: one JSON line per configuration (SA, PA, batch, serving),
each from a child process, then the PT headline.  With --workload: that
workload's JSON line (rank 0).  `value` is device-timed (CUDA events on the
launch stream, inputs resident in HBM, L2 flushed before each step); `e2e`
goes through the C ABI from host buffers (model build + upload, solve,
results back to the host) on the host clock.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

WORKLOADS = {
    "pt_pubo": dict(desc="PT on random PUBO N=4096, 20000 terms (orders 1-4), N(0,1) FP64, "
                         "32 temps geometric 0.05->3.0, 500 sweeps, swap every sweep, 16 restarts",
                    target="paralleltempering.qiotoolkit"),
    "sa_ising": dict(desc="SA on sparse Ising N=1000, 3000 ER couplings +-1, 1000 fields U[-0.5,0.5], "
                          "linear beta 0.1->5.0 over 1000 sweeps, 64 restarts, seed 0",
                     target="simulatedannealing.qiotoolkit"),
    "pa_square": dict(desc="PA on 2D periodic 256x256 +-J Ising, R=4096, 100 beta steps 0->3.0, "
                           "10 sweeps per step, the reference's Poisson resampling, counter streams",
                      target="populationannealing.cpu"),
    "serving_1e5": dict(desc="Serving under HBM pressure: Poisson arrivals at 200 req/s, 300 requests; "
                             "kinds uniform over ER Ising (mean degree U[4,16], N(0,1) FP32), PUBO (orders "
                             "U{1,2,3}, N(0,1), 3 terms per variable), weighted 3-SAT (ratio 4.2, U[1,10]); "
                             "N log-uniform [100, 1e5]; sweeps U{200..5000}; SA (8 restarts) or PT (8 "
                             "temperatures); admission budget 1 GiB of HBM",
                        target="mixed"),
    "serving": dict(desc="Serving: Poisson arrivals at 200 req/s, 200 requests; kinds uniform over "
                         "ER Ising (mean degree U[4,16], N(0,1) FP32), PUBO (orders U{1,2,3}, N(0,1), "
                         "3 terms per variable), weighted 3-SAT (ratio 4.2, U[1,10]); N log-uniform "
                         "[100, 1e4]; sweeps U{200..5000}; SA (8 restarts) or PT (8 temperatures)",
                    target="mixed"),
    "pf_sa": dict(desc="Parameter-free SA (linear search, repeated SA runs) on the sparse Ising "
                       "N=1000, 3000 ER couplings +-1, 1000 fields U[-0.5,0.5], min_num_restarts 64, "
                       "seed 0, timeout 3 s per solve",
                  target="simulatedannealing-parameterfree.qiotoolkit"),
    "pf_pa": dict(desc="Parameter-free PA (Bayesian search, repeated PA runs) on the sparse Ising "
                       "N=1000, 3000 ER couplings +-1, 1000 fields U[-0.5,0.5], counter streams (each walker "
                       "its own; threads 16), "
                       "seed 0, timeout 3 s per solve",
                  target="populationannealing-parameterfree.cpu"),
    "tabu_ising": dict(desc="Tabu search on the sparse Ising N=1000, 3000 ER couplings +-1, 1000 fields "
                            "U[-0.5,0.5], tabu_tenure 20, 200 sweeps, 1216 restarts, seed 0; attempts are "
                            "cost-difference evaluations (scan and hill-climbing sweeps)",
                       target="tabu.qiotoolkit"),
    "ssmc_ising": dict(desc="Substochastic Monte Carlo on the sparse Ising N=1000, 3000 ER couplings +-1, "
                            "1000 fields U[-0.5,0.5], target population 4096, 200 steps, 4 steps per walker, "
                            "alpha 1->0 and beta 0->5 linear, counter streams, seed 0; attempts are the "
                            "flips made (each a cost-difference evaluation)",
                       target="substochasticmontecarlo.cpu"),
    "qmc_ising": dict(desc="Quantum Monte Carlo on the sparse Ising N=1000, 3000 ER couplings +-1, 1000 "
                           "fields U[-0.5,0.5], 16 restarts x 32 Trotter slices, 200 sweeps, beta 1->5 and "
                           "transverse field 0->3 linear, replayed PCG streams, seed 0",
                      target="quantummontecarlo.qiotoolkit"),
    "qmc_ising_counter": dict(desc="Quantum Monte Carlo on the sparse Ising N=1000, 3000 ER couplings +-1, "
                                   "1000 fields U[-0.5,0.5], 16 restarts x 32 Trotter slices, 200 sweeps, "
                                   "beta 1->5 and transverse field 0->3 linear, counter streams (level-parallel "
                                   "kernel), seed 0",
                              target="quantummontecarlo.qiotoolkit"),
    "batch_cubic": dict(desc="Batched SA: 512 periodic cubic +-J instances, L uniform in [4,20] "
                             "(64-8000 spins), 16 restarts each, linear beta 0.1->3.0 over 2000 "
                             "sweeps, one captured CUDA graph",
                        target="simulatedannealing.qiotoolkit"),
    "batch_pubo": dict(desc="Batched SA on many-body models: 512 random PUBO instances, N log-uniform "
                            "in [100, 2000], 3N terms of orders 1-4 with N(0,1) FP64 coefficients, 16 "
                            "restarts each, linear beta 0.1->3.0 over 500 sweeps, one captured CUDA "
                            "graph (the windowed kernel's persistent queue)",
                       target="simulatedannealing.qiotoolkit"),
}

BATCH_PARAMS = {"seed": 0, "sweeps": 2000, "restarts": 16, "beta_start": 0.1, "beta_stop": 3.0}
BATCH_PUBO_PARAMS = {"seed": 0, "sweeps": 500, "restarts": 16, "beta_start": 0.1, "beta_stop": 3.0}


def batch_instances(n=512):
    """512 cubic +-J instances, L ~ U{4..20} from seed 2, couplings seeded per instance."""
    import numpy as np
    from qiotoolkit_gb300 import instances as I
    rng = np.random.default_rng(2)
    Ls = rng.integers(4, 21, size=n)
    return [(int(L), I.cubic_pm_j(int(L), seed=1000 + i)) for i, L in enumerate(Ls)]


def batch_pubo_instances(n=512):
    """512 random PUBO instances, N log-uniform in [100, 2000] from seed 3,
    3N terms each, seeded per instance; keyed by N."""
    import numpy as np
    from qiotoolkit_gb300 import instances as I
    rng = np.random.default_rng(3)
    Ns = np.exp(rng.uniform(np.log(100), np.log(2000), size=n)).astype(int)
    return [(int(N), I.random_pubo(int(N), 3 * int(N), seed=2000 + i)) for i, N in enumerate(Ns)]


# the sweep kernel a solver used (qio_solver_stats.sweep_kernel)
KERNEL_NAMES = {1: "sweep_kernel", 2: "lw_sweep_kernel", 3: "lv_sweep_kernel + lv_lowest_kernel",
                4: "tabu_kernel", 5: "ssmc_walk_kernel", 6: "qmc_kernel", 7: "qmc_level_kernel",
                8: "fc_sweep_kernel"}


def make_workload(name):
    from qiotoolkit_gb300 import instances as I
    if name == "pt_pubo":
        off, ids, coef = I.random_pubo(4096, 20000, seed=1)
        params = {"seed": 0, "sweeps": 500, "restarts": 16, "rng_mode": "replay",
                  "temperatures": {"type": "geometric", "initial": 0.05, "final": 3.0,
                                   "count": 32}}
        return "pubo", off, ids, coef, params
    if name == "sa_ising":
        off, ids, coef = I.er_ising(1000, 3000, seed=0)
        params = {"seed": 0, "sweeps": 1000, "restarts": 64, "beta_start": 0.1,
                  "beta_stop": 5.0}
        return "ising", off, ids, coef, params
    if name == "tabu_ising":
        off, ids, coef = I.er_ising(1000, 3000, seed=0)
        params = {"seed": 0, "sweeps": 200, "restarts": 1216, "tabu_tenure": 20}
        return "ising", off, ids, coef, params
    if name == "qmc_ising":
        off, ids, coef = I.er_ising(1000, 3000, seed=0)
        params = {"seed": 0, "sweeps": 200, "restarts": 16, "trotter_number": 32, "beta_start": 1.0,
                  "beta_stop": 5.0, "transverse_field_low": 0.0, "transverse_field_high": 3.0}
        return "ising", off, ids, coef, params
    if name == "qmc_ising_counter":
        kind, off, ids, coef, params = make_workload("qmc_ising")
        return kind, off, ids, coef, dict(params, rng_mode="counter")
    if name == "ssmc_ising":
        off, ids, coef = I.er_ising(1000, 3000, seed=0)
        params = {"seed": 0, "sweeps": 200, "target_population": 4096, "steps_per_walker": 4,
                  "threads": 16, "rng_mode": "counter"}
        return "ising", off, ids, coef, params
    if name == "pa_square":
        off, ids, coef = I.square_pm_j(256, seed=3)
        # the reference's resampling (Poisson on the master PCG stream, host
        # side) with counter walker streams (level-parallel sweeps)
        params = {"seed": 0, "sweeps": 100, "population": 4096, "beta_start": 0.0,
                  "beta_stop": 3.0, "sweeps_per_replica": 10, "rng_mode": "counter"}
        return "ising", off, ids, coef, params
    raise SystemExit(f"unknown workload {name}")


def attempts_per_step(kind, n_vars, params):
    if "target_population" in params or "tabu_tenure" in params:
        return 0  # counted from the run (see main)
    if "trotter_number" in params:
        return params["restarts"] * params["trotter_number"] * params["sweeps"] * n_vars
    if "temperatures" in params:
        return params["restarts"] * params["temperatures"]["count"] * params["sweeps"] * n_vars
    if "population" in params:
        return params["population"] * params["sweeps"] * params["sweeps_per_replica"] * n_vars
    return params["restarts"] * params["sweeps"] * n_vars


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.rows, self.proc, self.device = [], None, device

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
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
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if len(r) > 5 + i and r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def onchip(achieved, clocks):
    """The same algorithmic bytes against shared-memory bandwidth, the level
    where the sweeps keep their models' rows and the walkers' state (HBM
    carries a few percent of those bytes): 152 SMs x 128 bytes per clock at
    the SM clock sampled under load -- a nominal figure, not a measured one."""
    mhz = (clocks or {}).get("sm_mhz") or 2070.0
    peak = 152 * 128 * float(mhz) * 1e6 / 1e9
    return {"level": "shared memory", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": (achieved / peak) if achieved is not None else None,
            "peak_source": "nominal: 152 SMs x 128 B per clock x sampled SM clock"}


def committed_traffic(workload):
    """dram bytes per sweep launch from the committed ncu summary, if any
    (the `dram_bytes_per_launch:` line of profiles/sweep_<workload>_ncu.md)."""
    path = os.path.join(ROOT, "profiles", f"sweep_{workload}_ncu.md")
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("dram_bytes_per_launch:"):
                    return float(line.split(":", 1)[1])
    except (OSError, ValueError):
        return None
    return None


def cpu_baseline(kind, off, ids, coef, params, budget_s=15.0, threads=None):
    """The oracle (CPU restatement of the reference) on a bounded sample of
    the same workload: the full workload when it fits the time budget, else
    fewer sweeps (then fewer restarts / a smaller population).  `threads`
    host threads (OpenMP over replicas, as the reference); default all."""
    from oracle import oracle as O
    threads = threads or os.cpu_count() or 1
    # the Release-flag build of the oracle (the reference's cpp/CMakeLists.txt
    # flags); the parity build checks results, this one is only timed
    m = O.Model(kind, off=off, ids=ids, coef=coef, release=True)
    n = m.n_vars

    def run(restarts, sweeps):
        t0 = time.perf_counter()
        if "temperatures" in params:
            # one reference run per restart (restart k is the run seeded k),
            # each parallel over its replicas
            t = params["temperatures"]
            for k in range(restarts):
                O.run(m, "pt", seed=k, step_limit=sweeps, threads=threads,
                      sched=(t["type"], t["initial"], t["final"]), sched_count=t["count"],
                      use_inverse=False)
            a = restarts * t["count"] * sweeps * n
            d = f"{restarts} runs (seeds 0..{restarts - 1}) x {t['count']} replicas x {sweeps} sweeps"
        elif "population" in params:
            O.run(m, "pa", seed=0, step_limit=sweeps, population=restarts, pa_threads=threads,
                  threads=threads, sched=("linear", params["beta_start"], params["beta_stop"]),
                  sweeps_per_replica=params["sweeps_per_replica"], rng_mode="counter",
                  resampling=params.get("resampling", "reference"))
            a = restarts * sweeps * params["sweeps_per_replica"] * n
            d = f"population {restarts} x {sweeps} steps x {params['sweeps_per_replica']} sweeps"
        elif "trotter_number" in params:
            O.run(m, "qmc", seed=0, step_limit=sweeps, restarts=restarts, threads=threads,
                  trotter_number=params["trotter_number"], rng_mode=params.get("rng_mode", "replay"),
                  sched=("linear", params["beta_start"], params["beta_stop"]),
                  sched2=("linear", params["transverse_field_low"], params["transverse_field_high"]))
            a = restarts * params["trotter_number"] * sweeps * n
            d = f"{restarts} restarts x {params['trotter_number']} slices x {sweeps} sweeps"
        elif "target_population" in params:
            r = O.run(m, "ssmc", seed=0, step_limit=sweeps, population=restarts, threads=threads,
                      pa_threads=params["threads"], steps_per_walker=params["steps_per_walker"],
                      sched=("linear", 1.0, 0.0), sched2=("linear", 0.0, 5.0),
                      rng_mode=params.get("rng_mode", "replay"))
            a = int(np.sum(r.attempts))
            d = f"population {restarts} x {sweeps} steps x {params['steps_per_walker']} steps per walker"
        elif "tabu_tenure" in params:
            r = O.run(m, "tabu", seed=0, step_limit=sweeps, restarts=restarts, threads=threads,
                      tabu_tenure=params["tabu_tenure"])
            a = int(np.sum(r.attempts))
            d = f"{restarts} tabu walkers x {sweeps} sweeps"
        else:
            O.run(m, "sa", seed=0, step_limit=sweeps, restarts=restarts, threads=threads,
                  sched=("linear", params["beta_start"], params["beta_stop"]))
            a = restarts * sweeps * n
            d = f"{restarts} restarts x {sweeps} sweeps"
        return a, time.perf_counter() - t0, d

    full_r = params.get("restarts", params.get("population", params.get("target_population", 1)))
    full_s = params["sweeps"]
    # the parallel dimension first (replicas keep the cores busy), then sweeps
    r0 = min(full_r, max(threads, 1)) if "temperatures" not in params else 1
    restarts, sweeps = r0, min(full_s, 4)
    a, dt, desc = run(restarts, sweeps)
    per = a / (restarts * sweeps)  # attempts per (restart, sweep)
    for _ in range(3):  # grow the sample until it fills about half the budget
        full = restarts == full_r and sweeps == full_s
        if full or dt >= 0.5 * budget_s:
            break
        want = budget_s * a / max(dt, 1e-6)
        sweeps = min(full_s, max(sweeps, int(want / (per * restarts))))
        restarts = min(full_r, max(restarts, int(want / (per * sweeps))))
        a, dt, desc = run(restarts, sweeps)
    full = restarts == full_r and sweeps == full_s
    return {"value": a / dt, "unit": "flip attempts/s", "cores": threads, "kind": "port",
            "sample": f"oracle (C++ restatement, OpenMP over replicas; built with "
                      f"{O.release_flags()}) {desc}"
                      f"{' (the full workload)' if full else ''}, {a:.3g} attempts in {dt:.2f} s"}


def parity_check(kind, off, ids, coef, params, solver):
    """Recompute the timed solve's walkers on the oracle (outside the timed
    region) and compare them with the GPU's: costs, lowest costs, counts and
    states must be equal (the parity build of the oracle, replayed streams
    restated exactly).  PT checks the first ladder (the reference run seeded
    `seed`), SA every restart; other solvers report checked: false."""
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    mode = params.get("rng_mode", "replay")
    if "temperatures" in params:
        t = params["temperatures"]
        sl, what = slice(0, t["count"]), f"first ladder ({t['count']} walkers)"
        run = dict(solver="pt", step_limit=params["sweeps"], sched=(t["type"], t["initial"], t["final"]),
                   sched_count=t["count"], use_inverse=False)
    elif "beta_start" in params and not any(k in params for k in ("population", "trotter_number",
                                                                   "target_population", "tabu_tenure")):
        sl, what = slice(None), f"all {params['restarts']} restarts"
        run = dict(solver="sa", step_limit=params["sweeps"], restarts=params["restarts"],
                   sched=("linear", params["beta_start"], params["beta_stop"]))
    else:
        return {"checked": False, "why": "no in-bench oracle recompute for this solver "
                                         "(its parity is in tests/)"}
    t0 = time.perf_counter()
    m = O.Model(kind, off=off, ids=ids, coef=coef)
    r = O.run(m, seed=params["seed"], threads=threads, rng_mode=mode, **run)
    dt = time.perf_counter() - t0
    rep = solver.replicas()
    fields = {"cost": r.cost, "lowest": r.lowest, "attempts": r.attempts, "accepts": r.accepts,
              "states": r.states, "lowest_states": r.lowest_states}
    bad = [k for k, v in fields.items() if not np.array_equal(np.asarray(rep[k])[sl], v)]
    return {"checked": True, "equal": not bad, "mismatched": bad, "walkers": what,
            "compared": "final and lowest costs, attempt/accept counts, final and lowest states",
            "oracle_s": round(dt, 2)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
    return ws, rank


def reduce_max(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def run_reference(args, ws, rank):
    if rank != 0:
        return
    kind, off, ids, coef, params = make_workload(args.workload)
    from oracle import oracle as O
    O.build()
    times, attempts, desc = [], 0, ""
    for i in range(args.warmup + args.steps):
        cb = cpu_baseline(kind, off, ids, coef, params, budget_s=4.0)
        if i >= args.warmup:
            times.append(cb["value"])
            desc = cb["sample"]
    v = statistics.median(times)
    line = {"impl": "reference", "metric": "flip attempts/s", "value": v,
            "unit": "flip attempts/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOADS[args.workload]["desc"]},
            "cpu_baseline": {"value": v, "unit": "flip attempts/s",
                             "cores": os.cpu_count() or 1, "kind": "port", "sample": desc},
            "e2e": {"value": v, "unit": "flip attempts/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "the reference's own build needs rapidjson/pcg-cpp/googletest/protobuf "
                    "fetched at configure time (no network); timed: the oracle's C++ "
                    "restatement of its CPU path with OpenMP over replicas, built with the "
                    "reference's Release flags (" + O.release_flags() + ")"}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=None, choices=list(WORKLOADS),
                    help="one workload; without it every configuration's line is printed, "
                         "the parallel-tempering headline last")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--kernel", default=None, choices=["auto", "warp", "lanes", "levels", "fields"],
                    help="override the sweep kernel choice (params `kernel`)")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the oracle recompute of the timed solve")
    ap.add_argument("--sweeps", type=int, default=None,
                    help="override the workload's sweeps (small cases for profiler captures)")
    args = ap.parse_args()
    ws, rank = dist_setup()
    if args.impl == "reference":
        if args.workload is None:
            args.workload = "pt_pubo"
        run_reference(args, ws, rank)
        return
    if args.workload is not None:
        run_workload(args, ws, rank)
        return
    # the suite: one line per configuration, each with at least 3 warm-up
    # steps and at most 3 timed steps; the headline (configuration 2) last,
    # with the step counts given.  On one GPU each configuration runs in a
    # process of its own, so that a failure (a CUDA error ends its context)
    # costs only its own line; under torchrun the ranks run them in turn.
    import copy
    for w in SUITE:
        sub = copy.copy(args)
        sub.workload = w
        sub.steps = min(args.steps, 3)
        sub.warmup = 3
        if ws == 1:
            run_isolated(sub)
            continue
        try:
            run_workload(sub, ws, rank)
        except Exception as e:  # a failed line is reported, the suite goes on
            if rank == 0:
                print(json.dumps({"workload": w, "error": f"{type(e).__name__}: {e}"}), flush=True)
        import gc
        gc.collect()
    args.workload = "pt_pubo"
    run_workload(args, ws, rank)


def run_isolated(sub):
    """One configuration's line from a child process (one GPU)."""
    cmd = [sys.executable, os.path.abspath(__file__), "--workload", sub.workload,
           "--steps", str(sub.steps), "--warmup", str(sub.warmup), "--gpus", "1"]
    for flag in ("no_cpu_baseline", "no_e2e", "no_parity"):
        if getattr(sub, flag):
            cmd.append("--" + flag.replace("_", "-"))
    if sub.kernel:
        cmd += ["--kernel", sub.kernel]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, text=True)
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    if r.returncode != 0 or not lines:
        print(json.dumps({"workload": sub.workload, "error": f"exit status {r.returncode}"}), flush=True)
        return
    for ln in lines:
        print(ln, flush=True)


# configurations printed before the headline by a run without --workload
SUITE = ["sa_ising", "pa_square", "batch_cubic", "serving"]


def run_workload(args, ws, rank):
    if args.workload in ("batch_cubic", "batch_pubo"):
        main_batch(args, ws, rank)
        return
    if args.workload == "serving":
        main_serving(args, ws, rank)
        return
    if args.workload == "pf_sa":
        main_pf(args, ws, rank)
        return
    if args.workload == "pf_pa":
        main_pf_pa(args, ws, rank)
        return
    if args.workload == "serving_1e5":
        main_serving(args, ws, rank)
        return

    import torch
    import qiotoolkit_gb300 as q
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    q.load()
    kind, off, ids, coef, params = make_workload(args.workload)
    if args.sweeps:
        params["sweeps"] = args.sweeps
    if args.kernel:
        params["kernel"] = args.kernel
    target = WORKLOADS[args.workload]["target"]
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream

    model = q.Model(kind, off=off, ids=ids, coef=coef)
    tp = dict(params, profile_kernels=True)
    solver = q.Solver(model, target, {"params": tp})
    n = model.n_vars
    A = attempts_per_step(kind, n, params)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    last = {"launches": 0}

    def one_step():
        flush.fill_(1)  # L2 flush (256 MB > 129 MB L2), outside the timed region
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        solver.init(sh)
        solver.run(sh)
        e1.record(stream)
        e1.synchronize()
        st = solver.stats()
        # the solver counts launches cumulatively: keep this step's
        n = int(st.kernel_launches) - last["launches"]
        last["launches"] = int(st.kernel_launches)
        return e0.elapsed_time(e1), st, n

    st0 = None
    for _ in range(args.warmup):
        _, st0, _ = one_step()
    if target in ("tabu.qiotoolkit", "substochasticmontecarlo.cpu") or \
            (target == "populationannealing.cpu" and params.get("resampling") != "multinomial"):
        # evaluations depend on the run (a tabu scan stops at the first
        # improving flip; SSMC flips with probability alpha; a Poisson-resampled
        # population varies in size): count them (deterministic for the fixed
        # seed)
        if st0 is None:
            _, st0, _ = one_step()
        A = int(st0.attempts)
    barrier(ws)
    torch.cuda.synchronize()
    ms, sweep_ms, launches, att = [], [], 0, 0
    kernel_used = 1
    windows = (0, 0)
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            t, st, n_launch = one_step()
            ms.append(t)
            sweep_ms.append(st.sweep_kernel_ms)
            kernel_used = int(st.sweep_kernel)
            windows = (int(st.windows), int(st.attempts))
            launches += n_launch
            att += int(st.attempts)
    torch.cuda.synchronize()
    barrier(ws)
    total_s = reduce_max(sum(ms) / 1e3, ws)
    value = A * args.steps * ws / total_s
    if target in ("simulatedannealing.qiotoolkit", "tabu.qiotoolkit", "quantummontecarlo.qiotoolkit"):
        sweep_launches_per_step = 1
    elif target == "substochasticmontecarlo.cpu":
        sweep_launches_per_step = params["sweeps"]
    else:
        sweep_launches_per_step = params["sweeps"]
    avg_sweep_launch_ms = statistics.mean(sweep_ms) / sweep_launches_per_step
    attempts_per_launch = A / sweep_launches_per_step
    K = model.info.n_incidences
    info = model.info
    # coefficient bytes: int8 for small integer weights, int32 for other
    # integers, FP64 otherwise
    w = 1.0 if info.integer_weights and info.max_coupling <= 127 else (4.0 if info.integer_weights else 8.0)
    # row bounds 8 + own state 1 + per incidence (id 4 + coefficient w + state 1)
    bpa = 9.0 + (5.0 + w) * K / n
    if target == "tabu.qiotoolkit":
        # a tabu evaluation reads the variable's cached difference (FP64) and
        # its tabu expiry (uint64)
        bpa = 16.0
    achieved = bpa * attempts_per_launch / (avg_sweep_launch_ms / 1e3) / 1e9
    peak, peak_src = peaks()
    traffic = committed_traffic(args.workload)

    parity = None
    if rank == 0 and not args.no_parity:
        parity = parity_check(kind, off, ids, coef, params, solver)

    e2e = None
    if not args.no_e2e:
        e2e = measure_e2e(q, kind, off, ids, coef, params, target, A, args, stream)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(kind, off, ids, coef, params)
        one = cpu_baseline(kind, off, ids, coef, params, budget_s=8.0, threads=1)
        cpu["single_thread"] = {"value": one["value"], "cores": 1, "sample": one["sample"]}

    if rank == 0:
        line = {
            "metric": "flip attempts/s", "value": value, "unit": "flip attempts/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_s * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOADS[args.workload]["desc"], "n_vars": n,
                       "n_terms": model.n_terms, "attempts_per_step": A,
                       "rng_mode": params.get("rng_mode", "replay"),
                       "l2": "flushed before each step (256 MB write)"},
            "e2e": e2e,
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                         "peak_source": peak_src, "kernel": KERNEL_NAMES.get(kernel_used, "sweep_kernel"),
                         "bytes_per_attempt": bpa,
                         "avg_launch_ms": avg_sweep_launch_ms,
                         "attempts_per_window": (windows[1] / windows[0]) if windows[0] else None},
            "roofline_onchip": onchip(achieved, clk.summary()),
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "parity": parity,
        }
        print(json.dumps(line), flush=True)
        if parity and parity.get("checked") and not parity["equal"]:
            sys.exit(f"parity check failed: {parity['mismatched']}")


def serving_requests(n=48, rate=200.0, seed=4, nmax=1e4):
    """Requests of the serving configuration: Poisson arrivals at `rate`, the
    first n of them, N log-uniform in [100, nmax]."""
    import numpy as np
    from qiotoolkit_gb300 import instances as I
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    out = []
    for i in range(n):
        kind = int(rng.integers(0, 3))
        N = int(np.exp(rng.uniform(np.log(100), np.log(nmax))))
        sweeps = int(rng.integers(200, 5001))
        pt = bool(rng.integers(0, 2))
        if kind == 0:
            k, inst = "ising", I.er_ising_gauss(N, float(rng.uniform(4, 16)), seed=100 + i)
        elif kind == 1:
            k, inst = "pubo", I.random_pubo(N, 3 * N, seed=100 + i, orders=(1, 2, 3),
                                            probs=(1 / 3, 1 / 3, 1 / 3))
        else:
            k, inst = "maxsat", I.weighted_maxsat(N, seed=100 + i)
        if pt:
            target = "paralleltempering.qiotoolkit"
            params = {"seed": i, "sweeps": sweeps, "temperatures": {"type": "geometric", "initial": 0.1,
                                                                    "final": 3.0, "count": 8}}
        else:
            target = "simulatedannealing.qiotoolkit"
            params = {"seed": i, "sweeps": sweeps, "restarts": 8, "beta_start": 0.1, "beta_stop": 3.0}
        out.append((float(t[i]), k, inst, target, params))
    return out


PF_PARAMS = {"seed": 0, "min_num_restarts": 64, "timeout": 3}


def main_pf(args, ws, rank):
    """Parameter-free SA: flip attempts/s over whole parameter-free solves
    (every SA run of the search), the same solve through the C ABI from host
    buffers, and the oracle's restatement of the search on the host cores."""
    import torch
    import qiotoolkit_gb300 as q
    from qiotoolkit_gb300 import instances as I
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    q.load()
    target = WORKLOADS["pf_sa"]["target"]
    off, ids, coef = I.er_ising(1000, 3000, seed=0)
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    model = q.Model("ising", off=off, ids=ids, coef=coef)
    solver = q.Solver(model, target, {"params": PF_PARAMS})
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    def one_step():
        flush.fill_(1)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        solver.init(sh)
        solver.run(sh)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1), solver.stats()

    for _ in range(args.warmup):
        one_step()
    barrier(ws)
    torch.cuda.synchronize()
    ms, att, launches = [], 0, 0
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            t, st = one_step()
            ms.append(t)
            att += int(st.attempts)
            launches += int(st.kernel_launches)
    torch.cuda.synchronize()
    barrier(ws)
    total_s = reduce_max(sum(ms) / 1e3, ws)
    value = att * ws / total_s
    res = solver.result()
    runs = res["benchmark"]["parameter_free"]["runs"]
    best = res["solutions"]["cost"]

    e2e = None
    if not args.no_e2e:
        times, h2d, d2h = [], 0, 0
        for i in range(1 + min(args.steps, 3)):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            m = q.Model("ising", off=off, ids=ids, coef=coef)
            s = q.Solver(m, target, {"params": PF_PARAMS})
            s.init(sh)
            s.run(sh)
            r = s.result()
            torch.cuda.synchronize()
            if i > 0:
                times.append(time.perf_counter() - t0)
            h2d = int(m.info.device_bytes)
            d2h = int(m.n_vars * 8 + 64)
            s.close()
            m.close()
        e2e = {"value": att / args.steps / statistics.median(times), "unit": "flip attempts/s",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        # the same SA runs (sweeps, restarts, continuing master stream) on
        # the oracle, in order, until about 15 s of CPU time
        import math
        from oracle import oracle as O
        o = O.Model("ising", off=off, ids=ids, coef=coef)
        terms = [(float(coef[k]), [int(x) for x in ids[off[k]:off[k + 1]]]) for k in range(len(coef))]
        mn, mx = O.cost_diff_bounds("ising", terms)
        b0 = -math.log(0.5) / mx
        b1 = -math.log(0.0001) / (mn + 0.001 * (mx - mn))
        cores = os.cpu_count() or 1
        t0 = time.perf_counter()
        skip, a_cpu, same, k = 0, 0, True, 0
        for x in runs:
            r = O.run(o, "sa", seed=PF_PARAMS["seed"], step_limit=x["sweeps"], restarts=x["restarts"],
                      use_inverse=True, sched=("linear", b0, b1), threads=cores, master_skip=skip)
            skip += x["restarts"]
            a_cpu += x["sweeps"] * x["restarts"] * model.n_vars
            same = same and float(r.best_cost) == x["lowest"]
            k += 1
            if time.perf_counter() - t0 > 15.0:
                break
        dt = time.perf_counter() - t0
        cpu = {"value": a_cpu / dt, "unit": "flip attempts/s", "cores": cores, "kind": "port",
               "sample": f"the first {k} of the solve's {len(runs)} SA runs on the oracle (same sweeps, "
                         f"restarts and master stream), {a_cpu:.3g} attempts in {dt:.2f} s; identical "
                         f"lowest costs: {same}"}

    if rank == 0:
        kernel_s = sum(ms) / 1e3
        bpa = 100.0  # the sparse Ising N=1000 model: 8 + 7 x (4 + 8 + 1) + 1 bytes per attempt
        achieved = bpa * att / kernel_s / 1e9
        peak, peak_src = peaks()
        line = {
            "metric": "flip attempts/s", "value": value, "unit": "flip attempts/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_s * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": WORKLOADS["pf_sa"]["desc"], "runs_per_solve": len(runs),
                       "best_cost": best, "l2": "flushed before each step (256 MB write)"},
            "e2e": e2e, "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None, "peak_source": peak_src,
                         "kernel": "sweep_kernel (whole solves timed)", "bytes_per_attempt": bpa},
            "roofline_onchip": onchip(achieved, clk.summary()),
            "cpu_baseline": cpu, "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)


PF_PA_PARAMS = {"seed": 0, "timeout": 3, "threads": 16, "rng_mode": "counter", "resampling": "reference"}


def main_pf_pa(args, ws, rank):
    """Parameter-free PA: flip attempts/s over whole parameter-free solves
    (every PA run of the search, its attempts counted as walkers x sweeps x
    N per step), the same solve through the C ABI from host buffers, and the
    same runs replayed by the oracle on the host cores."""
    import torch
    import qiotoolkit_gb300 as q
    from qiotoolkit_gb300 import instances as I
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    q.load()
    target = WORKLOADS["pf_pa"]["target"]
    off, ids, coef = I.er_ising(1000, 3000, seed=0)
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    model = q.Model("ising", off=off, ids=ids, coef=coef)
    solver = q.Solver(model, target, {"params": PF_PA_PARAMS})
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    def one_step():
        flush.fill_(1)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        solver.init(sh)
        solver.run(sh)
        e1.record(stream)
        e1.synchronize()
        runs = solver.result()["benchmark"]["parameter_free"]["runs"]
        return e0.elapsed_time(e1), sum(int(r["attempts"]) for r in runs), solver.stats()

    for _ in range(args.warmup):
        one_step()
    barrier(ws)
    torch.cuda.synchronize()
    ms, att, launches = [], 0, 0
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            t, a, st = one_step()
            ms.append(t)
            att += a
            launches += int(st.kernel_launches)
    torch.cuda.synchronize()
    barrier(ws)
    total_s = reduce_max(sum(ms) / 1e3, ws)
    value = att * ws / total_s
    res = solver.result()
    runs = res["benchmark"]["parameter_free"]["runs"]
    best = res["solutions"]["cost"]

    e2e = None
    if not args.no_e2e:
        times, h2d, d2h, att_e = [], 0, 0, []
        for i in range(1 + min(args.steps, 3)):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            m = q.Model("ising", off=off, ids=ids, coef=coef)
            s = q.Solver(m, target, {"params": PF_PA_PARAMS})
            s.init(sh)
            s.run(sh)
            r = s.result()
            torch.cuda.synchronize()
            if i > 0:
                times.append(time.perf_counter() - t0)
                att_e.append(sum(int(x["attempts"]) for x in r["benchmark"]["parameter_free"]["runs"]))
            h2d = int(m.info.device_bytes)
            d2h = int(m.n_vars * 8 + 64)
            s.close()
            m.close()
        e2e = {"value": sum(att_e) / sum(times), "unit": "flip attempts/s",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        # the same PA runs (parameters, continuing master stream) on the
        # oracle, in order, until about 15 s of CPU time
        from oracle import oracle as O
        o = O.Model("ising", off=off, ids=ids, coef=coef)
        terms = [(float(coef[k]), [int(x) for x in ids[off[k]:off[k + 1]]]) for k in range(len(coef))]
        cores = min(PF_PA_PARAMS["threads"], os.cpu_count() or 1)
        whole = []
        for x in runs:
            if x["steps"] < x["step_limit"]:
                break  # a run the time limit cut short ends the replayable prefix
            whole.append(x)
        t0 = time.perf_counter()
        ref = O.pa_parameter_free_replay(o, "ising", terms, seed=PF_PA_PARAMS["seed"],
                                         threads=PF_PA_PARAMS["threads"], runs=[x["params"] for x in whole],
                                         budget_s=15.0, rng_mode=PF_PA_PARAMS["rng_mode"],
                                         resampling=PF_PA_PARAMS["resampling"])
        k = len(ref)
        a_cpu = sum(int(x["attempts"]) for x in whole[:k])
        same = all(r[2] == x["lowest"] for r, x in zip(ref, whole))
        dt = time.perf_counter() - t0
        cpu = {"value": a_cpu / dt if dt > 0 else None, "unit": "flip attempts/s", "cores": cores,
               "kind": "port",
               "sample": f"the first {k} of the solve's {len(runs)} PA runs replayed by the oracle "
                         f"(same parameters and master stream); {a_cpu:.3g} attempts; identical lowest "
                         f"costs: {same}"}

    if rank == 0:
        kernel_s = sum(ms) / 1e3
        bpa = 100.0  # the sparse Ising N=1000 model: 8 + 7 x (4 + 8 + 1) + 1 bytes per attempt
        achieved = bpa * att / kernel_s / 1e9
        peak, peak_src = peaks()
        line = {
            "metric": "flip attempts/s", "value": value, "unit": "flip attempts/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_s * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": WORKLOADS["pf_pa"]["desc"], "runs_per_solve": len(runs),
                       "best_cost": best, "l2": "flushed before each step (256 MB write)"},
            "e2e": e2e, "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None, "peak_source": peak_src,
                         "kernel": "sweep_kernel (whole solves timed)", "bytes_per_attempt": bpa},
            "roofline_onchip": onchip(achieved, clk.summary()),
            "cpu_baseline": cpu, "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)


def main_serving(args, ws, rank):
    """Continuous batching against the same request stream served one at a
    time (a queue alone): instances/s, p50/p99 submit-to-done latency."""
    import numpy as np
    import torch
    import qiotoolkit_gb300 as q
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    q.load()
    big = args.workload == "serving_1e5"
    reqs = serving_requests(n=300, nmax=1e5) if big else serving_requests(n=200)
    budget = (1 << 30) if big else 0
    models = [q.Model(k, off=o, ids=i, coef=c) for _, k, (o, i, c), _, _ in reqs]

    def attempts(m, target, p):
        w = 8
        per = m.n_vars if m.info.kind != 4 else 1  # MaxSat: one attempt per sweep
        return w * p["sweeps"] * per

    n_att = sum(attempts(m, t, p) for m, (_, _, _, t, p) in zip(models, reqs))

    foot = []
    launched = [0]  # kernel launches of the last serve() (the solves' own counts)

    def serve(max_active, count=None):
        srv = q.Server(memory_budget_bytes=budget, max_active=max_active)
        t0 = time.perf_counter()
        ids = []
        for m, (ta, _, _, target, p) in list(zip(models, reqs))[:count]:
            d = t0 + ta - time.perf_counter()
            if d > 0:
                time.sleep(d)
            pp = dict(p, kernel=args.kernel) if args.kernel else p
            ids.append(srv.submit(m, target, {"params": pp}))
        results = [srv.wait(i) for i in ids]
        dt = time.perf_counter() - t0
        best = [r["solutions"]["cost"] for r in results]
        launched[0] = sum(int(r["benchmark"]["gb300"]["kernel_launches"]) for r in results)
        st = srv.stats()
        foot.extend(srv.request_bytes(i) for i in ids)
        srv.close()
        return dt, st, best

    MAXA = 256  # every request's chains in flight at once (8 walkers each)
    serve(MAXA, 8)  # warm-up: module loading, table uploads
    with ClockSampler(local) as clk:
        dt_mix, st_mix, best_mix = serve(MAXA)
    launches_mix = launched[0]
    # continuous batching against a queue alone, on the first 48 requests
    # (the queue alone serves them one after another)
    nq = 0 if big else 48
    if nq:
        dt_q48, st_q48, best_q48 = serve(MAXA, nq)
        dt_one, st_one, best_one = serve(1, nq)
        same = best_q48 == best_one
    
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import oracle as O
        threads = os.cpu_count() or 1
        t_cpu, a_cpu = 0.0, 0
        for j in range(0, len(reqs), 20):
            _, k, (o, i, c), target, p = reqs[j]
            om = O.Model(k, off=o, ids=i, coef=c, release=True)
            t0 = time.perf_counter()
            if target.startswith("parallel"):
                O.run(om, "pt", seed=p["seed"], step_limit=p["sweeps"], threads=threads,
                      sched=("geometric", 0.1, 3.0), sched_count=8, use_inverse=False)
            else:
                O.run(om, "sa", seed=p["seed"], step_limit=p["sweeps"], restarts=8, threads=threads,
                      sched=("linear", 0.1, 3.0))
            t_cpu += time.perf_counter() - t0
            a_cpu += attempts(models[j], target, p)
        rate = a_cpu / t_cpu
        cpu = {"value": len(reqs) / (n_att / rate), "unit": "instances/s", "cores": threads,
               "kind": "port",
               "sample": f"oracle on every 20th request ({a_cpu:.3g} attempts in {t_cpu:.1f} s), "
                         f"requests one after another, extrapolated by attempts"}
    if rank == 0:
        line = {
            "metric": "instances/s served; p50/p99 solve latency", "value": len(reqs) / dt_mix,
            "unit": "instances/s", "n_gpus": ws, "steps": 1, "warmup": 1,
            "ms_per_step": dt_mix * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOADS[args.workload]["desc"], "requests": len(reqs),
                       "attempts": n_att, "max_active": MAXA, "memory_budget_bytes": budget,
                       "largest_request_vars": int(max(m.n_vars for m in models))},
            "latency_ms": {"p50": st_mix.p50_ms, "p99": st_mix.p99_ms, "max": st_mix.max_ms},
            "attempts_per_s": n_att / dt_mix,
            "peak_active": int(st_mix.peak_active),
            "admission": {"budget_bytes": int(st_mix.budget_bytes),
                          "largest_request_bytes": int(max(foot)) if foot else None,
                          "sum_request_bytes": int(sum(foot[8:8 + len(reqs)])) if foot else None},
            "queue_alone": ({"requests": nq, "value": nq / dt_one, "unit": "instances/s",
                             "latency_ms": {"p50": st_one.p50_ms, "p99": st_one.p99_ms},
                             "continuous_batching_value": nq / dt_q48,
                             "speedup": dt_one / dt_q48,
                             "same_results_alone_and_in_mix": bool(same)} if nq else None),
            "e2e": {"value": len(reqs) / dt_mix, "unit": "instances/s",
                    "h2d_bytes_per_step": int(sum(m.info.device_bytes for m in models)),
                    "d2h_bytes_per_step": int(sum(8 * m.n_vars for m in models))},
            "gpu_launches": launches_mix,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)


def main_batch(args, ws, rank):
    """Batched workload: instances/s of one captured graph over all instances,
    beside the plain path (one solve per instance) timed on one instance per
    distinct L (cubic lattices) or on every 32nd instance (PUBO) and
    extrapolated to the whole batch by its variable counts."""
    import numpy as np
    import torch
    import qiotoolkit_gb300 as q
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    q.load()
    pubo = args.workload == "batch_pubo"
    params = dict(BATCH_PUBO_PARAMS if pubo else BATCH_PARAMS)
    if args.sweeps:
        params["sweeps"] = args.sweeps
    target = WORKLOADS[args.workload]["target"]
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    inst = batch_pubo_instances() if pubo else batch_instances()
    kind = "pubo" if pubo else "ising"
    models = [q.Model(kind, off=o, ids=i, coef=c) for _, (o, i, c) in inst]
    n_att = sum(m.n_vars for m in models) * params["restarts"] * params["sweeps"]
    batch = q.Batch(models, target, {"params": params})
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    def one_step():
        flush.fill_(1)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        batch.run(sh)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1)

    for _ in range(args.warmup):
        one_step()
    barrier(ws)
    torch.cuda.synchronize()
    ms = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            ms.append(one_step())
    torch.cuda.synchronize()
    barrier(ws)
    total_s = reduce_max(sum(ms) / 1e3, ws)
    st = batch.stats()
    value = len(models) * args.steps * ws / total_s
    low_batch = batch.lowest()

    # the sweep kernel alone: one run outside the graph with events around it
    prof = q.Batch(models, target, {"params": dict(params, graph=False, profile_kernels=True)})
    prof.run(sh)
    pst = prof.stats()
    kernel_ms = pst.sweep_kernel_ms if pst.sweep_kernel_ms > 0 else st.run_ms
    prof.close()
    if pubo:
        # 8 row bounds + per incidence (4 term id + 8 coefficient + 1 term state) + 1 own state
        kbar = sum(m.info.n_incidences for m in models) / sum(m.n_vars for m in models)
        bpa = 8.0 + 13.0 * kbar + 1.0
    else:
        bpa = 45.0  # 8 row bounds + 6 x (4 id + 1 coefficient + 1 state) + 1 own state
    achieved = bpa * n_att / (kernel_ms / 1e3) / 1e9
    peak, peak_src = peaks()

    # plain path: one solve per instance (the drop-in path), one per distinct
    # L, timed like the batch: device-timed (CUDA events around init + run on
    # the stream), model and solver resident, after a warm-up solve
    per_L, rel = {}, []
    for idx, (L, _) in enumerate(inst):
        if L in per_L or (pubo and idx % 32):
            continue
        s = q.Solver(models[idx], target, {"params": params})
        s.init(sh).run(sh)
        best_ms = None
        for _ in range(2):
            flush.fill_(1)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            s.init(sh).run(sh)
            e1.record(stream)
            e1.synchronize()
            t = e0.elapsed_time(e1)
            best_ms = t if best_ms is None else min(best_ms, t)
        c, _ = s.best()
        per_L[L] = best_ms / 1e3
        rel.append(abs(low_batch[idx] - c) / max(abs(c), 1e-12))
        s.close()
    if pubo:
        # seconds per variable on the sampled instances, over the batch's sizes
        xs = sorted(per_L)
        plain_s = sum(float(np.interp(L, xs, [per_L[x] / x for x in xs])) * L for L, _ in inst)
    else:
        plain_s = sum(per_L[L] for L, _ in inst)
    plain_value = len(models) / plain_s

    e2e = None
    if not args.no_e2e:
        times = []
        for i in range(2):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            # the plan the timed batch found, reused as a caller would
            plan = dict(params, autotune=False, warps_per_block=int(st.warps_per_block),
                        smem_state=bool(st.smem))
            b = q.Batch(models, target, {"params": plan})
            b.run(sh)
            lo = b.lowest()
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
            b.close()
        h2d = int(sum(m.info.device_bytes for m in models))
        e2e = {"value": len(models) / min(times), "unit": "instances/s",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": int(lo.nbytes)}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import oracle as O
        threads = os.cpu_count() or 1
        t_cpu, L_seen = {}, set()
        nv = (lambda L: L) if pubo else (lambda L: L ** 3)
        for idx, (L, (o, i, c)) in enumerate(inst):
            if L in L_seen or (idx % 64 if pubo else L % 4):
                continue
            L_seen.add(L)
            om = O.Model(kind, off=o, ids=i, coef=c, release=True)
            t0 = time.perf_counter()
            O.run(om, "sa", seed=0, step_limit=params["sweeps"], restarts=params["restarts"],
                  threads=threads, sched=("linear", params["beta_start"], params["beta_stop"]))
            t_cpu[L] = (time.perf_counter() - t0) / nv(L)
        # seconds per variable at each sampled size, interpolated over the batch's sizes
        xs = sorted(t_cpu)
        cpu_s = sum(float(np.interp(L, xs, [t_cpu[x] for x in xs])) * nv(L) for L, _ in inst)
        what = "every 64th instance (N in %s)" % xs if pubo else "one instance for each L in %s" % xs
        cpu = {"value": len(models) / cpu_s, "unit": "instances/s", "cores": threads, "kind": "port",
               "sample": f"oracle SA (OpenMP over restarts) on {what}, full sweeps and restarts; "
                         f"per-variable time interpolated over the 512 sizes"}

    if rank == 0:
        line = {
            "metric": "instances/s batched", "value": value, "unit": "instances/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_s * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if pubo else "int32", "data": "synthetic",
            "config": {"workload": WORKLOADS[args.workload]["desc"], "instances": len(models),
                       "total_spins": int(sum(m.n_vars for m in models)),
                       "attempts_per_step": n_att, "rng_mode": "replay",
                       "plan": {"kernel": "lanes" if st.kernel == 2 else "warp",
                                "warps_per_block": st.warps_per_block, "smem": st.smem,
                                "graph": st.graph},
                       "l2": "flushed before each step (256 MB write)"},
            "attempts_per_s": n_att * args.steps * ws / total_s,
            "plain_per_instance": {"value": plain_value, "unit": "instances/s",
                                   "sample": ("one plain solve (default kernel choice) on every 32nd "
                                              "instance" if pubo else
                                              "one plain solve (default kernel choice) per distinct L") +
                                             ", device-timed like the batch (CUDA events around init + run, "
                                             "model resident, best of 2 after a warm-up), extrapolated "
                                             "over the 512 instances"},
            "speedup_vs_plain": value / plain_value,
            "best_energy_rel_diff_vs_plain": {"median": float(np.median(rel)), "max": float(max(rel))},
            "e2e": e2e,
            "gpu_launches": int(st.launches),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None, "peak_source": peak_src,
                         "kernel": "sweep_kernel" if st.kernel == 1 else "lw_sweep_kernel",
                         "bytes_per_attempt": bpa,
                         "avg_launch_ms": kernel_ms},
            "roofline_onchip": onchip(achieved, clk.summary()),
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)


def measure_e2e(q, kind, off, ids, coef, params, target, A, args, stream):
    """Same metric through the C ABI from host buffers: model build from the
    host term arrays, upload, solve, lowest costs and states back."""
    import torch
    times, h2d, d2h = [], 0, 0
    for i in range(1 + min(args.steps, 3)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        m = q.Model(kind, off=off, ids=ids, coef=coef)
        s = q.Solver(m, target, {"params": params})
        s.init(stream.cuda_stream)
        s.run(stream.cuda_stream)
        rep = s.replicas(states=True)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        if i > 0:
            times.append(dt)
        h2d = int(m.info.device_bytes)
        d2h = int(rep["lowest_states"].size + rep["states"].size + 32 * len(rep["cost"]))
        s.close()
        m.close()
    return {"value": A / statistics.median(times), "unit": "flip attempts/s",
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}


if __name__ == "__main__":
    main()
