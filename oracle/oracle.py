"""ctypes wrapper of the CPU oracle (oracle/qio_oracle.cc).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
as the checker, and by bench.py's CPU-baseline leg.  The product package never
imports this module.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libqio_oracle.so")
# the same source built with the reference's Release flags (-Ofast,
# -march=native): for timing the CPU baseline only, never for checking results
_REL_PATH = os.path.join(_HERE, "_build", "libqio_oracle_release.so")
_lock = threading.Lock()
_libs = {}

ISING, ISING_PLAIN, PUBO, PUBO_PLAIN, MAXSAT = 0, 1, 2, 3, 4
SA, PT, PA, TABU, SSMC, QMC = 0, 1, 2, 3, 4, 5
RNG_REPLAY, RNG_COUNTER = 0, 1
SCHED_LINEAR, SCHED_GEOMETRIC, SCHED_CONSTANT, SCHED_LIST = 0, 1, 2, 3

KIND_BY_NAME = {"ising": ISING, "ising_plain": ISING_PLAIN, "pubo": PUBO,
                "pubo_plain": PUBO_PLAIN, "maxsat": MAXSAT}


class Schedule(C.Structure):
    _fields_ = [("type", C.c_int), ("initial", C.c_double),
                ("final_value", C.c_double), ("has_start", C.c_int),
                ("has_stop", C.c_int), ("has_count", C.c_int),
                ("start", C.c_double), ("stop", C.c_double),
                ("count", C.c_int), ("n_values", C.c_int),
                ("values", C.POINTER(C.c_double))]


class Params(C.Structure):
    _fields_ = [("solver", C.c_int), ("seed", C.c_uint32),
                ("step_limit", C.c_int64), ("restarts", C.c_int64),
                ("use_inverse", C.c_int), ("sched", Schedule),
                ("sweeps_per_replica", C.c_int64),
                ("population", C.c_int64), ("alpha", C.c_double),
                ("constant_population", C.c_int),
                ("exp_repopulation", C.c_int), ("pa_threads", C.c_int),
                ("rng_mode", C.c_int), ("threads", C.c_int),
                ("number_of_solutions", C.c_int),
                ("has_cost_limit", C.c_int), ("cost_limit", C.c_double),
                ("full_maxsat_sweep", C.c_int), ("resampling", C.c_int),
                ("master_skip", C.c_int64), ("use_master_state", C.c_int),
                ("master_state", C.c_uint64), ("tabu_tenure", C.c_int64),
                ("sched2", Schedule), ("tabu_tenures", C.POINTER(C.c_int64)),
                ("n_tabu_tenures", C.c_int64), ("trotter_number", C.c_int64)]


def build(force: bool = False) -> str:
    """Compile the oracle with make (g++; a few seconds): the parity build and
    the Release-flag timing build."""
    with _lock:
        src = os.path.join(_HERE, "qio_oracle.cc")
        stale = any(not os.path.exists(f) or os.path.getmtime(f) < os.path.getmtime(src)
                    for f in (_LIB_PATH, _REL_PATH))
        if force or stale:
            subprocess.run(["make", "-s", "-j2", "-C", _HERE] + (["-B"] if force else []),
                           check=True)
    return _LIB_PATH


def release_flags() -> str:
    """The compiler flags of the Release-flag timing build."""
    try:
        with open(os.path.join(_HERE, "_build", "release_flags.txt")) as f:
            return f.read().strip()
    except OSError:
        return ""


def lib(release: bool = False):
    """The oracle library: the parity build, or with release=True the
    Release-flag build (timing only)."""
    if release not in _libs:
        build()
        L = C.CDLL(_REL_PATH if release else _LIB_PATH)
        vp, i64, u32, dbl, ip = C.c_void_p, C.c_int64, C.c_uint32, C.c_double, C.c_int
        P = C.POINTER
        L.orc_pcg_stream.argtypes = [u32, ip, ip, P(C.c_uint32)]
        L.orc_pcg_uniform.argtypes = [u32, ip, ip, P(dbl)]
        L.orc_pcg_fork_uniform.argtypes = [u32, ip, ip, P(dbl)]
        L.orc_pcg_state_uniform.argtypes = [P(C.c_uint64)]
        L.orc_pcg_state_uniform.restype = dbl
        L.orc_pcg_state_u32.argtypes = [P(C.c_uint64)]
        L.orc_pcg_state_u32.restype = u32
        L.orc_twister_uniform.argtypes = [u32, ip, ip, P(dbl)]
        L.orc_uniform_ln.argtypes = [P(dbl)]
        L.orc_metropolis_accept.argtypes = [dbl, dbl, P(C.c_uint32), ip, P(ip)]
        L.orc_metropolis_accept.restype = ip
        L.orc_counter_draw.argtypes = [C.c_uint64, C.c_uint64]
        L.orc_counter_draw.restype = C.c_uint64
        L.orc_qexp.argtypes = [C.c_double]
        L.orc_qexp.restype = C.c_double
        L.orc_counter_key.argtypes = [u32, C.c_uint64]
        L.orc_counter_key.restype = C.c_uint64
        L.orc_model_create.argtypes = [ip, i64, P(i64), P(C.c_int32), P(dbl), C.c_char_p, ip]
        L.orc_model_create.restype = vp
        L.orc_model_destroy.argtypes = [vp]
        for f in ("orc_model_n_vars", "orc_model_n_terms"):
            getattr(L, f).argtypes = [vp]
            getattr(L, f).restype = i64
        for f in ("orc_model_const_cost", "orc_model_scale_factor"):
            getattr(L, f).argtypes = [vp]
            getattr(L, f).restype = dbl
        L.orc_model_var_names.argtypes = [vp, P(C.c_int32)]
        L.orc_state_cost.argtypes = [vp, P(C.c_uint8)]
        L.orc_state_cost.restype = dbl
        L.orc_state_cost_difference.argtypes = [vp, P(C.c_uint8), i64]
        L.orc_state_cost_difference.restype = dbl
        L.orc_model_twister_min.argtypes = [vp, u32, ip, dbl]
        L.orc_model_twister_min.restype = dbl
        L.orc_run.argtypes = [vp, P(Params), C.c_char_p, ip]
        L.orc_run.restype = vp
        for f in ("orc_res_n_replicas", "orc_res_n_vars", "orc_res_last_step",
                  "orc_res_n_solutions"):
            getattr(L, f).argtypes = [vp]
            getattr(L, f).restype = i64
        L.orc_res_replicas.argtypes = [vp, P(dbl), P(dbl), P(C.c_uint64), P(C.c_uint64)]
        L.orc_res_states.argtypes = [vp, P(C.c_uint8)]
        L.orc_res_lowest_states.argtypes = [vp, P(C.c_uint8)]
        L.orc_res_best_cost.argtypes = [vp]
        L.orc_res_best_cost.restype = dbl
        L.orc_res_master_state.argtypes = [vp]
        L.orc_res_master_state.restype = C.c_uint64
        L.orc_res_best_state.argtypes = [vp, P(C.c_uint8)]
        L.orc_res_solutions.argtypes = [vp, P(dbl), P(C.c_uint8)]
        L.orc_res_pt_observables.argtypes = [vp, P(dbl)]
        L.orc_res_pa_trace.argtypes = [vp, P(i64), P(dbl), P(i64), i64]
        L.orc_res_destroy.argtypes = [vp]
        L.orc_pt_toy.argtypes = [u32, i64, P(dbl), ip, ip, P(dbl), P(dbl)]
        L.orc_pt_toy.restype = ip
        _libs[release] = L
    return _libs[release]


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


# ---------------------------------------------------------------- rng pins
def pcg_stream(seed=None, n=8):
    out = np.zeros(n, np.uint32)
    lib().orc_pcg_stream(0 if seed is None else seed, 1 if seed is None else 0,
                         n, _p(out, C.c_uint32))
    return out


def pcg_uniform(seed=None, n=8):
    out = np.zeros(n, np.float64)
    lib().orc_pcg_uniform(0 if seed is None else seed, 1 if seed is None else 0,
                          n, _p(out, C.c_double))
    return out


def pcg_fork_uniform(seed, n_forks, n):
    out = np.zeros((n, n_forks + 1), np.float64)
    lib().orc_pcg_fork_uniform(seed, n_forks, n, _p(out, C.c_double))
    return out


def twister_uniform(seed=None, n=8):
    out = np.zeros(n, np.float64)
    lib().orc_twister_uniform(0 if seed is None else seed,
                              1 if seed is None else 0, n, _p(out, C.c_double))
    return out


def uniform_ln():
    out = np.zeros((4, 256), np.float64)
    lib().orc_uniform_ln(_p(out, C.c_double))
    return out


def metropolis_accept(cost_diff, beta, draws):
    d = np.ascontiguousarray(draws, np.uint32)
    used = C.c_int(0)
    a = lib().orc_metropolis_accept(float(cost_diff), float(beta),
                                    _p(d, C.c_uint32), len(d), C.byref(used))
    return bool(a), used.value


def counter_key(seed, stream):
    return lib().orc_counter_key(seed, stream)


def counter_draw(key, ctr):
    return lib().orc_counter_draw(key, ctr)


# ---------------------------------------------------------------- model
def flatten_terms(terms):
    """terms: list of (coef, [ids]) -> (offsets int64, ids int32, coef f64)."""
    off = np.zeros(len(terms) + 1, np.int64)
    for i, (_, ids) in enumerate(terms):
        off[i + 1] = off[i] + len(ids)
    ids = np.fromiter((v for _, t in terms for v in t), np.int32, count=int(off[-1]))
    coef = np.array([c for c, _ in terms], np.float64)
    return off, ids, coef


class Model:
    """release=True builds the model in the Release-flag library (timing
    only); run() then uses that library too."""

    def __init__(self, kind, terms=None, *, off=None, ids=None, coef=None, release=False):
        if isinstance(kind, str):
            kind = KIND_BY_NAME[kind]
        if terms is not None:
            off, ids, coef = flatten_terms(terms)
        self.off = np.ascontiguousarray(off, np.int64)
        self.ids = np.ascontiguousarray(ids, np.int32)
        self.coef = np.ascontiguousarray(coef, np.float64)
        self.kind = kind
        self.L = lib(release)
        err = C.create_string_buffer(512)
        self.h = self.L.orc_model_create(kind, len(self.coef), _p(self.off, C.c_int64),
                                        _p(self.ids, C.c_int32), _p(self.coef, C.c_double),
                                        err, 512)
        if not self.h:
            raise ValueError(err.value.decode())

    def __del__(self):
        if getattr(self, "h", None) and getattr(self, "L", None) is not None:
            self.L.orc_model_destroy(self.h)
            self.h = None

    @property
    def n_vars(self):
        return self.L.orc_model_n_vars(self.h)

    @property
    def n_terms(self):
        return self.L.orc_model_n_terms(self.h)

    @property
    def const_cost(self):
        return self.L.orc_model_const_cost(self.h)

    @property
    def scale_factor(self):
        return self.L.orc_model_scale_factor(self.h)

    def var_names(self):
        out = np.zeros(self.n_vars, np.int32)
        self.L.orc_model_var_names(self.h, _p(out, C.c_int32))
        return out

    def cost(self, spins):
        s = np.ascontiguousarray(spins, np.uint8)
        return self.L.orc_state_cost(self.h, _p(s, C.c_uint8))

    def cost_difference(self, spins, var):
        s = np.ascontiguousarray(spins, np.uint8)
        return self.L.orc_state_cost_difference(self.h, _p(s, C.c_uint8), int(var))

    def twister_min(self, seed, iters, T):
        return self.L.orc_model_twister_min(self.h, seed, iters, T)


def schedule(kind="linear", initial=0.0, final=0.0, values=None, start=None,
             stop=None, count=None):
    s = Schedule()
    s.type = {"linear": SCHED_LINEAR, "geometric": SCHED_GEOMETRIC,
              "constant": SCHED_CONSTANT, "list": SCHED_LIST}[kind]
    s.initial, s.final_value = float(initial), float(final)
    s.has_start, s.start = (start is not None), float(start or 0)
    s.has_stop, s.stop = (stop is not None), float(stop or 0)
    s.has_count, s.count = (count is not None), int(count or 0)
    keep = None
    if values is not None:
        keep = np.ascontiguousarray(values, np.float64)
        s.n_values = len(keep)
        s.values = _p(keep, C.c_double)
    return s, keep


class Result:
    def __init__(self, h, L):
        self.h = h
        n = L.orc_res_n_replicas(h)
        self.n_vars = L.orc_res_n_vars(h)
        self.last_step = L.orc_res_last_step(h)
        self.cost = np.zeros(n)
        self.lowest = np.zeros(n)
        self.attempts = np.zeros(n, np.uint64)
        self.accepts = np.zeros(n, np.uint64)
        if n:
            L.orc_res_replicas(h, _p(self.cost, C.c_double), _p(self.lowest, C.c_double),
                               _p(self.attempts, C.c_uint64), _p(self.accepts, C.c_uint64))
        self.states = np.zeros((n, self.n_vars), np.uint8)
        self.lowest_states = np.zeros((n, self.n_vars), np.uint8)
        if n and self.n_vars:
            L.orc_res_states(h, _p(self.states, C.c_uint8))
            L.orc_res_lowest_states(h, _p(self.lowest_states, C.c_uint8))
        self.best_cost = L.orc_res_best_cost(h)
        self.master_state = L.orc_res_master_state(h)
        self.best_state = np.zeros(self.n_vars, np.uint8)
        L.orc_res_best_state(h, _p(self.best_state, C.c_uint8))
        ns = L.orc_res_n_solutions(h)
        self.solution_costs = np.zeros(ns)
        self.solution_states = np.zeros((ns, self.n_vars), np.uint8)
        if ns:
            L.orc_res_solutions(h, _p(self.solution_costs, C.c_double),
                                _p(self.solution_states, C.c_uint8))
        self.pt_obs = np.zeros((n, 5))
        if n:
            L.orc_res_pt_observables(h, _p(self.pt_obs, C.c_double))
        steps = C.c_int64(0)
        tb = np.zeros(1 << 16)
        tp = np.zeros(1 << 16, np.int64)
        L.orc_res_pa_trace(h, C.byref(steps), _p(tb, C.c_double), _p(tp, C.c_int64), 1 << 16)
        self.pa_beta = tb[:steps.value].copy()
        self.pa_population = tp[:steps.value].copy()
        L.orc_res_destroy(h)
        self.h = None


def run(model: Model, solver="sa", *, seed=0, step_limit=100, restarts=1,
        use_inverse=True, sched=("linear", 0.0, 0.01), sched_values=None,
        sched_count=None, sweeps_per_replica=1, population=16, alpha=2.0,
        constant_population=False, exp_repopulation=False, pa_threads=1,
        rng_mode="replay", threads=1, number_of_solutions=1, cost_limit=None,
        full_maxsat_sweep=False, resampling="reference", master_skip=0, master_state=None,
        tabu_tenure=0, sched2=None, steps_per_walker=1, trotter_number=2, tabu_tenures=None):
    """sched / sched2 are (kind, initial, final) or (kind, initial, final,
    start, stop); SSMC takes alpha from sched and beta from sched2, the
    target population from `population`, its streams from `pa_threads`."""
    p = Params()
    p.solver = {"sa": SA, "pt": PT, "pa": PA, "tabu": TABU, "ssmc": SSMC, "qmc": QMC}[solver]
    p.seed = seed & 0xFFFFFFFF
    p.step_limit = step_limit
    p.restarts = restarts
    p.use_inverse = 1 if use_inverse else 0
    kind, a, b, *rng_ = sched
    p.sched, keep = schedule(kind, a, b, values=sched_values, count=sched_count,
                             start=rng_[0] if rng_ else None, stop=rng_[1] if rng_ else None)
    if sched2 is not None:
        kind2, a2, b2, *rng2 = sched2
        p.sched2, _ = schedule(kind2, a2, b2, start=rng2[0] if rng2 else None,
                               stop=rng2[1] if rng2 else None)
    p.sweeps_per_replica = sweeps_per_replica if solver != "ssmc" else steps_per_walker
    p.population = population
    p.alpha = alpha
    p.constant_population = int(constant_population)
    p.exp_repopulation = int(exp_repopulation)
    p.pa_threads = pa_threads
    p.rng_mode = RNG_REPLAY if rng_mode == "replay" else RNG_COUNTER
    p.threads = threads
    p.number_of_solutions = number_of_solutions
    p.has_cost_limit = cost_limit is not None
    p.cost_limit = float(cost_limit or 0.0)
    p.full_maxsat_sweep = int(full_maxsat_sweep)
    p.resampling = {"reference": 0, "multinomial": 1}[resampling]
    p.master_skip = int(master_skip)
    p.use_master_state = 0 if master_state is None else 1
    p.master_state = 0 if master_state is None else int(master_state)
    p.tabu_tenure = int(tabu_tenure)
    keep_ten = None
    if tabu_tenures is not None:
        keep_ten = np.ascontiguousarray(tabu_tenures, np.int64)
        p.tabu_tenures = _p(keep_ten, C.c_int64)
        p.n_tabu_tenures = len(keep_ten)
    p.trotter_number = int(trotter_number)
    err = C.create_string_buffer(512)
    h = model.L.orc_run(model.h, C.byref(p), err, 512)
    del keep, keep_ten
    if not h:
        raise ValueError(err.value.decode())
    return Result(h, model.L)


def qexp(x):
    """exp of the multinomial resampling mode (x <= 0)."""
    return lib().orc_qexp(float(x))


def pt_toy(seed, steps, temps, use_inverse=False):
    t = np.ascontiguousarray(temps, np.float64)
    obs = np.zeros((len(t), 5))
    best = C.c_double(0)
    lib().orc_pt_toy(seed, steps, _p(t, C.c_double), len(t), int(use_inverse),
                     _p(obs, C.c_double), C.byref(best))
    return obs, best.value


# ---------------------------------------------------------------- parameter-free SA
MIN_DELTA_DEFAULT = 0.1  # model/graph_model.h:16


def _least_diff_one(vals):
    """utils::least_diff_method (one multiset), utils/utils.cc:43-53."""
    s = sorted(vals)
    while len(s) > 1:
        a = s.pop()
        b = s.pop()
        d = a - b
        # keep the list sorted
        lo, hi = 0, len(s)
        while lo < hi:
            mid = (lo + hi) // 2
            if s[mid] <= d:
                lo = mid + 1
            else:
                hi = mid
        s.insert(lo, d)
    return s[0]


def _least_diff_two(a, b):
    """utils::least_diff_method (two multisets), utils/utils.cc:55-100."""
    a, b = sorted(a), sorted(b)
    mn = float(np.finfo(np.float64).max)
    if not a and b:
        return b[0]
    if a and not b:
        return a[0]
    import bisect
    while a and b:
        ca, cb = a.pop(), b.pop()
        d = ca - cb
        if d > 0:
            bisect.insort(a, d)
        elif d < 0:
            d = -d
            bisect.insort(b, d)
        elif len(a) < len(b):
            bisect.insort(a, ca)
        else:
            bisect.insort(b, cb)
        if mn > d and d != 0:
            mn = d
    return mn


def cost_diff_bounds(kind, terms):
    """(estimate_min_cost_diff, estimate_max_cost_diff) of an Ising or PUBO
    term list (model/ising.h:176-224, model/pubo.h:127-184, graph/graph.h:
    453-485): per variable, the coefficients of the terms it appears in
    (constant terms excluded)."""
    inc = {}
    for c, ids in terms:
        for v in set(ids):
            inc.setdefault(v, []).append(float(c))
    ising = kind.startswith("ising")

    def seq_abs_sum(cs):  # left to right in doubles (Python's sum() compensates)
        t = 0.0
        for c in cs:
            t += abs(c)
        return t
    mx = max(seq_abs_sum(cs) for cs in inc.values())
    big = float(np.finfo(np.float64).max)
    mn = big
    for cs in inc.values():
        if ising:
            local = _least_diff_one([abs(c) for c in cs])
        else:
            local = _least_diff_two([c for c in cs if c > 0], [-c for c in cs if c < 0])
        if local == 0:
            continue
        mn = min(mn, local)
    if mn == big:
        mn = MIN_DELTA_DEFAULT
    return (mn * 2, mx * 2) if ising else (mn, mx)


def sa_parameter_free(model: Model, kind, terms, *, seed, min_num_restarts, samples=(10, 20, 30, 50),
                      max_prob=0.5, min_prob=0.0001, adjust=0.001, change=1.5,
                      nonimprovement_limit=8, max_runs=400, threads=4):
    """ParameterFreeLinearSearchSolver<SAParameterFree> restated
    (solver/parameter_free_solver.h:65-151, strategy/linear_search.cc,
    solver/sa_parameter_free.h): repeated oracle SA runs whose restarts fork
    from one continuing master stream.  Returns the per-run trace
    [(sweeps, restarts, lowest)], the best cost and state, and the best run's
    (sweeps, restarts).  Stops on the non-improvement rule (no time limit)."""
    import math
    mn, mx = cost_diff_bounds(kind, terms)
    b0 = -math.log(max_prob) / mx
    b1 = -math.log(min_prob) / (mn + adjust * (mx - mn))
    points = list(samples)
    objs = [float(np.finfo(np.float64).max)] * len(points)
    init_min = points[0]
    cur = -1
    skip = 0
    best = None
    best_state = None
    best_exec = 0.0
    best_params = None
    stable = 0
    trace = []
    for _ in range(max_runs):
        cur += 1
        if cur >= len(points):
            cur = 0
            lowest = objs.index(min(objs))
            if lowest == 0:
                if points[0] > init_min:
                    points = [int(p / change) for p in points]
            elif lowest == len(points) - 1:
                points = [int(p * change) for p in points]
            objs = [float(np.finfo(np.float64).max)] * len(points)
        sweeps, back = points[cur], points[-1]
        sl = max(sweeps, 2)
        r = min_num_restarts * back // sweeps
        res = run(model, "sa", seed=seed, step_limit=sl, restarts=r, use_inverse=True,
                  sched=("linear", b0, b1), threads=threads, master_skip=skip)
        skip += r
        obj = float(res.best_cost)
        objs[cur] = obj
        trace.append((sl, r, obj))
        exec_cost = float(sl) * float(r)
        done = False
        if best is not None and abs(best - obj) < 10E-12:
            stable += 1
            if exec_cost < best_exec:
                best, best_state, best_exec, best_params = obj, res.best_state.copy(), exec_cost, (sl, r)
        if stable >= nonimprovement_limit:
            done = True
        if best is None or best - obj > 10E-12:
            stable = 0
            best, best_state, best_exec, best_params = obj, res.best_state.copy(), exec_cost, (sl, r)
        if done:
            break
    return {"trace": trace, "best": best, "best_state": best_state, "params": best_params,
            "betas": (b0, b1)}


def tabu_tenures(n_tenures, n_vars, denominator=4, max_optimal=20):
    """TabuParameterFree::determine_all_tenures_ (solver/tabu_parameter_free.h:
    86-124): the optimal tenure min(20, N / 4), its half when above 10, then
    tenures stepping by max((N - optimal) / (remaining * 4), 1) below N,
    repeated until n_tenures values."""
    opt = min(max_optimal, n_vars // denominator)
    out = []
    todo = n_tenures
    while todo > 0:
        out.append(opt)
        todo -= 1
        if todo > 0 and opt > max_optimal // 2:
            out.append(opt // 2)
            todo -= 1
        if todo > 0:
            inc = max((n_vars - opt) // (todo * denominator), 1)
            t = opt + inc
            while todo > 0 and t < n_vars:
                out.append(t)
                todo -= 1
                t += inc
    return out


def tabu_parameter_free(model: Model, *, seed, min_num_restarts, samples=(10, 20, 30, 50),
                        change=1.5, nonimprovement_limit=8, max_runs=400, threads=4):
    """ParameterFreeLinearSearchSolver<TabuParameterFree> restated
    (solver/parameter_free_solver.h:65-151, strategy/linear_search.cc,
    solver/tabu_parameter_free.h): repeated oracle tabu runs with the
    tenure list, restarts forking from one master stream that configure()
    already drew once from (replica_rng_ = rng_->fork()).  Returns the trace
    [(sweeps, restarts, lowest)], the best cost and state and its run's
    (sweeps, restarts).  Stops on the non-improvement rule."""
    n_vars = model.n_vars
    points = list(samples)
    objs = [float(np.finfo(np.float64).max)] * len(points)
    init_min = points[0]
    cur = -1
    skip = 1
    best = best_state = best_params = None
    best_exec = 0.0
    stable = 0
    trace = []
    for _ in range(max_runs):
        cur += 1
        if cur >= len(points):
            cur = 0
            lowest = objs.index(min(objs))
            if lowest == 0:
                if points[0] > init_min:
                    points = [int(p / change) for p in points]
            elif lowest == len(points) - 1:
                points = [int(p * change) for p in points]
            objs = [float(np.finfo(np.float64).max)] * len(points)
        sweeps, back = points[cur], points[-1]
        sl = max(sweeps, 2)
        r = min_num_restarts * back // sweeps
        res = run(model, "tabu", seed=seed, step_limit=sl, restarts=r, threads=threads,
                  master_skip=skip, tabu_tenures=tabu_tenures(r, n_vars))
        skip += r
        obj = float(res.best_cost)
        objs[cur] = obj
        trace.append((sl, r, obj))
        exec_cost = float(sl) * float(r)
        done = False
        if best is not None and abs(best - obj) < 10E-12:
            stable += 1
            if exec_cost < best_exec:
                best, best_state, best_exec, best_params = obj, res.best_state.copy(), exec_cost, (sl, r)
        if stable >= nonimprovement_limit:
            done = True
        if best is None or best - obj > 10E-12:
            stable = 0
            best, best_state, best_exec, best_params = obj, res.best_state.copy(), exec_cost, (sl, r)
        if done:
            break
    return {"trace": trace, "best": best, "best_state": best_state, "params": best_params}


def _pf_betas(b0, b1, num):
    """PTParameterFree::determine_all_betas_ (solver/pt_parameter_free.h:
    155-173): geometric ladders of 4, 9, 14, ... values from b0 to b1,
    concatenated until `num` values."""
    out = []
    size = 5
    while len(out) < num:
        n = size - 1
        for i in range(n):
            p = min(1.0, max(0.0, i / (n - 1)))
            out.append(b0 * (b1 / b0) ** p)
            if len(out) >= num:
                break
        size += 5
    return out


def pt_parameter_free(model: Model, kind, terms, *, seed, min_num_betas, samples=(10, 20, 30, 50),
                      max_prob=0.5, min_prob=0.0001, adjust=0.001, change=1.5,
                      nonimprovement_limit=8, max_runs=400, threads=4):
    """ParameterFreeLinearSearchSolver<PTParameterFree> restated
    (solver/parameter_free_solver.h:65-151, strategy/linear_search.cc,
    solver/pt_parameter_free.h): repeated oracle PT runs on one master stream
    (replica forks and swap draws) that continues from run to run."""
    import math
    mn, mx = cost_diff_bounds(kind, terms)
    b0 = -math.log(max_prob) / mx
    b1 = -math.log(min_prob) / (mn + adjust * (mx - mn))
    betas = _pf_betas(b0, b1, min_num_betas)
    big = float(np.finfo(np.float64).max)
    points = list(samples)
    objs = [big] * len(points)
    init_min = points[0]
    cur = -1
    state = None
    best = best_state = best_params = None
    best_exec = 0.0
    stable = 0
    trace = []
    for _ in range(max_runs):
        cur += 1
        if cur >= len(points):
            cur = 0
            lowest = objs.index(min(objs))
            if lowest == 0:
                if points[0] > init_min:
                    points = [int(p / change) for p in points]
            elif lowest == len(points) - 1:
                points = [int(p * change) for p in points]
            objs = [big] * len(points)
        sl = max(points[cur], 2)
        res = run(model, "pt", seed=seed, step_limit=sl, use_inverse=True, sched=("list", 0.0, 0.0),
                  sched_values=betas, threads=threads, master_state=state)
        state = res.master_state
        obj = float(res.best_cost)
        objs[cur] = obj
        trace.append((sl, len(betas), obj))
        exec_cost = float(sl) * float(len(betas))
        done = False
        if best is not None and abs(best - obj) < 10E-12:
            stable += 1
            if exec_cost < best_exec:
                best, best_state, best_exec, best_params = obj, res.best_state.copy(), exec_cost, sl
        if stable >= nonimprovement_limit:
            done = True
        if best is None or best - obj > 10E-12:
            stable = 0
            best, best_state, best_exec, best_params = obj, res.best_state.copy(), exec_cost, sl
        if done:
            break
    return {"trace": trace, "best": best, "best_state": best_state, "sweeps": best_params,
            "betas": betas}


# ------------------------------------------- parameter-free PA / SSMC (replay)
_PCG_MULT, _PCG_INC = 6364136223846793005, 1442695040888963407


def _pcg_seed_state(seed):
    """The state of a PCG32 stream seeded with `seed` (Pcg32::seed64)."""
    return ((seed + _PCG_INC) * _PCG_MULT + _PCG_INC) % (1 << 64)


def _pcg_u32(state):
    """One 32-bit output of the stream in `state`: (value, next state)."""
    st = C.c_uint64(state)
    x = lib().orc_pcg_state_u32(C.byref(st))
    return int(x), st.value


def _pcg_draw(state):
    """One uniform() of the stream in `state`: (value, next state)."""
    st = C.c_uint64(state)
    u = lib().orc_pcg_state_uniform(C.byref(st))
    return u, st.value


def pa_parameter_free_replay(model: Model, kind, terms, *, seed, threads, runs, initial_samples=4,
                             initial_sweeps=20, initial_alpha=2.0, initial_min_prob_log=2.0,
                             max_prob=0.5, max_population_mult=128, alpha_low=1.00000001,
                             budget_s=None, rng_mode="replay", resampling="reference"):
    """The runs of a parameter-free population-annealing search
    (solver/parameter_free_solver.h:65-151 with solver/pa_parameter_free.h)
    replayed on one master stream: the first `initial_samples` parameter
    vectors from the adapter's initial values (get_initial_parameter_values,
    :228-260, the alpha jitter drawn from the master), later ones as given
    in `runs` (the strategy's picks), each applied as update_parameters
    (:262-330) and run by the oracle's PA from the master's state (with
    counter streams, each run keys them with one master draw).  Returns
    [(params, step_limit, lowest, lowest state)] for as many runs as `runs`
    lists (fewer
    when `budget_s` seconds have passed).  The walker cap is threads x
    max_population_mult (memory is not the limit)."""
    import time
    t_start = time.perf_counter()
    mn_mx = cost_diff_bounds(kind, terms)
    mn, mx = mn_mx
    beta_start = -math.log(max_prob) / mx
    cap = threads * max_population_mult

    def adjust(x):
        r = min(int(x), cap)
        return max(r, threads) if cap > threads else cap

    state = _pcg_seed_state(seed & 0xFFFFFFFF)
    out = []
    for k, given in enumerate(runs):
        if k < initial_samples:
            u, state = _pcg_draw(state)
            v = [float(initial_sweeps + k * 10), float(adjust(threads * (k + 1))),
                 initial_alpha + 0.5 * (u - 0.5), k + 1.0, initial_min_prob_log + k * 2]
        else:
            v = list(given)
        spr = max(1, int(round(v[3])))
        sl = max(int(math.ceil(v[0] / spr)), 2)
        pop = adjust(v[1])
        alpha = max(v[2], alpha_low)
        b1 = v[4] / mn
        run_seed = seed
        if rng_mode == "counter":
            run_seed, state = _pcg_u32(state)
        res = run(model, "pa", seed=run_seed, master_state=state, step_limit=sl, sweeps_per_replica=spr,
                  population=pop, alpha=alpha, sched=("geometric", beta_start, b1), pa_threads=threads,
                  threads=min(threads, 16), rng_mode=rng_mode, resampling=resampling)
        state = res.master_state
        out.append((v, sl, float(res.best_cost), res.best_state.copy()))
        if budget_s is not None and time.perf_counter() - t_start > budget_s:
            break
    return out


def ssmc_parameter_free_replay(model: Model, *, seed, threads, runs, sweep_size, initial_samples=4,
                               initial_sweeps=20, initial_spw=1, initial_alpha_final=0.00001,
                               initial_alpha_scope=0.8, initial_beta_initial=0.00001,
                               initial_beta_scope=5.0, max_replica_mult=3, rng_mode="replay"):
    """The runs of a parameter-free SSMC search (solver/ssmc_parameter_free.h
    get_initial_parameter_values :160-178, update_parameters :180-224) on one
    master stream, as pa_parameter_free_replay does for PA."""
    cap = threads * max_replica_mult

    def adjust(x):
        r = min(int(x), cap)
        return max(r, threads) if cap > threads else cap

    state = _pcg_seed_state(seed & 0xFFFFFFFF)
    out = []
    for k, given in enumerate(runs):
        if k < initial_samples:
            u, state = _pcg_draw(state)
            v = [float(initial_sweeps * sweep_size * (1 + k)), float(min(threads + k, cap)), float(initial_spw),
                 initial_alpha_final, initial_alpha_scope, initial_beta_initial, initial_beta_scope + u]
        else:
            v = list(given)
        sl = max(int(math.floor(v[0])), 2)
        pop = adjust(v[1])
        spw = max(int(v[2]), 1)
        run_seed = seed
        if rng_mode == "counter":
            run_seed, state = _pcg_u32(state)
        res = run(model, "ssmc", seed=run_seed, master_state=state, step_limit=sl, population=pop,
                  pa_threads=threads, threads=min(threads, 16), steps_per_walker=spw,
                  sched=("linear", v[3] + v[4], v[3]), sched2=("linear", v[5], v[5] + v[6]),
                  rng_mode=rng_mode)
        state = res.master_state
        out.append((v, sl, float(res.best_cost), res.best_state.copy()))
    return out

