"""Python mirror of the reference's model/solver plugin API over the C ABI.

Model      ~ markov::Model (calculate_cost / calculate_cost_difference /
             apply_transition), built from the reference's term list or JSON.
Solver     ~ solver::Solver (configure from params, init, run, get_result),
             selected by the reference's `target` strings.
run_json   ~ app::Runner::run.
"""
from __future__ import annotations

import ctypes as C
import json
from typing import Iterable, Sequence

import numpy as np

from ._lib import ModelInfo, QioError, SolverStats, check, load

KINDS = {"ising": 0, "ising_plain": 1, "pubo": 2, "pubo_plain": 3, "maxsat": 4}
TARGETS = ("simulatedannealing.qiotoolkit", "paralleltempering.qiotoolkit",
           "populationannealing.cpu", "simulatedannealing-parameterfree.qiotoolkit",
           "paralleltempering-parameterfree.qiotoolkit", "tabu.qiotoolkit",
           "substochasticmontecarlo.cpu", "quantummontecarlo.qiotoolkit",
           "tabu-parameterfree.qiotoolkit", "populationannealing-parameterfree.cpu",
           "substochasticmontecarlo-parameterfree.cpu")


def _ptr(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def flatten_terms(terms: Iterable[Sequence]):
    """[(c, [ids...]), ...] -> (offsets int64, ids int32, coef float64)."""
    terms = list(terms)
    off = np.zeros(len(terms) + 1, np.int64)
    for i, (_, ids) in enumerate(terms):
        off[i + 1] = off[i] + len(ids)
    ids = np.fromiter((v for _, t in terms for v in t), np.int32, count=int(off[-1]))
    coef = np.array([c for c, _ in terms], np.float64)
    return off, ids, coef


class Model:
    def __init__(self, kind, terms=None, *, off=None, ids=None, coef=None, _handle=None):
        L = load()
        if _handle is not None:
            self._h = _handle
        else:
            if isinstance(kind, str):
                kind = KINDS[kind]
            if terms is not None:
                off, ids, coef = flatten_terms(terms)
            off = np.ascontiguousarray(off, np.int64)
            ids = np.ascontiguousarray(ids, np.int32)
            coef = np.ascontiguousarray(coef, np.float64)
            h = C.c_void_p()
            check(L.qio_model_create(int(kind), len(coef), _ptr(off, C.c_int64),
                                     _ptr(ids, C.c_int32), _ptr(coef, C.c_double),
                                     C.byref(h)))
            self._h = h
        info = ModelInfo()
        check(L.qio_model_get_info(self._h, C.byref(info)))
        self.info = info

    @classmethod
    def from_json(cls, doc, kind: int = -1) -> "Model":
        if not isinstance(doc, str):
            doc = json.dumps(doc)
        h = C.c_void_p()
        check(load().qio_model_create_json(doc.encode(), int(kind), C.byref(h)))
        return cls(None, _handle=h)

    def cost_diff_bounds(self):
        """(min, max) estimates of one flip's cost difference."""
        lo, hi = C.c_double(), C.c_double()
        check(load().qio_model_cost_diff_bounds(self._h, C.byref(lo), C.byref(hi)))
        return lo.value, hi.value

    @classmethod
    def from_proto_folder(cls, path: str) -> "Model":
        """Model from a protobuf problem folder (<name>/<name>_<k>.pb)."""
        h = C.c_void_p()
        check(load().qio_model_create_proto_folder(str(path).encode(), C.byref(h)))
        return cls(None, _handle=h)

    @classmethod
    def from_dimacs(cls, text: str) -> "Model":
        """MaxSAT model from DIMACS cnf / wcnf text."""
        h = C.c_void_p()
        check(load().qio_model_create_dimacs(text.encode(), C.byref(h)))
        return cls(None, _handle=h)

    def close(self):
        if getattr(self, "_h", None):
            load().qio_model_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n_vars(self) -> int:
        return self.info.n_vars

    @property
    def n_terms(self) -> int:
        return self.info.n_terms

    @property
    def const_cost(self) -> float:
        return self.info.const_cost

    def var_names(self) -> np.ndarray:
        out = np.zeros(self.n_vars, np.int32)
        check(load().qio_model_get_var_names(self._h, _ptr(out, C.c_int32)))
        return out

    def _states(self, states):
        s = np.ascontiguousarray(states, np.uint8)
        if s.ndim == 1:
            s = s[None, :]
        if s.shape[1] != self.n_vars:
            raise ValueError("state width must equal n_vars")
        return s

    def calculate_cost(self, states, stream=None) -> np.ndarray:
        s = self._states(states)
        out = np.zeros(len(s))
        check(load().qio_states_cost(self._h, len(s), _ptr(s, C.c_uint8),
                                     _ptr(out, C.c_double), stream))
        return out

    def calculate_cost_difference(self, states, vars, stream=None) -> np.ndarray:
        s = self._states(states)
        v = np.ascontiguousarray(np.broadcast_to(np.asarray(vars, np.int64), (len(s),)))
        out = np.zeros(len(s))
        check(load().qio_states_cost_difference(self._h, len(s), _ptr(s, C.c_uint8),
                                                _ptr(v, C.c_int64), _ptr(out, C.c_double),
                                                stream))
        return out

    def apply_transition(self, states, vars) -> np.ndarray:
        s = self._states(states).copy()
        v = np.ascontiguousarray(np.broadcast_to(np.asarray(vars, np.int64), (len(s),)))
        check(load().qio_states_apply(self._h, len(s), _ptr(s, C.c_uint8), _ptr(v, C.c_int64)))
        return s


class Solver:
    def __init__(self, model: Model, target: str, params: dict | str):
        if not isinstance(params, str):
            params = json.dumps(params if "params" in params else {"params": params})
        self.model = model
        h = C.c_void_p()
        check(load().qio_solver_create(model._h, target.encode(), params.encode(), C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            load().qio_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init(self, stream=None):
        check(load().qio_solver_init(self._h, stream))
        return self

    def run(self, stream=None):
        check(load().qio_solver_run(self._h, stream))
        return self

    def result(self) -> dict:
        p = C.c_void_p()
        L = load()
        check(L.qio_solver_result_json(self._h, C.byref(p)))
        try:
            return json.loads(C.string_at(p).decode())
        finally:
            L.qio_free(p)

    def replicas(self, states: bool = True) -> dict:
        L = load()
        n = C.c_int64(0)
        check(L.qio_solver_replicas(self._h, C.byref(n), None, None, None, None, None, None))
        n = n.value
        N = self.model.n_vars
        out = {"cost": np.zeros(n), "lowest": np.zeros(n),
               "attempts": np.zeros(n, np.uint64), "accepts": np.zeros(n, np.uint64)}
        ls = np.zeros((n, N), np.uint8) if states else None
        st = np.zeros((n, N), np.uint8) if states else None
        nn = C.c_int64(0)
        check(L.qio_solver_replicas(
            self._h, C.byref(nn), _ptr(out["cost"], C.c_double), _ptr(out["lowest"], C.c_double),
            _ptr(out["attempts"], C.c_uint64), _ptr(out["accepts"], C.c_uint64),
            _ptr(ls, C.c_uint8) if states and n and N else None,
            _ptr(st, C.c_uint8) if states and n and N else None))
        if states:
            out["lowest_states"] = ls
            out["states"] = st
        return out

    def best(self):
        c = C.c_double(0)
        s = np.zeros(max(self.model.n_vars, 1), np.uint8)
        check(load().qio_solver_best(self._h, C.byref(c), _ptr(s, C.c_uint8)))
        return c.value, s[:self.model.n_vars]

    def stats(self) -> SolverStats:
        s = SolverStats()
        check(load().qio_solver_get_stats(self._h, C.byref(s)))
        return s

    def pt_observables(self) -> np.ndarray:
        n = self.stats().replicas
        out = np.zeros((n, 5))
        if n:
            check(load().qio_solver_pt_observables(self._h, _ptr(out, C.c_double)))
        return out


def run_json(input_json, params_json, target: str) -> dict:
    """app::Runner::run: model JSON + params JSON + target -> result dict."""
    if not isinstance(input_json, str):
        input_json = json.dumps(input_json)
    if not isinstance(params_json, str):
        params_json = json.dumps(params_json)
    L = load()
    p = C.c_void_p()
    check(L.qio_run_json(input_json.encode(), params_json.encode(), target.encode(), C.byref(p)))
    try:
        return json.loads(C.string_at(p).decode())
    finally:
        L.qio_free(p)


def bayes_recommend(ranges, xs, ys, *, seed: int = 0, count: int = 1) -> np.ndarray:
    """The parameter-free solvers' Bayesian strategy on caller samples:
    `count` points in the box `ranges` [(lo, hi), ...] expected to improve on
    the lowest of the objectives ys at the points xs (n x dims)."""
    r = np.ascontiguousarray(ranges, np.float64).reshape(-1, 2)
    d = r.shape[0]
    x = np.ascontiguousarray(xs, np.float64).reshape(-1, d)
    y = np.ascontiguousarray(ys, np.float64).reshape(-1)
    if x.shape[0] != y.shape[0]:
        raise ValueError("xs and ys differ in length")
    lo, hi = np.ascontiguousarray(r[:, 0]), np.ascontiguousarray(r[:, 1])
    out = np.zeros((count, d))
    D = C.c_double
    check(load().qio_bayes_recommend(d, _ptr(lo, D), _ptr(hi, D), x.shape[0], _ptr(x, D), _ptr(y, D),
                                     seed & 0xFFFFFFFF, count, _ptr(out, D)))
    return out


class Batch:
    """Independent solves of many models with one target and params, run as
    one captured CUDA graph (qio_batch_*).  Instance i's result equals
    Solver(models[i], target, params).init().run().result()."""

    def __init__(self, models, target: str, params: dict | str):
        if not isinstance(params, str):
            params = json.dumps(params if "params" in params else {"params": params})
        self.models = list(models)
        arr = (C.c_void_p * len(self.models))(*[m._h.value if isinstance(m._h, C.c_void_p) else m._h
                                                for m in self.models])
        h = C.c_void_p()
        check(load().qio_batch_create(arr, len(self.models), target.encode(), params.encode(),
                                      C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            load().qio_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, stream=None):
        check(load().qio_batch_run(self._h, stream))
        return self

    def result(self, i: int) -> dict:
        p = C.c_void_p()
        L = load()
        check(L.qio_batch_result_json(self._h, i, C.byref(p)))
        try:
            return json.loads(C.string_at(p).decode())
        finally:
            L.qio_free(p)

    def lowest(self) -> np.ndarray:
        out = np.zeros(len(self.models))
        check(load().qio_batch_lowest(self._h, _ptr(out, C.c_double)))
        return out

    def stats(self):
        from ._lib import BatchStats
        st = BatchStats()
        check(load().qio_batch_get_stats(self._h, C.byref(st)))
        return st


class Server:
    """Continuous batching of solve requests (qio_server_*): requests are
    admitted by device footprint, solved resident on the device in
    overlapping pieces, and retired when their sweeps are spent.  A result
    equals Solver(model, target, params)'s for the same inputs."""

    PENDING, RUNNING, DONE, FAILED = 0, 1, 2, 3

    def __init__(self, memory_budget_bytes: int = 0, max_active: int = 64,
                 sa_sweeps_per_piece: int = 64, pt_steps_per_piece: int = 16):
        cfg = json.dumps({"memory_budget_bytes": memory_budget_bytes, "max_active": max_active,
                          "sa_sweeps_per_piece": sa_sweeps_per_piece,
                          "pt_steps_per_piece": pt_steps_per_piece})
        h = C.c_void_p()
        check(load().qio_server_create(cfg.encode(), C.byref(h)))
        self._h = h
        self._models = {}  # keep models alive until their requests finish

    def close(self):
        if getattr(self, "_h", None):
            load().qio_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, model: Model, target: str, params: dict | str) -> int:
        if not isinstance(params, str):
            params = json.dumps(params if "params" in params else {"params": params})
        rid = C.c_int64()
        check(load().qio_server_submit(self._h, model._h, target.encode(), params.encode(),
                                       C.byref(rid)))
        self._models[rid.value] = model
        return rid.value

    def _finish(self, rid, state, p):
        L = load()
        text = None
        if p.value:
            try:
                text = C.string_at(p).decode()
            finally:
                L.qio_free(p)
        if state >= self.DONE:
            self._models.pop(rid, None)
        if state == self.DONE:
            return json.loads(text)
        if state == self.FAILED:
            raise QioError(6, text or "request failed")
        return None

    def poll(self, rid: int):
        """The result dict when done, None while pending or running."""
        st, p = C.c_int32(), C.c_void_p()
        check(load().qio_server_poll(self._h, rid, C.byref(st), C.byref(p)))
        return self._finish(rid, st.value, p)

    def wait(self, rid: int, timeout_s: float = -1.0):
        st, p = C.c_int32(), C.c_void_p()
        check(load().qio_server_wait(self._h, rid, float(timeout_s), C.byref(st), C.byref(p)))
        return self._finish(rid, st.value, p)

    def forget(self, rid: int):
        check(load().qio_server_forget(self._h, rid))

    def request_bytes(self, rid: int) -> int:
        b = C.c_int64()
        check(load().qio_server_request_bytes(self._h, rid, C.byref(b)))
        return b.value

    def stats(self):
        from ._lib import ServerStats
        st = ServerStats()
        check(load().qio_server_get_stats(self._h, C.byref(st)))
        return st

