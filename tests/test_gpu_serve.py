"""Serving (qio_server_*): each request's result is the same alone and in a
mix, and equals the plain solver's (tolerance: exact -- the pieces replay
the same trajectory)."""
import time

import numpy as np
import pytest

import qiotoolkit_gb300 as q
from qiotoolkit_gb300 import instances as I

pytestmark = pytest.mark.gpu

SA = "simulatedannealing.qiotoolkit"
PT = "paralleltempering.qiotoolkit"


def _strip(res):
    res = dict(res)
    b = dict(res["benchmark"])
    b.pop("gb300", None)
    res["benchmark"] = b
    return res


def _requests():
    reqs = []
    off, ids, coef = I.er_ising(400, 1600, seed=51)
    reqs.append((q.Model("ising", off=off, ids=ids, coef=coef), SA,
                 {"seed": 1, "sweeps": 150, "restarts": 8, "beta_start": 0.1, "beta_stop": 3.0}))
    off, ids, coef = I.random_pubo(300, 900, seed=52)
    reqs.append((q.Model("pubo", off=off, ids=ids, coef=coef), PT,
                 {"seed": 2, "sweeps": 40, "temperatures": {"type": "geometric", "initial": 0.1,
                                                            "final": 3.0, "count": 8}}))
    off, ids, coef = I.weighted_maxsat(120, seed=53)
    reqs.append((q.Model("maxsat", off=off, ids=ids, coef=coef), SA,
                 {"seed": 3, "sweeps": 90, "restarts": 4, "beta_start": 0.1, "beta_stop": 2.0,
                  "maxsat_full_sweep": True}))
    off, ids, coef = I.cubic_pm_j(5, seed=54)
    reqs.append((q.Model("ising", off=off, ids=ids, coef=coef), SA,
                 {"seed": 4, "sweeps": 200, "restarts": 16, "beta_start": 0.1, "beta_stop": 3.0,
                  "rng_mode": "counter"}))
    off, ids, coef = I.random_pubo(200, 600, seed=55, integer=True)
    reqs.append((q.Model("pubo", off=off, ids=ids, coef=coef), PT,
                 {"seed": 5, "sweeps": 30, "all_betas": [0.2, 0.6, 1.2, 2.5], "restarts": 2}))
    return reqs


def test_serving_same_alone_and_in_mix():
    reqs = _requests()
    plain = [_strip(q.Solver(m, t, {"params": p}).init().run().result()) for m, t, p in reqs]
    # alone: one slot, requests one after another
    alone = q.Server(max_active=1, sa_sweeps_per_piece=37, pt_steps_per_piece=7)
    ids = [alone.submit(m, t, {"params": p}) for m, t, p in reqs]
    res_alone = [_strip(alone.wait(i)) for i in ids]
    assert alone.stats().peak_active == 1
    alone.close()
    # mix: all at once, overlapping pieces, submitted in another order
    mix = q.Server(max_active=16, sa_sweeps_per_piece=16, pt_steps_per_piece=3)
    order = [3, 0, 4, 1, 2]
    ids = {k: mix.submit(reqs[k][0], reqs[k][1], {"params": reqs[k][2]}) for k in order}
    res_mix = {k: _strip(mix.wait(ids[k])) for k in order}
    st = mix.stats()
    assert st.completed == len(reqs) and st.failed == 0 and st.peak_active > 1
    assert st.p99_ms >= st.p50_ms > 0
    mix.close()
    for k in range(len(reqs)):
        assert res_alone[k] == plain[k]
        assert res_mix[k] == plain[k]


def test_serving_admission_by_memory():
    """Equal requests under a budget of one footprint run one at a time, and
    still give the plain solver's results."""
    m, t, p = _requests()[0]
    params = [dict(p, seed=s) for s in (11, 12, 13)]
    probe = q.Server(max_active=8)
    rid = probe.submit(m, t, {"params": params[0]})
    size = probe.request_bytes(rid)
    probe.wait(rid)
    probe.close()
    srv = q.Server(memory_budget_bytes=size, max_active=8)
    ids = [srv.submit(m, t, {"params": pp}) for pp in params]
    out = [_strip(srv.wait(i)) for i in ids]
    st = srv.stats()
    assert st.peak_active == 1 and st.used_bytes == 0 and st.completed == 3
    for o, pp in zip(out, params):
        assert o == _strip(q.Solver(m, t, {"params": pp}).init().run().result())


def test_serving_rejects_and_polls():
    m, t, p = _requests()[0]
    srv = q.Server(max_active=2)
    with pytest.raises(q.QioError, match="cost_limit"):
        srv.submit(m, t, {"params": dict(p, cost_limit=-5)})
    rid = srv.submit(m, t, {"params": p})
    t0 = time.time()
    res = None
    while res is None and time.time() - t0 < 60:
        res = srv.poll(rid)
        time.sleep(0.01)
    assert res is not None and "solutions" in res
    srv.forget(rid)
    srv.close()
