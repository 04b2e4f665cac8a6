"""Tabu search (tabu.qiotoolkit) on the device against the oracle.

The reference's TabuWalker (markov/tabu_walker.h:60-129) is deterministic
once its random start state is drawn: the scan takes the first variable whose
flip beats the walker's lowest cost, otherwise the lowest-difference variable
off the tabu list (first on ties), and an improving flip hands over to a
hill climber until a sweep stops improving.  Bar: bit-exact per walker (final
and lowest cost, difference evaluations, accepted transitions, final and
lowest states).
"""
import numpy as np
import pytest

import qiotoolkit_gb300 as q
from qiotoolkit_gb300 import instances as I
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TABU = "tabu.qiotoolkit"

MODELS = {
    "ising_real": ("ising", lambda: I.er_ising(300, 900, seed=11)),
    "ising_int": ("ising", lambda: I.cubic_pm_j(6, seed=12)),
    "ising_plain": ("ising_plain", lambda: I.er_ising(200, 600, seed=13)),
    "pubo_real": ("pubo", lambda: I.random_pubo(400, 1600, seed=14)),
    "pubo_int": ("pubo", lambda: I.random_pubo(300, 1200, seed=15, integer=True)),
    "pubo_plain": ("pubo_plain", lambda: I.random_pubo(200, 700, seed=16)),
    # fewer variables than one 32-variable scan chunk
    "small": ("ising", lambda: I.er_ising(20, 40, seed=3)),
}


def same(s, r):
    g = s.replicas()
    np.testing.assert_array_equal(g["cost"], r.cost)
    np.testing.assert_array_equal(g["lowest"], r.lowest)
    np.testing.assert_array_equal(g["attempts"], r.attempts)
    np.testing.assert_array_equal(g["accepts"], r.accepts)
    np.testing.assert_array_equal(g["states"], r.states)
    np.testing.assert_array_equal(g["lowest_states"], r.lowest_states)
    c, _ = s.best()
    assert c == r.best_cost


@pytest.mark.parametrize("name", list(MODELS))
@pytest.mark.parametrize("mode", ["replay", "counter"])
@pytest.mark.parametrize("tenure", [0, 7])
def test_tabu_walkers(name, mode, tenure):
    kind, gen = MODELS[name]
    off, ids, coef = gen()
    g = q.Model(kind, off=off, ids=ids, coef=coef)
    o = O.Model(kind, off=off, ids=ids, coef=coef)
    params = {"seed": 31, "sweeps": 40, "restarts": 9, "tabu_tenure": tenure, "rng_mode": mode}
    s = q.Solver(g, TABU, {"params": params}).init().run()
    r = O.run(o, "tabu", seed=31, step_limit=40, restarts=9, tabu_tenure=tenure,
              rng_mode=mode, threads=4)
    same(s, r)


def test_tabu_many_walkers_long():
    """More walkers than one block holds and enough sweeps for the tabu list
    to expire and the hill climber to hand back many times."""
    off, ids, coef = I.cubic_pm_j(8, seed=5)
    g = q.Model("ising", off=off, ids=ids, coef=coef)
    o = O.Model("ising", off=off, ids=ids, coef=coef)
    params = {"seed": 77, "sweeps": 300, "restarts": 70, "tabu_tenure": 12}
    s = q.Solver(g, TABU, {"params": params}).init().run()
    r = O.run(o, "tabu", seed=77, step_limit=300, restarts=70, tabu_tenure=12, threads=8)
    same(s, r)
    # lowest states recompute to the lowest costs (integer couplings: exact)
    rep = s.replicas()
    np.testing.assert_array_equal(g.calculate_cost(rep["lowest_states"]), rep["lowest"])


def test_tabu_result_document():
    off, ids, coef = I.er_ising(120, 360, seed=2)
    g = q.Model("ising", off=off, ids=ids, coef=coef)
    s = q.Solver(g, TABU, {"params": {"seed": 4, "sweeps": 25, "restarts": 3,
                                      "tabu_tenure": 2}}).init().run()
    doc = s.result()
    assert doc["solutions"]["parameters"]["tabu_tenure"] == 2
    assert doc["solutions"]["parameters"]["restarts"] == 3
    c, st = s.best()
    assert g.calculate_cost(st[None, :])[0] == pytest.approx(c, abs=1e-9)


def test_tabu_pieces_and_time_limit():
    """A solve served in pieces of 7 sweeps (the walker state, cached
    differences and tabu list stay on the device between launches) and a
    solve under a time limit (launches of step_limit / 100 sweeps) give the
    plain solve's walkers."""
    off, ids, coef = I.random_pubo(200, 700, seed=6)
    g = q.Model("pubo", off=off, ids=ids, coef=coef)
    o = O.Model("pubo", off=off, ids=ids, coef=coef)
    p = {"seed": 8, "sweeps": 60, "restarts": 5, "tabu_tenure": 4}
    s = q.Solver(g, TABU, {"params": p}).init().run()
    same(s, O.run(o, "tabu", seed=8, step_limit=60, restarts=5, tabu_tenure=4))
    srv = q.Server(max_active=4, sa_sweeps_per_piece=7)
    try:
        res = srv.wait(srv.submit(g, TABU, {"params": p}))
    finally:
        srv.close()
    assert res["solutions"] == s.result()["solutions"]
    t = q.Solver(g, TABU, {"params": dict(p, timeout=1000)}).init().run()
    same(t, O.run(o, "tabu", seed=8, step_limit=60, restarts=5, tabu_tenure=4))
    assert t.stats().kernel_launches > s.stats().kernel_launches


@pytest.mark.parametrize("full", [False, True])
@pytest.mark.parametrize("mode", ["replay", "counter"])
def test_tabu_maxsat(full, mode):
    """MaxSat sweeps get_sweep_size() variables (1, the reference's default,
    or all with maxsat_full_sweep); states drawn one uniform() per variable."""
    off, ids, coef = I.weighted_maxsat(120, seed=17)
    g = q.Model("maxsat", off=off, ids=ids, coef=coef)
    o = O.Model("maxsat", off=off, ids=ids, coef=coef)
    params = {"seed": 5, "sweeps": 30, "restarts": 7, "tabu_tenure": 3, "rng_mode": mode,
              "maxsat_full_sweep": full}
    s = q.Solver(g, TABU, {"params": params}).init().run()
    r = O.run(o, "tabu", seed=5, step_limit=30, restarts=7, tabu_tenure=3, rng_mode=mode,
              full_maxsat_sweep=full)
    same(s, r)
