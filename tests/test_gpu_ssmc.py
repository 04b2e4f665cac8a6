"""Substochastic Monte Carlo (substochasticmontecarlo.cpu) on the device
against the oracle.

Replay streams emulate the reference's OpenMP threads (`threads` PCG streams
forked from the master, each serving a contiguous block of walkers); counter
streams key each walker slot.  Resampling runs in the reference's host
arithmetic.  Bar: bit-exact per walker (cost, lowest, difference evaluations,
accepted transitions, states, lowest states) and the solver's best.
"""
import numpy as np
import pytest

import qiotoolkit_gb300 as q
from qiotoolkit_gb300 import instances as I
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SSMC = "substochasticmontecarlo.cpu"

MODELS = {
    "ising_real": ("ising", lambda: I.er_ising(300, 900, seed=11)),
    "ising_int": ("ising", lambda: I.cubic_pm_j(6, seed=12)),
    "ising_plain": ("ising_plain", lambda: I.er_ising(200, 600, seed=13)),
    "pubo_real": ("pubo", lambda: I.random_pubo(400, 1600, seed=14)),
    "pubo_int": ("pubo", lambda: I.random_pubo(300, 1200, seed=15, integer=True)),
    "pubo_plain": ("pubo_plain", lambda: I.random_pubo(200, 700, seed=16)),
    "maxsat_real": ("maxsat", lambda: I.weighted_maxsat(150, seed=17)),
    "maxsat_int": ("maxsat", lambda: I.weighted_maxsat(120, seed=18, integer=True)),
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
def test_ssmc_walkers(name, mode):
    kind, gen = MODELS[name]
    off, ids, coef = gen()
    g = q.Model(kind, off=off, ids=ids, coef=coef)
    o = O.Model(kind, off=off, ids=ids, coef=coef)
    # 37 walkers over 4 streams: uneven blocks of 10, 9, 9, 9
    params = {"seed": 5, "sweeps": 60, "target_population": 37, "steps_per_walker": 3,
              "threads": 4, "rng_mode": mode}
    s = q.Solver(g, SSMC, {"params": params}).init().run()
    r = O.run(o, "ssmc", seed=5, step_limit=60, population=37, pa_threads=4,
              steps_per_walker=3, sched=("linear", 1.0, 0.0), sched2=("linear", 0.0, 5.0),
              rng_mode=mode)
    same(s, r)


def test_ssmc_schedules_with_ranges():
    """alpha / beta with start and stop (the reference's toy-model test
    shape, solver/test/substochastic_monte_carlo_test.cc:54-89)."""
    off, ids, coef = I.er_ising(150, 450, seed=4)
    g = q.Model("ising", off=off, ids=ids, coef=coef)
    o = O.Model("ising", off=off, ids=ids, coef=coef)
    params = {"seed": 42, "target_population": 100, "step_limit": 300, "threads": 8,
              "alpha": {"type": "linear", "start": 60, "stop": 240, "initial": 0.8, "final": 0.2},
              "beta": {"type": "linear", "start": 60, "stop": 240, "initial": 0.2, "final": 0.8},
              "number_of_solutions": 2}
    s = q.Solver(g, SSMC, {"params": params}).init().run()
    r = O.run(o, "ssmc", seed=42, step_limit=300, population=100, pa_threads=8,
              sched=("linear", 0.8, 0.2, 60, 240), sched2=("linear", 0.2, 0.8, 60, 240))
    same(s, r)
    doc = s.result()
    par = doc["solutions"]["parameters"]
    assert par["target_population"] == 100
    assert par["alpha"]["initial"] == 0.8 and par["beta"]["final"] == 0.8
    assert len(doc["solutions"]["solutions"]) == 2


def test_ssmc_pieces():
    """Served in pieces of 7 steps: the same walkers and result."""
    off, ids, coef = I.random_pubo(150, 500, seed=6)
    g = q.Model("pubo", off=off, ids=ids, coef=coef)
    p = {"seed": 9, "sweeps": 40, "target_population": 24, "threads": 4}
    s = q.Solver(g, SSMC, {"params": p}).init().run()
    srv = q.Server(max_active=4, sa_sweeps_per_piece=7)
    try:
        res = srv.wait(srv.submit(g, SSMC, {"params": p}))
    finally:
        srv.close()
    assert res["solutions"] == s.result()["solutions"]
