"""Quantum Monte Carlo (quantummontecarlo.qiotoolkit) on the device against
the oracle.

Each restart holds `trotter_number` imaginary-time slices; the walkers are
the slices (slot r * trotter + k) and a slice's lowest is its restart's.
Bar: bit-exact per slice (cost, lowest, difference evaluations, flips,
states, lowest states) and the best, with no acceptance decided within
1e-15 of the device exp() (near_ties == 0).
"""
import numpy as np
import pytest

import qiotoolkit_gb300 as q
from qiotoolkit_gb300 import instances as I
from oracle import oracle as O

pytestmark = pytest.mark.gpu

QMC = "quantummontecarlo.qiotoolkit"

MODELS = {
    "ising_real": ("ising", lambda: I.er_ising(300, 900, seed=11)),
    "ising_int": ("ising", lambda: I.cubic_pm_j(6, seed=12)),
    "ising_plain": ("ising_plain", lambda: I.er_ising(200, 600, seed=13)),
    "pubo_real": ("pubo", lambda: I.random_pubo(400, 1600, seed=14)),
    "pubo_int": ("pubo", lambda: I.random_pubo(300, 1200, seed=15, integer=True)),
    "pubo_plain": ("pubo_plain", lambda: I.random_pubo(200, 700, seed=16)),
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
    assert s.stats().near_ties == 0


def run_both(kind, gen, mode, restarts, trotter, sweeps=30, seed=7):
    off, ids, coef = gen()
    g = q.Model(kind, off=off, ids=ids, coef=coef)
    o = O.Model(kind, off=off, ids=ids, coef=coef)
    params = {"seed": seed, "sweeps": sweeps, "restarts": restarts, "trotter_number": trotter,
              "beta_start": 0.5, "beta_stop": 3.0, "transverse_field_low": 0.2,
              "transverse_field_high": 2.0, "rng_mode": mode}
    s = q.Solver(g, QMC, {"params": params}).init().run()
    r = O.run(o, "qmc", seed=seed, step_limit=sweeps, restarts=restarts, trotter_number=trotter,
              sched=("linear", 0.5, 3.0), sched2=("linear", 0.2, 2.0), rng_mode=mode)
    return s, r


@pytest.mark.parametrize("name", list(MODELS))
@pytest.mark.parametrize("mode", ["replay", "counter"])
def test_qmc_slices(name, mode):
    kind, gen = MODELS[name]
    s, r = run_both(kind, gen, mode, restarts=5, trotter=12)
    same(s, r)


@pytest.mark.parametrize("trotter", [2, 33, 70])
def test_qmc_trotter_numbers(trotter):
    """Slices beyond one warp's lanes (lane k % 32 serves slice k)."""
    s, r = run_both("ising", lambda: I.er_ising(120, 360, seed=3), "replay", restarts=3,
                    trotter=trotter, sweeps=20)
    same(s, r)


def test_qmc_result_document():
    off, ids, coef = I.er_ising(100, 300, seed=2)
    g = q.Model("ising", off=off, ids=ids, coef=coef)
    s = q.Solver(g, QMC, {"params": {"seed": 4, "sweeps": 20, "restarts": 4, "trotter_number": 8,
                                     "number_of_solutions": 3}}).init().run()
    doc = s.result()
    par = doc["solutions"]["parameters"]
    assert par["trotter_number"] == 8 and par["restarts"] == 4
    sols = doc["solutions"]["solutions"]
    assert len(sols) == 3  # one candidate per restart, not per slice
    assert [x["cost"] for x in sols] == sorted(x["cost"] for x in sols)


def test_qmc_pieces():
    off, ids, coef = I.random_pubo(150, 500, seed=6)
    g = q.Model("pubo", off=off, ids=ids, coef=coef)
    p = {"seed": 9, "sweeps": 30, "restarts": 3, "trotter_number": 6}
    s = q.Solver(g, QMC, {"params": p}).init().run()
    srv = q.Server(max_active=4, sa_sweeps_per_piece=7)
    try:
        res = srv.wait(srv.submit(g, QMC, {"params": p}))
    finally:
        srv.close()
    assert res["solutions"] == s.result()["solutions"]


@pytest.mark.parametrize("trotter", [12, 70])
def test_qmc_level_kernel_counter_streams(trotter):
    """Counter streams run the level-parallel kernel (variables of one level
    at once, costs summed per slice in variable order after each sweep): the
    same slices as the oracle and as the one-warp-per-restart kernel."""
    off, ids, coef = I.er_ising(150, 450, seed=31)
    g = q.Model("ising", off=off, ids=ids, coef=coef)
    o = O.Model("ising", off=off, ids=ids, coef=coef)
    params = {"seed": 13, "sweeps": 25, "restarts": 4, "trotter_number": trotter,
              "beta_start": 0.5, "beta_stop": 3.0, "transverse_field_low": 0.2,
              "transverse_field_high": 2.0, "rng_mode": "counter"}
    s = q.Solver(g, QMC, {"params": params}).init().run()
    assert s.stats().sweep_kernel == 7
    r = O.run(o, "qmc", seed=13, step_limit=25, restarts=4, trotter_number=trotter,
              sched=("linear", 0.5, 3.0), sched2=("linear", 0.2, 2.0), rng_mode="counter")
    same(s, r)
    w = q.Solver(g, QMC, {"params": dict(params, kernel="warp")}).init().run()
    assert w.stats().sweep_kernel == 6
    np.testing.assert_array_equal(w.replicas()["states"], s.replicas()["states"])
    np.testing.assert_array_equal(w.replicas()["cost"], s.replicas()["cost"])


@pytest.mark.parametrize("full", [False, True])
@pytest.mark.parametrize("mode", ["replay", "counter"])
def test_qmc_maxsat(full, mode):
    """MaxSat: the sweep visits get_sweep_size() variables (1 by default)."""
    off, ids, coef = I.weighted_maxsat(100, seed=18)
    g = q.Model("maxsat", off=off, ids=ids, coef=coef)
    o = O.Model("maxsat", off=off, ids=ids, coef=coef)
    params = {"seed": 3, "sweeps": 15, "restarts": 3, "trotter_number": 8, "beta_start": 0.5,
              "beta_stop": 3.0, "transverse_field_low": 0.2, "transverse_field_high": 2.0,
              "rng_mode": mode, "maxsat_full_sweep": full}
    s = q.Solver(g, QMC, {"params": params}).init().run()
    r = O.run(o, "qmc", seed=3, step_limit=15, restarts=3, trotter_number=8,
              sched=("linear", 0.5, 3.0), sched2=("linear", 0.2, 2.0), rng_mode=mode,
              full_maxsat_sweep=full)
    same(s, r)
