"""The windowed kernel (`"kernel": "warp"`) on its edge cases, against the
oracle through the C ABI (GPU required).

Bar: bit-exact -- every walker's final and lowest cost (== on FP64),
attempt/accept counts and final/lowest states equal the oracle's.  The edge
models: rows of more than 32 incidences (recomputed exactly every round),
blocks with more incidences than a shared-memory tile (incidences read from
global memory), terms of five or six members, MaxSat's negated literals,
population annealing where a stream serves several walkers in turn, and a
run cut into one-sweep launches.
"""
import numpy as np
import pytest

import qiotoolkit_gb300 as q
from qiotoolkit_gb300 import instances as I
from oracle import oracle as O
from test_gpu_fields import dense_block_ising, hub_pubo

pytestmark = pytest.mark.gpu

SA = "simulatedannealing.qiotoolkit"
PT = "paralleltempering.qiotoolkit"
PA = "populationannealing.cpu"

MODELS = {
    "ising_real": ("ising", lambda: I.er_ising(300, 900, seed=11)),
    "ising_dense_block": ("ising", dense_block_ising),
    "pubo_real": ("pubo", lambda: I.random_pubo(400, 1600, seed=14)),
    "pubo_hub": ("pubo", hub_pubo),
    "maxsat_real": ("maxsat", lambda: I.weighted_maxsat(150, seed=17)),
}


def both(kind, off, ids, coef):
    return (q.Model(kind, off=off, ids=ids, coef=coef),
            O.Model(kind, off=off, ids=ids, coef=coef))


def assert_same_walkers(g, o):
    np.testing.assert_array_equal(g["cost"], o.cost)
    np.testing.assert_array_equal(g["lowest"], o.lowest)
    np.testing.assert_array_equal(g["attempts"], o.attempts)
    np.testing.assert_array_equal(g["accepts"], o.accepts)
    np.testing.assert_array_equal(g["states"], o.states)
    np.testing.assert_array_equal(g["lowest_states"], o.lowest_states)


@pytest.mark.parametrize("name", list(MODELS))
@pytest.mark.parametrize("mode", ["replay", "counter"])
def test_windowed_sa(name, mode):
    kind, gen = MODELS[name]
    g, o = both(kind, *gen())
    params = {"seed": 77, "sweeps": 40, "restarts": 12, "beta_start": 0.1, "beta_stop": 4.0,
              "rng_mode": mode, "maxsat_full_sweep": kind == "maxsat", "kernel": "warp"}
    s = q.Solver(g, SA, {"params": params}).init().run()
    assert s.stats().sweep_kernel == 1
    r = O.run(o, "sa", seed=77, step_limit=40, restarts=12, sched=("linear", 0.1, 4.0),
              rng_mode=mode, threads=4, full_maxsat_sweep=kind == "maxsat")
    assert_same_walkers(s.replicas(), r)
    assert s.best()[0] == r.best_cost


@pytest.mark.parametrize("name", ["ising_dense_block", "pubo_real", "pubo_hub", "maxsat_real"])
def test_windowed_pt(name):
    kind, gen = MODELS[name]
    g, o = both(kind, *gen())
    temps = {"type": "geometric", "initial": 0.05, "final": 3.0, "count": 8}
    params = {"seed": 42, "sweeps": 30, "temperatures": temps, "sweeps_per_replica": 2,
              "maxsat_full_sweep": True, "kernel": "warp"}
    s = q.Solver(g, PT, {"params": params}).init().run()
    r = O.run(o, "pt", seed=42, step_limit=30, use_inverse=False,
              sched=("geometric", 0.05, 3.0), sched_count=8, sweeps_per_replica=2,
              threads=4, full_maxsat_sweep=True)
    assert_same_walkers(s.replicas(), r)
    np.testing.assert_array_equal(s.pt_observables()[:, :4], r.pt_obs[:, :4])


def test_windowed_pa_streams_serve_several_walkers():
    """Population annealing on FP64 PUBO: 4 emulated streams serve 40
    walkers, so each warp runs ten walkers in turn."""
    g, o = both("pubo", *I.random_pubo(200, 800, seed=23))
    params = {"seed": 9, "sweeps": 20, "population": 40, "threads": 4, "beta_start": 0.0,
              "beta_stop": 2.0, "sweeps_per_replica": 2}
    s = q.Solver(g, PA, {"params": params}).init().run()
    r = O.run(o, "pa", seed=9, step_limit=20, population=40, pa_threads=4,
              sched=("linear", 0.0, 2.0), sweeps_per_replica=2)
    assert_same_walkers(s.replicas(), r)
    assert s.best()[0] == r.best_cost


def test_chunked_launches_keep_the_running_cost():
    """A cost limit cuts the sweeps into one-sweep launches: the running cost
    and the lowest carry over from one launch to the next."""
    g, o = both("pubo", *I.random_pubo(300, 1200, seed=61))
    params = {"seed": 9, "sweeps": 30, "restarts": 6, "beta_start": 0.1, "beta_stop": 3.0,
              "cost_limit": -1e9, "kernel": "warp"}
    s = q.Solver(g, SA, {"params": params}).init().run()
    r = O.run(o, "sa", seed=9, step_limit=30, restarts=6, sched=("linear", 0.1, 3.0), threads=4)
    assert_same_walkers(s.replicas(), r)
