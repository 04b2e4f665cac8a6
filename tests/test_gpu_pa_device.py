"""Population annealing with device-side multinomial resampling.

"resampling": "multinomial" (counter streams) keeps the whole resampling
step on the device: FP64 Boltzmann weights with the library's exp,
fixed-point prefix sums, parents from counter draws, exact replica copies and
the family census.  The oracle restates the same definition; walkers must
match exactly, with the warp kernel and with the lane kernel.
"""
import numpy as np
import pytest

import qiotoolkit_gb300 as q
from qiotoolkit_gb300 import instances as I
from oracle import oracle as O

pytestmark = pytest.mark.gpu

PA = "populationannealing.cpu"

MODELS = {
    "square_int": ("ising", lambda: I.square_pm_j(12, seed=41)),
    "er_real": ("ising", lambda: I.er_ising(150, 450, seed=42)),
    "pubo_real": ("pubo", lambda: I.random_pubo(120, 400, seed=43)),
}


def _same(g, o):
    np.testing.assert_array_equal(g["cost"], o.cost)
    np.testing.assert_array_equal(g["lowest"], o.lowest)
    np.testing.assert_array_equal(g["attempts"], o.attempts)
    np.testing.assert_array_equal(g["accepts"], o.accepts)
    np.testing.assert_array_equal(g["states"], o.states)
    np.testing.assert_array_equal(g["lowest_states"], o.lowest_states)


@pytest.mark.parametrize("name", list(MODELS))
@pytest.mark.parametrize("kernel", ["warp", "lanes"])
def test_pa_multinomial_matches_oracle(name, kernel):
    kind, gen = MODELS[name]
    if kernel == "lanes" and kind != "ising":
        pytest.skip("the lane kernel runs two-body Ising models")
    off, ids, coef = gen()
    g = q.Model(kind, off=off, ids=ids, coef=coef)
    o = O.Model(kind, off=off, ids=ids, coef=coef)
    params = {"seed": 21, "sweeps": 30, "population": 70, "beta_start": 0.0, "beta_stop": 2.5,
              "sweeps_per_replica": 3, "rng_mode": "counter", "resampling": "multinomial",
              "kernel": kernel}
    s = q.Solver(g, PA, {"params": params}).init().run()
    r = O.run(o, "pa", seed=21, step_limit=30, population=70, sched=("linear", 0.0, 2.5),
              sweeps_per_replica=3, rng_mode="counter", resampling="multinomial", threads=4)
    _same(s.replicas(), r)
    c, _ = s.best()
    assert c == r.best_cost


def test_pa_multinomial_restarts_match_oracle():
    """A low alpha threshold is never hit; a high one restarts often."""
    kind, gen = MODELS["square_int"]
    off, ids, coef = gen()
    g = q.Model(kind, off=off, ids=ids, coef=coef)
    o = O.Model(kind, off=off, ids=ids, coef=coef)
    params = {"seed": 4, "sweeps": 40, "population": 50, "beta_start": 0.0, "beta_stop": 4.0,
              "sweeps_per_replica": 1, "rng_mode": "counter", "resampling": "multinomial",
              "alpha": 40.0}
    s = q.Solver(g, PA, {"params": params}).init().run()
    r = O.run(o, "pa", seed=4, step_limit=40, population=50, sched=("linear", 0.0, 4.0),
              sweeps_per_replica=1, rng_mode="counter", resampling="multinomial", alpha=40.0,
              threads=4)
    _same(s.replicas(), r)
