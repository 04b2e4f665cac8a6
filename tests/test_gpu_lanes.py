"""Lane-per-walker sweep kernel (one walker per thread) against the oracle.

Ising models whose terms have one or two members run on the lane kernel when
asked for (params "kernel": "lanes") or when there are many walkers.  The bar
is the same as for the warp kernel: identical trajectories, costs compared
with ==, final and lowest states equal.
"""
import numpy as np
import pytest

import qiotoolkit_gb300 as q
from qiotoolkit_gb300 import instances as I
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SA = "simulatedannealing.qiotoolkit"

def _er_int(n, m, seed, big=300):
    """ER couplings with integer weights up to +-big (|c| > 127: the lane
    kernel's int2 records rather than the packed 32-bit ones)."""
    import numpy as np
    off, ids, _ = I.er_ising(n, m, seed=seed)
    rng = np.random.default_rng(seed)
    coef = rng.integers(-big, big + 1, len(off) - 1).astype(float)
    return off, ids, coef


MODELS = {
    "er_real": lambda: I.er_ising(300, 900, seed=21),
    "er_bigint": lambda: _er_int(200, 700, 25),
    "cubic_int": lambda: I.cubic_pm_j(6, seed=22),
    "square_int": lambda: I.square_pm_j(16, seed=23),
    "cubic_odd": lambda: I.cubic_pm_j(5, seed=24),
}


def _both(gen):
    off, ids, coef = gen()
    return (q.Model("ising", off=off, ids=ids, coef=coef),
            O.Model("ising", off=off, ids=ids, coef=coef))


def _same(g, o):
    np.testing.assert_array_equal(g["cost"], o.cost)
    np.testing.assert_array_equal(g["lowest"], o.lowest)
    np.testing.assert_array_equal(g["attempts"], o.attempts)
    np.testing.assert_array_equal(g["accepts"], o.accepts)
    np.testing.assert_array_equal(g["states"], o.states)
    np.testing.assert_array_equal(g["lowest_states"], o.lowest_states)


@pytest.mark.parametrize("name", list(MODELS))
@pytest.mark.parametrize("mode", ["replay", "counter"])
def test_lanes_sa_trajectories(name, mode):
    g, o = _both(MODELS[name])
    # 40 restarts: one full group of 32 lanes and a partial one
    params = {"seed": 77, "sweeps": 80, "restarts": 40, "beta_start": 0.05,
              "beta_stop": 2.5, "rng_mode": mode, "kernel": "lanes"}
    s = q.Solver(g, SA, {"params": params}).init().run()
    r = O.run(o, "sa", seed=77, step_limit=80, restarts=40, sched=("linear", 0.05, 2.5),
              rng_mode=mode, threads=4)
    _same(s.replicas(), r)
    c, _ = s.best()
    assert c == r.best_cost


@pytest.mark.parametrize("name", ["square_int", "er_real"])
def test_lanes_equal_warp_kernel(name):
    """Lane kernel with its spins in shared memory, in global memory, and the
    warp kernel: the same walkers."""
    g, _ = _both(MODELS[name])
    out = {}
    for tag, kern, smem in (("lanes_smem", "lanes", True), ("lanes_global", "lanes", False),
                            ("warp", "warp", True)):
        p = {"seed": 5, "sweeps": 50, "restarts": 70, "beta_start": 0.2, "beta_stop": 4.0,
             "kernel": kern, "smem_state": smem}
        out[tag] = q.Solver(g, SA, {"params": p}).init().run().replicas()
    for k in ("cost", "lowest", "attempts", "accepts", "states", "lowest_states"):
        np.testing.assert_array_equal(out["lanes_smem"][k], out["warp"][k])
        np.testing.assert_array_equal(out["lanes_global"][k], out["warp"][k])


def test_lanes_cost_limit_chunks():
    """Cost limit: one sweep per launch, the lane state carried across launches."""
    g, o = _both(MODELS["cubic_int"])
    params = {"seed": 9, "sweeps": 200, "restarts": 33, "beta_start": 0.5,
              "beta_stop": 3.0, "kernel": "lanes", "cost_limit": -300}
    s = q.Solver(g, SA, {"params": params}).init().run()
    r = O.run(o, "sa", seed=9, step_limit=200, restarts=33, sched=("linear", 0.5, 3.0),
              threads=4, cost_limit=-300)
    _same(s.replicas(), r)


def test_lanes_reject_higher_order_models():
    off, ids, coef = I.random_pubo(50, 100, seed=3)
    m = q.Model("ising", off=off, ids=ids, coef=coef)
    s = q.Solver(m, SA, {"params": {"seed": 1, "sweeps": 5, "restarts": 4, "kernel": "lanes"}})
    with pytest.raises(q.QioError, match="at most two members"):
        s.init()
