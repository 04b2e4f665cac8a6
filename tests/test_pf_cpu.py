"""Parameter-free simulated annealing, host side.

The cost-difference estimates that place the temperature range are pinned
by the reference's own model tests (model/test/ising_test.cc,
model/test/pubo_test.cc; tests/golden/estimator_pins.json), for the library
and for the oracle's restatement.  Parameter errors follow
solver/sa_parameter_free.h and solver/parameter_free_solver.h.
"""
import pytest

import qiotoolkit_gb300 as q
from oracle import oracle as O

PF = "simulatedannealing-parameterfree.qiotoolkit"


def test_estimates_match_reference_tests(golden):
    for case in golden("estimator_pins.json")["cases"]:
        kind, terms = case["model"]["type"], case["model"]["terms"]
        got = dict(zip(("estimate_min_cost_diff", "estimate_max_cost_diff"),
                       q.Model(kind, [(c, ids) for c, ids in terms]).cost_diff_bounds()))
        ora = dict(zip(("estimate_min_cost_diff", "estimate_max_cost_diff"), O.cost_diff_bounds(kind, terms)))
        for k, v in case["expected"].items():
            assert got[k] == pytest.approx(v, abs=1e-12), case["source"]
            assert ora[k] == pytest.approx(v, abs=1e-12), case["source"]


def test_estimates_agree_on_random_models():
    import numpy as np
    from qiotoolkit_gb300 import instances as I
    for kind, (off, ids, coef) in (("ising", I.er_ising(80, 200, seed=3)),
                                   ("pubo", I.random_pubo(60, 150, seed=4))):
        terms = [(float(coef[k]), [int(x) for x in ids[off[k]:off[k + 1]]]) for k in range(len(coef))]
        lib = q.Model(kind, off=off, ids=ids, coef=coef).cost_diff_bounds()
        assert lib == O.cost_diff_bounds(kind, terms)


@pytest.mark.parametrize("params,msg", [
    ({"max_prob": 0}, "parameter `max_prob`: must be in \\(0, 1\\]"),
    ({"min_prob": 2}, "parameter `min_prob`: must be in \\(0, 1\\]"),
    ({"initial_sweeps_sample_points": [10, 20]}, "initial_sweeps_sample_points"),
    ({"min_num_restarts": 0}, "min_num_restarts"),
    ({"rng_mode": "counter"}, "rng_mode"),
    ({"number_of_solutions": 2}, "number_of_solutions"),
])
def test_parameter_errors(params, msg):
    m = q.Model("ising", [(1.0, [0, 1]), (-2.0, [1, 2])])
    with pytest.raises(q.QioError, match=msg):
        q.Solver(m, PF, {"params": dict({"seed": 1}, **params)})


def test_pt_parameter_errors():
    m = q.Model("ising", [(1.0, [0, 1]), (-2.0, [1, 2])])
    pt = "paralleltempering-parameterfree.qiotoolkit"
    with pytest.raises(q.QioError, match="min_num_betas"):
        q.Solver(m, pt, {"params": {"seed": 1, "min_num_betas": 0}})
    q.Solver(m, pt, {"params": {"seed": 1, "min_num_betas": 6}}).close()


def test_pt_betas_match_oracle():
    """the ladder of the parameter-free PT: geometric groups of 4, 9, 14, ...
    values, as the oracle restates them"""
    import json as _json
    m = q.Model("ising", [(1.0, [0, 1]), (-2.0, [1, 2]), (0.5, [2, 3])])
    s = q.Solver(m, "paralleltempering-parameterfree.qiotoolkit", {"params": {"seed": 1, "min_num_betas": 16}})
    mn, mx = O.cost_diff_bounds("ising", [(1.0, [0, 1]), (-2.0, [1, 2]), (0.5, [2, 3])])
    import math
    b0 = -math.log(0.5) / mx
    b1 = -math.log(0.0001) / (mn + 0.001 * (mx - mn))
    assert len(O._pf_betas(b0, b1, 16)) == 16
    s.close()


def test_maxsat_not_supported():
    m = q.Model("maxsat", [(1.0, [1, 2]), (2.0, [-1, 3])])
    with pytest.raises(q.QioError, match="maxsat"):
        q.Solver(m, PF, {"params": {"seed": 1}})
