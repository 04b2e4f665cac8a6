"""Substochastic Monte Carlo, host side: parameter validation as
solver/substochastic_monte_carlo.h:171-232 (messages as the reference's)."""
import pytest

import qiotoolkit_gb300 as q

SSMC = "substochasticmontecarlo.cpu"


@pytest.mark.parametrize("params,msg", [
    ({"target_population": 0}, "target_population"),
    ({"steps_per_walker": 0}, "steps_per_walker"),
    ({"alpha": {"type": "linear", "initial": 0.1, "final": 0.9}},
     "the schedule for alpha must be decreasing \\(i.e., alpha.initial > alpha.final\\). "
     "Found alpha.initial = 0.1 <= 0.9 = alpha.final."),
    ({"beta": {"type": "linear", "initial": 2.0, "final": 1.0}},
     "the schedule for beta must be increasing"),
    ({"alpha": {"type": "linear", "initial": 1, "final": 0, "start": 0, "stop": 10},
      "beta": {"type": "linear", "initial": 0, "final": 1, "start": 0, "stop": 20}},
     "The schedules for alpha and beta must have the same length"),
    ({"number_of_solutions": 3000000}, "number_of_solutions"),
])
def test_parameter_errors(params, msg):
    m = q.Model("ising", [(1.0, [0, 1]), (-2.0, [1, 2])])
    with pytest.raises(q.QioError, match=msg):
        q.Solver(m, SSMC, {"params": dict({"seed": 1, "step_limit": 100}, **params)})


def test_maxsat_configures():
    """MaxSat models are taken (their walkers draw one uniform() per
    variable at init); the params are validated on the host."""
    m = q.Model("maxsat", [(1.0, [1, 2]), (2.0, [-1, 3])])
    q.Solver(m, SSMC, {"params": {"seed": 1, "target_population": 8}}).close()
    with pytest.raises(q.QioError, match="target_population"):
        q.Solver(m, SSMC, {"params": {"seed": 1, "target_population": 0}})


def test_one_schedule_with_a_range_lends_it_to_the_other():
    m = q.Model("pubo", [(1.0, [0, 1]), (-2.0, [1, 2])])
    q.Solver(m, SSMC, {"params": {"seed": 1, "step_limit": 50,
                                  "beta": {"type": "linear", "initial": 0, "final": 3,
                                           "start": 0, "stop": 40}}}).close()
