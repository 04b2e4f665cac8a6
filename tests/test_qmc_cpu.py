"""Quantum Monte Carlo, host side: parameter validation as
solver/quantum_monte_carlo.h:185-229."""
import pytest

import qiotoolkit_gb300 as q

QMC = "quantummontecarlo.qiotoolkit"


@pytest.mark.parametrize("params,msg", [
    ({"beta_stop": 0}, "beta_stop"),
    ({"beta_start": 2.0, "beta_stop": 1.0}, "beta_start"),
    ({"transverse_field_low": -1}, "transverse_field_low"),
    ({"transverse_field_low": 2, "transverse_field_high": 1}, "transverse_field_high"),
    ({"trotter_number": 1}, "trotter_number"),
    ({"restarts": 0}, "restarts"),
    ({"number_of_solutions": 3000000}, "number_of_solutions"),
])
def test_parameter_errors(params, msg):
    m = q.Model("ising", [(1.0, [0, 1]), (-2.0, [1, 2])])
    with pytest.raises(q.QioError, match=msg):
        q.Solver(m, QMC, {"params": dict({"seed": 1, "sweeps": 10}, **params)})


def test_maxsat_accepted():
    m = q.Model("maxsat", [(1.0, [1, 2]), (2.0, [-1, 3])])
    q.Solver(m, QMC, {"params": {"seed": 1, "sweeps": 5, "trotter_number": 4}}).close()


def test_restarts_capped_like_the_reference():
    """restarts = min(restarts, max(threads, 16))."""
    m = q.Model("ising", [(1.0, [0, 1]), (-2.0, [1, 2])])
    s = q.Solver(m, QMC, {"params": {"seed": 1, "sweeps": 10, "restarts": 100000,
                                     "threads": 2, "trotter_number": 4}})
    s.close()
