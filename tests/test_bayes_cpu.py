"""The parameter-free solvers' Bayesian strategy (host code, no GPU) and the
configuration checks of the parameter-free PA and SSMC solvers."""
import numpy as np
import pytest

import qiotoolkit_gb300 as q


def quad(x):
    return (x[:, 0] - 3.0) ** 2 + 2.0 * (x[:, 1] + 1.0) ** 2


def test_strategy_finds_a_quadratic_minimum():
    rng = np.random.default_rng(0)
    ranges = [(-5.0, 5.0), (-4.0, 4.0)]
    xs = rng.uniform([-5, -4], [5, 4], (6, 2))
    ys = quad(xs)
    for it in range(20):
        p = q.bayes_recommend(ranges, xs, ys, seed=it, count=1)
        assert (p >= [-5, -4]).all() and (p <= [5, 4]).all()
        xs = np.vstack([xs, p])
        ys = np.append(ys, quad(p))
    assert ys.min() < 0.05


def test_strategy_is_deterministic_and_spreads_its_batch():
    rng = np.random.default_rng(1)
    d = 7
    ranges = [(0.0, 1.0)] * d
    xs = rng.uniform(0, 1, (40, d))
    ys = ((xs - 0.3) ** 2).sum(1)
    a = q.bayes_recommend(ranges, xs, ys, seed=3, count=4)
    b = q.bayes_recommend(ranges, xs, ys, seed=3, count=4)
    np.testing.assert_array_equal(a, b)
    assert ((a >= 0) & (a <= 1)).all()
    # the believer's points are not all the same point
    assert np.ptp(a, axis=0).max() > 1e-4
    # flat objectives still give points in the box
    c = q.bayes_recommend(ranges, xs, np.ones(40), seed=3, count=2)
    assert ((c >= 0) & (c <= 1)).all()


def test_strategy_argument_errors():
    with pytest.raises(q.QioError, match="two samples"):
        q.bayes_recommend([(0, 1)], [[0.5]], [1.0])
    with pytest.raises(q.QioError, match="lo <= hi"):
        q.bayes_recommend([(1, 0)], [[0.5], [0.2]], [1.0, 2.0])


@pytest.mark.parametrize("target", ["populationannealing-parameterfree.cpu",
                                    "substochasticmontecarlo-parameterfree.cpu"])
def test_parameter_free_configuration_errors(target):
    m = q.Model("ising", [(1.0, [0, 1]), (-2.0, [1, 2])])
    with pytest.raises(q.QioError, match="rng_mode"):
        q.Solver(m, target, {"params": {"seed": 1, "rng_mode": "sobol"}})
    q.Solver(m, target, {"params": {"seed": 1, "rng_mode": "counter"}}).close()
    with pytest.raises(q.QioError, match="nonimprovement_limit"):
        q.Solver(m, target, {"params": {"seed": 1, "nonimprovement_limit": 0}})
    with pytest.raises(q.QioError, match="max_step_divider"):
        q.Solver(m, target, {"params": {"seed": 1, "max_step_divider": 1.0}})
    with pytest.raises(q.QioError, match="max_steps"):
        q.Solver(m, target, {"params": {"seed": 1, "max_steps": 100}})
    with pytest.raises(q.QioError, match="reserved_population"):
        q.Solver(m, target, {"params": {"seed": 1, "reserved_population": 4}})
    with pytest.raises(q.QioError, match="larger than final"):
        rng = "alpha_range" if target.startswith("pop") else "steps_range"
        q.Solver(m, target, {"params": {"seed": 1, rng: {"initial": 3, "final": 2}}})
    q.Solver(m, target, {"params": {"seed": 1}}).close()


def test_pa_parameter_free_refusals():
    m = q.Model("ising", [(1.0, [0, 1]), (-2.0, [1, 2])])
    pf = "populationannealing-parameterfree.cpu"
    with pytest.raises(q.QioError, match="max_population_mult"):
        q.Solver(m, pf, {"params": {"seed": 1, "max_population_mult": 5}})
    with pytest.raises(q.QioError, match="linear_schedule"):
        q.Solver(m, pf, {"params": {"seed": 1, "resampling_strategy": "geometric_schedule"}})
    with pytest.raises(q.QioError, match="final_min_prob_log"):
        q.Solver(m, pf, {"params": {"seed": 1, "final_min_prob_log": 0.0}})
    ms = q.Model("maxsat", [(1.0, [1, -2]), (2.0, [2, 3])])
    with pytest.raises(q.QioError, match="Ising and PUBO"):
        q.Solver(ms, pf, {"params": {"seed": 1}})


def test_oracle_replay_initial_vectors():
    """The oracle's initial parameter vectors follow the adapters'
    get_initial_parameter_values (solver/pa_parameter_free.h:228-260,
    solver/ssmc_parameter_free.h:160-178), the jitter drawn from the seeded
    master stream before each run's forks."""
    from oracle import oracle as O
    terms = [(1.0, [0, 1]), (-2.0, [1, 2]), (0.5, [2, 3]), (1.5, [3, 0]), (0.25, [1])]
    off = np.cumsum([0] + [len(t) for _, t in terms])
    ids = np.array([i for _, t in terms for i in t], np.int32)
    coef = np.array([c for c, _ in terms])
    o = O.Model("ising", off=off, ids=ids, coef=coef)
    pa = O.pa_parameter_free_replay(o, "ising", terms, seed=5, threads=2, runs=[None] * 2)
    u0, st = O._pcg_draw(O._pcg_seed_state(5))
    assert pa[0][0] == [20.0, 2.0, 2.0 + 0.5 * (u0 - 0.5), 1.0, 2.0]
    assert pa[1][0][:2] == [30.0, 4.0] and pa[1][0][3:] == [2.0, 4.0]
    assert pa[0][1] == 20 and pa[1][1] == 15  # ceil(sweeps / sweeps_per_replica)
    ss = O.ssmc_parameter_free_replay(o, seed=5, threads=2, runs=[None] * 2, sweep_size=4)
    assert ss[0][0] == [80.0, 2.0, 1.0, 0.00001, 0.8, 0.00001, 5.0 + u0]
    assert ss[1][0][:2] == [160.0, 3.0]


def test_strategy_gradients_match_finite_differences(tmp_path):
    """The analytic gradients the strategy ascends (log marginal likelihood
    in the hyperparameters, expected improvement in the point) agree with
    central differences."""
    import os
    import shutil
    import subprocess
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = str(tmp_path / "grad")
    subprocess.run([cxx, "-std=c++17", "-O2", os.path.join(root, "tests", "integration", "bayes_gradients.cc"),
                    "-o", out], check=True, capture_output=True, text=True)
    r = subprocess.run([out], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    _, lml, _, ei = r.stdout.split()
    assert float(lml) < 1e-6 and float(ei) < 1e-6
