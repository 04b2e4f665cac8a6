"""The benchmark configurations at their full model sizes, on the GPU, against
the oracle (GPU required).

Bar: bit-exact under replayed PCG streams -- every walker's final cost,
lowest cost, attempt/accept counts and final/lowest states equal the
oracle's (== on FP64 costs).  The models are the configurations' own
instances; only the sweep counts are cut so that the oracle finishes in
seconds.  With independent (counter) streams the modes are compared by
distribution: two-sample KS on best energies, p > 0.01.
"""
import numpy as np
import pytest

import qiotoolkit_gb300 as q
from qiotoolkit_gb300 import instances as I
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SA = "simulatedannealing.qiotoolkit"
PT = "paralleltempering.qiotoolkit"
PA = "populationannealing.cpu"


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


@pytest.fixture(scope="module")
def er1000():
    """SA workload model: N=1000, 3000 ER couplings +-1, 1000 fields U[-0.5, 0.5]."""
    return both("ising", *I.er_ising(1000, 3000, seed=0))


@pytest.fixture(scope="module")
def pubo4096():
    """PT workload model: N=4096, 20000 terms of order 1-4, N(0,1) FP64."""
    return both("pubo", *I.random_pubo(4096, 20000, seed=1))


@pytest.mark.parametrize("kernel", ["auto", "warp", "lanes"])
def test_sa_er1000_64_restarts(er1000, kernel):
    g, o = er1000
    params = {"seed": 0, "sweeps": 60, "restarts": 64, "beta_start": 0.1, "beta_stop": 5.0,
              "kernel": kernel}
    s = q.Solver(g, SA, {"params": params}).init().run()
    r = O.run(o, "sa", seed=0, step_limit=60, restarts=64, sched=("linear", 0.1, 5.0), threads=8)
    assert_same_walkers(s.replicas(), r)
    assert s.best()[0] == r.best_cost


@pytest.mark.parametrize("mode", ["replay", "counter"])
def test_pt_pubo4096_32_temperatures(pubo4096, mode):
    g, o = pubo4096
    temps = {"type": "geometric", "initial": 0.05, "final": 3.0, "count": 32}
    params = {"seed": 0, "sweeps": 25, "restarts": 2, "temperatures": temps, "rng_mode": mode}
    s = q.Solver(g, PT, {"params": params}).init().run()
    assert s.stats().near_ties == 0
    rep = s.replicas()
    for k in range(2):  # restart k is the reference run seeded k
        r = O.run(o, "pt", seed=k, step_limit=25, use_inverse=False,
                  sched=("geometric", 0.05, 3.0), sched_count=32, rng_mode=mode, threads=8)
        sl = slice(32 * k, 32 * k + 32)
        assert_same_walkers({key: v[sl] for key, v in rep.items()}, r)


def test_pt_pubo4096_observables(pubo4096):
    g, o = pubo4096
    temps = {"type": "geometric", "initial": 0.05, "final": 3.0, "count": 32}
    s = q.Solver(g, PT, {"params": {"seed": 3, "sweeps": 20, "temperatures": temps}}).init().run()
    r = O.run(o, "pt", seed=3, step_limit=20, use_inverse=False,
              sched=("geometric", 0.05, 3.0), sched_count=32, threads=8)
    obs = s.pt_observables()
    np.testing.assert_array_equal(obs[:, :4], r.pt_obs[:, :4])
    np.testing.assert_array_equal(obs[:-1, 4], r.pt_obs[:-1, 4])


def test_sa_cubic_instance_sizes():
    """The batched workload's instance sizes (L = 4 .. 20) one by one."""
    for L in (4, 11, 20):
        g, o = both("ising", *I.cubic_pm_j(L, seed=1000 + L))
        params = {"seed": 0, "sweeps": 30, "restarts": 16, "beta_start": 0.1, "beta_stop": 3.0}
        s = q.Solver(g, SA, {"params": params}).init().run()
        r = O.run(o, "sa", seed=0, step_limit=30, restarts=16, sched=("linear", 0.1, 3.0),
                  threads=8)
        assert_same_walkers(s.replicas(), r)


def test_ks_counter_vs_replay_er1000(er1000):
    """Independent (counter) streams against the reference's PCG streams on
    the SA workload's model, 256 restarts of the full 1000-sweep schedule:
    the best-energy distributions agree (two-sample KS, p > 0.01)."""
    scipy_stats = pytest.importorskip("scipy.stats")
    g, o = er1000
    params = {"seed": 1, "sweeps": 1000, "restarts": 256, "beta_start": 0.1, "beta_stop": 5.0}
    sc = q.Solver(g, SA, {"params": dict(params, rng_mode="counter")}).init().run()
    sr = q.Solver(g, SA, {"params": params}).init().run()
    lc = sc.replicas(states=False)["lowest"]
    lr = sr.replicas(states=False)["lowest"]
    assert scipy_stats.ks_2samp(lc, lr).pvalue > 0.01
    # the replay run is the reference's own trajectory set
    r = O.run(o, "sa", seed=1, step_limit=1000, restarts=256, sched=("linear", 0.1, 5.0),
              threads=8)
    np.testing.assert_array_equal(lr, r.lowest)


def test_ks_pa_counter_vs_replay_streams():
    """Population annealing with the reference's Poisson resampling: counter
    (independent) walker streams against the reference's replayed PCG
    streams, 256 seeds on a 16x16 periodic +-J lattice (population 256):
    best and mean final energies agree by distribution (two-sample KS,
    p > 0.01).  The resampling draws stay on the master PCG stream in both."""
    scipy_stats = pytest.importorskip("scipy.stats")
    off, ids, coef = I.square_pm_j(16, seed=31)
    g = q.Model("ising", off=off, ids=ids, coef=coef)
    base = {"sweeps": 30, "population": 256, "beta_start": 0.0, "beta_stop": 1.5,
            "sweeps_per_replica": 2, "threads": 4}
    best = {"replay": [], "counter": []}
    mean = {"replay": [], "counter": []}
    for seed in range(256):
        for mode in ("replay", "counter"):
            s = q.Solver(g, PA, {"params": dict(base, seed=seed, rng_mode=mode)}).init().run()
            rep = s.replicas(states=False)
            best[mode].append(float(np.min(rep["lowest"])))
            mean[mode].append(float(np.mean(rep["cost"])))
    assert scipy_stats.ks_2samp(best["replay"], best["counter"]).pvalue > 0.01
    assert scipy_stats.ks_2samp(mean["replay"], mean["counter"]).pvalue > 0.01


def _exact_mean_energy(off, ids, coef, beta):
    """<E> at beta by enumerating every state of a small model."""
    n = int(ids.max()) + 1
    states = 1 - 2 * ((np.arange(1 << n)[:, None] >> np.arange(n)) & 1)
    e = np.zeros(1 << n)
    for t in range(len(coef)):
        e += coef[t] * np.prod(states[:, ids[off[t]:off[t + 1]]], axis=1)
    w = np.exp(-beta * (e - e.min()))
    return float((w * e).sum() / w.sum())


@pytest.mark.parametrize("mode", ["poisson", "residual", "multinomial"])
def test_pa_resampling_samples_boltzmann(mode):
    """Every resampling scheme -- the reference's Poisson (default) and
    residual (constant_population) schemes and the device multinomial
    option -- leaves a population whose mean energy at beta_stop is the
    exact Boltzmann average of a 4x4 periodic +-J lattice (2^16 states
    enumerated): 64 seeds, |mean - exact| < 4.5 standard errors.  Restarts
    are switched off (alpha near 1): the reference's restart rule re-starts
    Poisson populations whose families died out, which the schemes do at
    different rates (their family-size variances differ), so short anneals
    with restarts differ by distribution even between the reference's own
    two schemes."""
    off, ids, coef = I.square_pm_j(4, seed=31)
    g = q.Model("ising", off=off, ids=ids, coef=coef)
    beta = 0.6
    exact = _exact_mean_energy(off, ids, coef, beta)
    extra = {"poisson": {}, "residual": {"constant_population": True},
             "multinomial": {"rng_mode": "counter", "resampling": "multinomial"}}[mode]
    means = []
    for seed in range(64):
        p = dict(seed=seed, sweeps=100, population=512, beta_start=0.0, beta_stop=beta,
                 sweeps_per_replica=4, threads=4, alpha=1.0001, **extra)
        s = q.Solver(g, PA, {"params": p}).init().run()
        means.append(float(np.mean(s.replicas(states=False)["cost"])))
    mu = np.mean(means)
    se = np.std(means, ddof=1) / np.sqrt(len(means))
    assert abs(mu - exact) < 4.5 * se + 1e-9, (mu, exact, se)
