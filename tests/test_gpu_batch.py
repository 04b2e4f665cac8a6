"""Batched solves (qio_batch_*): every instance equals its plain solve.

A batch runs many models with one target and params as one captured CUDA
graph; instance i's result JSON (best cost, configuration, solutions,
counters) must equal Solver(models[i], target, params)'s exactly.
"""
import numpy as np
import pytest

import qiotoolkit_gb300 as q
from qiotoolkit_gb300 import instances as I

pytestmark = pytest.mark.gpu

SA = "simulatedannealing.qiotoolkit"


def _strip(res):
    res = dict(res)
    b = dict(res["benchmark"])
    b.pop("gb300", None)
    res["benchmark"] = b
    return res


def _plain(model, params):
    return _strip(q.Solver(model, SA, {"params": params}).init().run().result())


def _lattices(seed0=100):
    out = []
    for i, L in enumerate([3, 5, 4, 6, 3, 7]):
        off, ids, coef = I.cubic_pm_j(L, seed=seed0 + i)
        out.append(q.Model("ising", off=off, ids=ids, coef=coef))
    return out


@pytest.mark.parametrize("mode", ["replay", "counter"])
def test_batch_lattices_equal_plain_solves(mode):
    models = _lattices()
    params = {"seed": 17, "sweeps": 60, "restarts": 16, "beta_start": 0.1, "beta_stop": 3.0,
              "rng_mode": mode, "number_of_solutions": 3}
    b = q.Batch(models, SA, {"params": params}).run()
    st = b.stats()
    assert st.kernel == 2 and st.graph == 1 and st.walkers == 16 * len(models)
    for i, m in enumerate(models):
        assert _strip(b.result(i)) == _plain(m, params)
    low = b.lowest()
    assert list(low) == [b.result(i)["solutions"]["cost"] for i in range(len(models))]


def test_batch_real_weights_and_reruns():
    models = []
    for i, n in enumerate([120, 300, 64, 200]):
        off, ids, coef = I.er_ising(n, 3 * n, seed=200 + i)
        models.append(q.Model("ising", off=off, ids=ids, coef=coef))
    params = {"seed": 3, "sweeps": 40, "restarts": 20, "beta_start": 0.2, "beta_stop": 2.0}
    b = q.Batch(models, SA, {"params": params})
    first = [_strip(b.run().result(i)) for i in range(len(models))]
    second = [_strip(b.run().result(i)) for i in range(len(models))]  # graph relaunch
    assert first == second
    for i, m in enumerate(models):
        assert first[i] == _plain(m, params)
    nog = q.Batch(models, SA, {"params": dict(params, graph=False, autotune=False)}).run()
    assert [_strip(nog.result(i)) for i in range(len(models))] == first


def _pubos(sizes, seed0=300, integer=False):
    out = []
    for i, n in enumerate(sizes):
        off, ids, coef = I.random_pubo(n, 3 * n, seed=seed0 + i, integer=integer)
        out.append(q.Model("pubo", off=off, ids=ids, coef=coef))
    return out


@pytest.mark.parametrize("mode", ["replay", "counter"])
def test_batch_pubo_one_queued_launch(mode):
    """PUBO instances of different sizes: the windowed kernel runs every
    walker from one persistent launch fed by a device queue (longest
    instance first); each instance equals its plain solve."""
    models = _pubos([80, 150, 40, 120, 33])
    params = {"seed": 8, "sweeps": 30, "restarts": 8, "beta_start": 0.1, "beta_stop": 2.0,
              "rng_mode": mode}
    b = q.Batch(models, SA, {"params": params}).run()
    st = b.stats()
    assert st.kernel == 1 and st.launches == len(models) + 1
    assert st.warps_per_block in (1, 2, 4, 8)
    for i, m in enumerate(models):
        assert _strip(b.result(i)) == _plain(m, params)


def test_batch_mixed_kinds_one_launch_per_kind():
    """FP64 PUBO, integer PUBO, many-body Ising and MaxSat in one batch: one
    queued launch per kind of model (flavour and coefficient kind: counter
    FP64 -- the PUBOs and MaxSat --, counter integer, parity FP64), results
    equal to the plain solves; reruns replay the captured graph."""
    models = _pubos([60, 90]) + _pubos([70, 50], seed0=320, integer=True)
    off, ids, coef = I.random_pubo(64, 200, seed=330)
    models.append(q.Model("ising", off=off, ids=ids, coef=coef))  # terms of up to four spins
    off, ids, coef = I.weighted_maxsat(40, seed=331)
    models.append(q.Model("maxsat", off=off, ids=ids, coef=coef))
    params = {"seed": 4, "sweeps": 25, "restarts": 6, "beta_start": 0.2, "beta_stop": 2.5,
              "maxsat_full_sweep": True}
    b = q.Batch(models, SA, {"params": params})
    first = [_strip(b.run().result(i)) for i in range(len(models))]
    assert b.stats().launches == len(models) + 3
    assert [_strip(b.run().result(i)) for i in range(len(models))] == first
    for i, m in enumerate(models):
        assert first[i] == _plain(m, params)


def test_batch_without_staged_state_launches_per_instance():
    models = _pubos([50, 70])
    params = {"seed": 2, "sweeps": 20, "restarts": 4, "smem_state": False}
    b = q.Batch(models, SA, {"params": params}).run()
    assert b.stats().launches == 2 * len(models)
    for i, m in enumerate(models):
        assert _strip(b.result(i)) == _plain(m, params)
