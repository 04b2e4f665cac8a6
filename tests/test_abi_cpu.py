"""The C-ABI library on a machine without a GPU: it loads, exports every
symbol include/qio_gb300.h declares, builds models (host-side
normalisation), validates params like the reference, and refuses to run
without a device (no CPU fallback)."""
import ctypes as C
import json
import os
import re

import numpy as np
import pytest

import qiotoolkit_gb300 as q
from qiotoolkit_gb300 import _lib
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    src = open(os.path.join(ROOT, "include", "qio_gb300.h")).read()
    return sorted(set(re.findall(r"\b(qio_[a-z_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    L = q.load()
    declared = header_symbols()
    assert declared, "no declarations found"
    for name in declared:
        assert hasattr(L, name), name
    assert sorted(q.SYMBOLS) == declared
    assert b"sm_103a" in L.qio_version()


def test_model_normalisation_matches_oracle(golden):
    pins = {p["name"]: p for p in golden("model_pins.json")}
    for name, kind in [("ising_ring10", "ising"), ("pubo_ring10", "pubo"),
                       ("pubo_names", "pubo"), ("maxsat_small", "maxsat"),
                       ("ising_const", "ising"), ("pubo_const", "pubo")]:
        terms = pins[name]["terms"]
        m = q.Model(kind, terms)
        o = O.Model(kind, terms)
        assert m.n_vars == o.n_vars and m.n_terms == o.n_terms
        assert m.const_cost == o.const_cost
        assert list(m.var_names()) == list(o.var_names())
    with pytest.raises(q.QioError, match="Duplicated ids detected in term!"):
        q.Model("ising", pins["ising_dup"]["terms"])


def test_random_model_normalisation_matches_oracle():
    from qiotoolkit_gb300 import instances as I
    for kind, (off, ids, coef) in [("pubo", I.random_pubo(300, 900, seed=5)),
                                   ("ising", I.er_ising(200, 500, seed=6)),
                                   ("maxsat", I.weighted_maxsat(150, seed=7))]:
        m = q.Model(kind, off=off, ids=ids, coef=coef)
        o = O.Model(kind, off=off, ids=ids, coef=coef)
        assert (m.n_vars, m.n_terms) == (o.n_vars, o.n_terms)
        assert list(m.var_names()) == list(o.var_names())
        assert m.info.scale_factor == o.scale_factor


def test_integer_weight_detection():
    assert q.Model("ising", [(1, [0, 1]), (-2, [1, 2])]).info.integer_weights == 1
    assert q.Model("ising", [(0.5, [0, 1]), (-2, [1, 2])]).info.integer_weights == 0


def test_model_from_json_and_errors():
    doc = {"cost_function": {"type": "pubo", "version": "1.1",
                             "terms": [{"c": 1, "ids": [0]}, {"c": 2, "ids": [2, 100]}]}}
    m = q.Model.from_json(doc)
    assert list(m.var_names()) == [0, 2, 100]
    bad = {"cost_function": {"type": "pubo", "version": "-7", "terms": [{"c": 1, "ids": [0]}]}}
    with pytest.raises(q.QioError, match="Expecting `version` equals 1.0 or 1.1, but found: -7"):
        q.Model.from_json(bad)
    with pytest.raises(q.QioError, match="JSON parse error"):
        q.Model.from_json("{\"cost_function\": [}")
    with pytest.raises(q.QioError, match="size must be greater than 0"):
        q.Model.from_json({"cost_function": {"type": "ising", "terms": []}})


def test_params_validation_like_reference():
    m = q.Model("ising", [(1, [0, 1])])
    with pytest.raises(q.QioError, match="number_of_solutions"):
        q.Solver(m, "paralleltempering.qiotoolkit",
                 {"params": {"step_limit": 100, "seed": 42, "number_of_solutions": 3000000}})
    with pytest.raises(q.QioError, match="unable to initialize schedule"):
        q.Solver(m, "paralleltempering.qiotoolkit",
                 {"params": {"step_limit": 100, "temperatures": [], "seed": 42}})
    with pytest.raises(q.QioError, match="Unknown solver"):
        q.Solver(m, "substochasticmontecarlo.qiotoolkit", {"params": {}})
    with pytest.raises(q.QioError, match="number of sweeps must be greater than 1"):
        q.Solver(m, "simulatedannealing.qiotoolkit", {"params": {"step_limit": 1}})
    with pytest.raises(q.QioError, match="params"):
        q.Solver(m, "simulatedannealing.qiotoolkit", "{}")


def test_no_cpu_fallback_without_device():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    m = q.Model("ising", [(1, [0, 1])])
    s = q.Solver(m, "simulatedannealing.qiotoolkit", {"params": {"seed": 1, "sweeps": 10}})
    with pytest.raises(q.QioError) as e:
        s.init()
    assert e.value.status in (3, 5)
    with pytest.raises(q.QioError):
        m.calculate_cost(np.zeros(2, np.uint8))


def test_batch_configuration_errors():
    """Batch parameter checks run on the host (no device needed)."""
    from qiotoolkit_gb300 import instances as I
    off, ids, coef = I.random_pubo(30, 60, seed=1)
    pubo = q.Model("pubo", off=off, ids=ids, coef=coef)
    off, ids, coef = I.cubic_pm_j(3, seed=1)
    cube = q.Model("ising", off=off, ids=ids, coef=coef)
    sa = "simulatedannealing.qiotoolkit"
    with pytest.raises(q.QioError, match="batches run"):
        q.Batch([cube], "paralleltempering.qiotoolkit", {"params": {"sweeps": 5}})
    with pytest.raises(q.QioError, match="at most two members"):
        q.Batch([cube, pubo], sa, {"params": {"sweeps": 5, "kernel": "lanes"}})
    with pytest.raises(q.QioError, match="cost_limit"):
        q.Batch([cube], sa, {"params": {"sweeps": 5, "cost_limit": -3}})
    b = q.Batch([cube, pubo], sa, {"params": {"sweeps": 5, "restarts": 2}})
    with pytest.raises(q.QioError, match="run\\(\\) must be called"):
        b.result(0)


def test_kernel_parameter_validation():
    from qiotoolkit_gb300 import instances as I
    off, ids, coef = I.cubic_pm_j(3, seed=1)
    m = q.Model("ising", off=off, ids=ids, coef=coef)
    with pytest.raises(q.QioError, match='must be "auto", "warp", "lanes", "levels" or "fields"'):
        q.Solver(m, "simulatedannealing.qiotoolkit", {"params": {"sweeps": 5, "kernel": "fast"}})
    with pytest.raises(q.QioError, match="not available for parallel tempering"):
        q.Solver(m, "paralleltempering.qiotoolkit", {"params": {"sweeps": 5, "kernel": "lanes"}})
    with pytest.raises(q.QioError, match='needs "rng_mode": "counter"'):
        q.Solver(m, "populationannealing.cpu", {"params": {"sweeps": 5, "resampling": "multinomial"}})
    sa = "simulatedannealing.qiotoolkit"
    with pytest.raises(q.QioError, match='"levels" needs "rng_mode": "counter"'):
        q.Solver(m, sa, {"params": {"sweeps": 5, "kernel": "levels"}})
    with pytest.raises(q.QioError, match='"levels" is not available for parallel tempering'):
        q.Solver(m, "paralleltempering.qiotoolkit", {"params": {"sweeps": 5, "kernel": "levels"}})
    with pytest.raises(q.QioError, match='"levels" is not available for batches'):
        q.Batch([m], sa, {"params": {"sweeps": 5, "kernel": "levels", "rng_mode": "counter"}})
    off, ids, coef = I.er_ising(50, 120, seed=3)  # real couplings: no integer level schedule
    r = q.Model("ising", off=off, ids=ids, coef=coef)
    with pytest.raises(q.QioError, match='"levels" needs an Ising model with integer coefficients'):
        q.Solver(r, sa, {"params": {"sweeps": 5, "kernel": "levels", "rng_mode": "counter"}})
    pubo = q.Model("pubo", [(1.0, [0, 1, 2]), (2.0, [1, 3])])
    with pytest.raises(q.QioError, match='"levels" needs an Ising model'):
        q.Solver(pubo, "populationannealing.cpu",
                 {"params": {"sweeps": 5, "kernel": "levels", "rng_mode": "counter"}})
    # eligible: created without complaint (no device needed before init)
    q.Solver(m, sa, {"params": {"sweeps": 5, "kernel": "levels", "rng_mode": "counter"}}).close()


def test_graph_size_properties_pin():
    """graph/test/properties_test.cc:30-66: the graph::Size properties of the
    reference's seven-term graph (max / min / mean term order, sum of orders,
    sum of order * (order - 1), largest and smallest |coefficient|), which the
    benchmark block reports under the keys of utils/config.h."""
    terms = [(1, [0, 1]), (0.2, [0, 2]), (1, [0, 3]), (1, [1, 4]), (1, [2, 3, 4]), (1, [3]),
             (-10, [4, 5])]
    m = q.Model("pubo", terms)
    info = m.info
    assert info.n_terms == 7 and info.n_vars == 6
    assert info.max_locality == 3 and info.min_locality == 1
    assert info.avg_locality == 2.0
    assert info.accumulated_dependent_vars == 16
    assert info.sum_coefficient_degrees_total == 14
    assert info.max_coupling == 10.0 and info.min_coupling == 0.2
