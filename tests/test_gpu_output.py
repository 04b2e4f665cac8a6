"""The result JSON of a run (qio_run_json) against the reference's output
format (GPU required): the benchmark object carries Solver::get_benchmark's
keys (solver/solver.h:78-145, names from utils/config.h:24-47) and the
runner's (app/runner.cc:546-631), the extensions list holds counters, solver
and model, and MaxSat (not a graph model) reports -1 localities."""
import json

import pytest

import qiotoolkit_gb300 as q
from qiotoolkit_gb300 import instances as I

pytestmark = pytest.mark.gpu

SA = "simulatedannealing.qiotoolkit"

SOLVER_KEYS = {"cost_function_evaluation_count", "cost_difference_evaluation_count", "num_variables",
               "num_terms", "locality", "min_locality", "avg_locality", "accumulated_dependent_vars",
               "sum_coefficient_degrees_total", "max_coupling_magnitude", "min_coupling_magnitude",
               "extensions"}
RUNNER_KEYS = {"threads", "solver_time_ms", "cpu_time_ms", "max_mem_bytes", "disk_io_read_bytes",
               "disk_io_write_bytes", "end2end_time_ms", "end2end_cputime_ms", "preprocessing_time_ms",
               "postprocessing_time_ms"}


def _doc(kind, terms):
    return {"cost_function": {"type": kind, "version": "1.0",
                              "terms": [{"c": c, "ids": ids} for c, ids in terms]}}


def test_graph_model_benchmark_keys():
    terms = [(1, [0, 1]), (0.2, [0, 2]), (1, [0, 3]), (1, [1, 4]), (1, [2, 3, 4]), (1, [3]),
             (-10, [4, 5])]
    doc = _doc("pubo", terms)
    res = q.run_json(doc, {"params": {"seed": 1, "sweeps": 20, "restarts": 4}}, SA)
    b = res["benchmark"]
    assert SOLVER_KEYS | RUNNER_KEYS <= set(b)
    assert (b["num_variables"], b["num_terms"], b["locality"], b["min_locality"]) == (6, 7, 3, 1)
    assert b["avg_locality"] == 2.0
    assert (b["accumulated_dependent_vars"], b["sum_coefficient_degrees_total"]) == (16, 14)
    assert (b["max_coupling_magnitude"], b["min_coupling_magnitude"]) == (10.0, 0.2)
    names = [e["name"] for e in b["extensions"]]
    assert names[:3] == ["counters", "solver", "model"]
    counters = b["extensions"][0]["value"]
    assert counters["difference_evaluations"] == b["cost_difference_evaluation_count"] == 20 * 4 * 6
    size = b["extensions"][2]["value"]["graph"]["size"]
    assert (size["nodes"], size["edges"]) == (6, 7)
    assert b["disk_io_read_bytes"] == len(json.dumps(doc))
    assert b["solver_time_ms"] > 0 and b["end2end_time_ms"] >= b["solver_time_ms"]


def test_maxsat_benchmark_has_no_graph_properties():
    off, ids, coef = I.weighted_maxsat(40, seed=3)
    terms = [(float(coef[t]), [int(x) for x in ids[off[t]:off[t + 1]]]) for t in range(len(coef))]
    res = q.run_json(_doc("maxsat", terms), {"params": {"seed": 1, "sweeps": 20, "restarts": 4}}, SA)
    b = res["benchmark"]
    assert (b["locality"], b["min_locality"], b["avg_locality"]) == (-1, -1, -1)
    assert "num_variables" not in b
    assert RUNNER_KEYS <= set(b)
