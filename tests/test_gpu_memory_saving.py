"""The runner's memory-saving retry (app/runner.cc:500-535): an init that runs
out of device memory is tried once more with the memory-saving models.

The device is made "full" by QIO_DEVICE_MEMORY_LIMIT, a cap on the bytes the
library's buffers hold, set between the footprint of a population with the
per-term cache (M bytes per walker, twice) and one without.  The solves run
in a child process so that no other test's buffers count against the cap.
"""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import json, sys
import qiotoolkit_gb300 as q
from qiotoolkit_gb300 import instances as I
off, ids, coef = I.random_pubo(2000, 20000, seed=71)
terms = [{"c": float(coef[k]), "ids": [int(x) for x in ids[off[k]:off[k + 1]]]} for k in range(len(coef))]
doc = {"cost_function": {"type": "pubo", "version": "1.0", "terms": terms}}
out = {}
for name, target, extra in [("pa", "populationannealing.cpu", {"population": 512, "threads": 4}),
                            ("ssmc", "substochasticmontecarlo.cpu", {"target_population": 512, "threads": 4})]:
    for feat in ([], [3]):
        p = dict({"seed": 3, "sweeps": 20}, **extra)
        if feat:
            p["enabled_features"] = feat
        try:
            r = q.run_json(doc, {"params": p}, target)
            out[name + str(feat)] = {"cost": r["solutions"]["cost"],
                                     "retry": r["benchmark"].get("memory_saving_retry", False)}
        except q.QioError as e:
            out[name + str(feat)] = {"error": e.status}
print(json.dumps(out))
"""


def _run(limit):
    env = dict(os.environ)
    if limit:
        env["QIO_DEVICE_MEMORY_LIMIT"] = str(limit)
    else:
        env.pop("QIO_DEVICE_MEMORY_LIMIT", None)
    r = subprocess.run([sys.executable, "-c", CHILD], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_out_of_memory_retries_with_memory_saving_models():
    free = _run(0)
    capped = _run(12 << 20)
    # without the cap nothing retries; memory saving gives the same solve
    assert not free["pa[]"]["retry"] and free["pa[]"]["cost"] == free["pa[3]"]["cost"]
    # with it the cached population does not fit: PA retries with the
    # counter-free model and returns the memory-saving solve
    assert capped["pa[]"]["retry"] is True
    assert capped["pa[]"]["cost"] == free["pa[3]"]["cost"]
    assert capped["pa[3]"]["cost"] == free["pa[3]"]["cost"] and not capped["pa[3]"]["retry"]
    # the SSMC targets keep their models (Runner::target_support_memory_saving):
    # no retry, the out-of-memory status stands
    assert capped["ssmc[]"] == {"error": 2}
