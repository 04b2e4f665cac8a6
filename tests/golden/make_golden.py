"""Generate the golden fixtures in tests/golden/ from the reference's own tests.

Run where a QIOToolkit checkout is readable, giving its root directory as the
first argument or in QIO_REFERENCE.  Tests never run this script; they use
the committed JSON files.

Sources (paths relative to the reference's cpp/ or data/ directory):
  rng_pins.json      utils/test/random_generator_test.cc:18-79
  pt_toy_pin.json    solver/test/parallel_tempering_test.cc:113-190
  model_pins.json    model/test/ising_term_cached_test.cc:24-102,
                     model/test/ising_test.cc:119-160,326-360,619-662,
                     model/test/pubo_with_counter_test.cc:59-100,206-244,
                     model/test/max_sat_test.cc:22-80
  solver_pins.json   solver/test/simulated_annealing_test.cc:194-260,
                     solver/test/parallel_tempering_test.cc:239-281,
                     solver/test/population_annealing_test.cc:243-329,
                     solver/test/tabu_test.cc:98-184,
                     solver/test/substochastic_monte_carlo_test.cc:104-176,
                     solver/test/quantum_monte_carlo_test.cc:86-148 (data/params_qmc.json),
                     solver/test/{tabu,sa,pt,pa,ssmc}_pf_test.cc:23-115 (data/pf5s.json),
                     with their data/ inputs and data/params1.json
  planted.json       data/input_e2e_pipeline/{wishart_planting_N_16_alpha_0.81,
                     combined_4_local_N_16}_qualitytest (instances + energies)
  dimacs_pins.json   utils/test/dimacs_test.cc (inputs and expected parses)
  estimator_pins.json  model/test/ising_test.cc, model/test/pubo_test.cc:
                     the estimate_min_cost_diff / estimate_max_cost_diff tests
                     (inline or fixture models, expected values)
  proto_pins.json    data/*_pb/*.pb (bytes as written by the reference's
                     protobuf serialiser) with the terms their writers put
                     in: utils/test/stream_test.h:145-168,
                     model/test/test_utils.h:11-55, graph/test/graph_test.cc:
                     28-48, and the assertions of utils/test/
                     stream_proto_test.cc (ProtoMessagesTest)

Expected values are parsed from the test sources where they are plain
literals (EXPECT_* and ElementsAre lines), so a change in the reference shows
up as a change in the fixtures.
"""
from __future__ import annotations

import json
import os
import re
import sys

REFERENCE = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("QIO_REFERENCE", "")
if not REFERENCE:
    sys.exit("usage: make_golden.py <QIOToolkit checkout> (or set QIO_REFERENCE)")
CPP = os.path.join(REFERENCE, "cpp")
DATA = os.path.join(REFERENCE, "data")
OUT = os.path.dirname(os.path.abspath(__file__))


def read(rel, base=CPP):
    with open(os.path.join(base, rel)) as f:
        return f.read()


def lines(rel, a, b, base=CPP):
    return read(rel, base).splitlines()[a - 1:b]


def terms_of(model_json):
    cf = model_json["cost_function"]
    return {"type": cf["type"], "terms": [[t["c"], list(t["ids"])] for t in cf["terms"]]}


def rng_pins():
    src = "\n".join(lines("utils/test/random_generator_test.cc", 18, 79))
    blocks = {}
    for name in ("Twister, DefaultSeed", "Twister, CustomSeed", "PCG, DefaultSeed",
                 "PCG, CustomSeed"):
        body = src.split("TEST(" + name + ")")[1].split("TEST(")[0]
        vals = [int(v) for v in re.findall(r"\*\s*100\),\s*(\d+)\)", body)]
        blocks[name] = vals[:3]
    forks = [list(map(int, m.split(","))) for m in
             re.findall(r"ElementsAre\(([\d,\s]+)\)", src)]
    return {
        "source": "utils/test/random_generator_test.cc:18-79",
        "twister_default": blocks["Twister, DefaultSeed"],
        "twister_42": blocks["Twister, CustomSeed"],
        "pcg_default": blocks["PCG, DefaultSeed"],
        "pcg_42": blocks["PCG, CustomSeed"],
        "pcg_42_fork": forks,  # master, fork1, fork2, fork3 (12 draws each)
    }


def pt_toy_pin():
    src = "\n".join(lines("solver/test/parallel_tempering_test.cc", 113, 190))
    rows = re.findall(r"\{\s*\"T\":\s*([\d.]+),\s*\"acc_rate\":\s*([\d.]+),\s*"
                      r"\"avg_cost\":\s*([\d.]+),\s*\"avg_dir\":\s*([\d.]+)"
                      r"(?:,\s*\"swap_rate\":\s*([\d.]+))?", src)
    obs = [[float(x) if x else None for x in r] for r in rows]
    return {"source": "solver/test/parallel_tempering_test.cc:113-190",
            "seed": 42, "step_limit": 200,
            "temperatures": {"type": "linear", "initial": 0.5, "final": 0.1, "count": 5},
            "observables": obs,  # per replica: T, acc_rate, avg_cost, avg_dir, swap_rate
            "format": "%f (std::to_string)"}


def ring10(c=1):
    return [[c, [i, (i + 1) % 10]] for i in range(10)]


def model_pins():
    pins = []
    # ring of 10 ferromagnetic couplings: costs 10 / -4 / 6 / 4 / 10
    # (ising_term_cached_test.cc:61-76, ising_test.cc:119-134) and Twister(188)
    # Metropolis minimum -10 (ising_term_cached_test.cc:78-102)
    pins.append({"name": "ising_ring10", "kind": "ising", "terms": ring10(),
                 "source": "model/test/ising_term_cached_test.cc:24-102",
                 "single_updates": {"cost0": 10, "diff0": -4, "cost1": 6, "diff1": 4,
                                    "cost2": 10},
                 "twister_min": {"seed": 188, "iters": 1000, "T": 0.5, "min": -10}})
    # PUBO ring: 10 / -2 / 8 / 2 / 10, Twister min 0
    # (pubo_with_counter_test.cc:59-100; the fixture is the same ring)
    src = read("model/test/pubo_with_counter_test.cc")
    m = re.search(r"R\"\((\{.*?\})\)\"", src, re.S)
    pubo_fixture = terms_of(json.loads(m.group(1)))
    pins.append({"name": "pubo_ring10", "kind": "pubo", "terms": pubo_fixture["terms"],
                 "source": "model/test/pubo_with_counter_test.cc:24-100",
                 "single_updates": {"cost0": 10, "diff0": -2, "cost1": 8, "diff1": 2,
                                    "cost2": 10},
                 "twister_min": {"seed": 188, "iters": 1000, "T": 0.5, "min": 0}})
    # constant terms (ising_test.cc:326-360, pubo_with_counter_test.cc:227-244)
    pins.append({"name": "ising_const", "kind": "ising",
                 "terms": [[100, []], [2, []]], "const_cost": 102,
                 "source": "model/test/ising_test.cc:326-343"})
    pins.append({"name": "pubo_const", "kind": "pubo",
                 "terms": [[1, []], [2, []]], "const_cost": 3,
                 "source": "model/test/pubo_with_counter_test.cc:227-244"})
    # duplicated ids in an Ising term throw (ising_test.cc:362)
    pins.append({"name": "ising_dup", "kind": "ising", "terms": [[1, [0, 0]]],
                 "throws": True, "source": "model/test/ising_test.cc:362-380"})
    # disordered ids / renumbering (pubo_with_counter_test.cc:206-225)
    pins.append({"name": "pubo_names", "kind": "pubo",
                 "terms": [[1, [0]], [2, [2, 100]]], "var_names": [0, 2, 100],
                 "source": "model/test/pubo_with_counter_test.cc:206-225"})
    # MaxSAT 1(!x) + 4(x||y) + 2(!y): costs 4/1/2/3 and diffs
    # (max_sat_test.cc:22-80)
    pins.append({"name": "maxsat_small", "kind": "maxsat",
                 "terms": [[1, [-1]], [4, [1, 2]], [2, [-2]]],
                 "source": "model/test/max_sat_test.cc:22-80",
                 "costs": {"00": 4, "10": 1, "01": 2, "11": 3},
                 "diffs": {"00": [1 - 4, 2 - 4], "01": [3 - 2, 4 - 2],
                           "10": [4 - 1, 3 - 1], "11": [2 - 3, 1 - 3]}})
    # all solvers on a 3-spin instance -> -2 (ising_test.cc:619-662)
    pins.append({"name": "ising_3spin", "kind": "ising",
                 "terms": [[-1, [0, 1]], [1, [2]]], "seed": 88, "min": -2.0,
                 "source": "model/test/ising_test.cc:619-662"})
    return pins


def solver_pins():
    params1 = json.loads(read("params1.json", DATA))["params"]
    cases = []
    specs = [
        # (solver, model kind, data file, expected cost, configuration pins, source)
        ("sa", "pubo", "cpupubojobstest.json", -12, {}, "solver/test/simulated_annealing_test.cc:194-202"),
        ("sa", "pubo", "puboempty.json", 2, {}, "solver/test/simulated_annealing_test.cc:204-212"),
        ("sa", "ising", "isingempty.json", 12, {}, "solver/test/simulated_annealing_test.cc:214-222"),
        ("sa", "pubo", "puboemptymixed.json", -104, {"1": 1, "12": 1}, "solver/test/simulated_annealing_test.cc:224-234"),
        ("sa", "ising", "isingemptymixed.json", -100, {"1": -1, "10": 1}, "solver/test/simulated_annealing_test.cc:250-260"),
        ("pt", "pubo", "puboempty.json", 2, {}, "solver/test/parallel_tempering_test.cc:239-247"),
        ("pt", "ising", "isingempty.json", 12, {}, "solver/test/parallel_tempering_test.cc:249-257"),
        ("pt", "pubo", "puboemptymixed.json", -104, {"1": 1, "12": 1}, "solver/test/parallel_tempering_test.cc:259-269"),
        ("pt", "ising", "isingemptymixed.json", -100, {"1": -1, "10": 1}, "solver/test/parallel_tempering_test.cc:271-281"),
        ("pa", "pubo", "cpupubojobstest.json", "<=-12", {}, "solver/test/population_annealing_test.cc:243-251"),
        ("pa", "ising", "ising1.json", -10, {}, "solver/test/population_annealing_test.cc:263-271"),
        ("pa", "pubo", "puboempty.json", 2, {}, "solver/test/population_annealing_test.cc:283-291"),
        ("pa", "ising", "isingempty.json", 12, {}, "solver/test/population_annealing_test.cc:293-301"),
        ("pa", "pubo", "puboemptymixed.json", -104, {"1": 1, "12": 1}, "solver/test/population_annealing_test.cc:303-315"),
        ("pa", "ising", "isingemptymixed.json", -100, {"1": -1, "10": 1}, "solver/test/population_annealing_test.cc:317-329"),
        ("tabu", "pubo", "cpupubojobstest.json", "<=-12", {}, "solver/test/tabu_test.cc:98-106"),
        ("tabu", "ising", "ising1.json", -10, {}, "solver/test/tabu_test.cc:118-126"),
        ("tabu", "pubo", "puboempty.json", 2, {}, "solver/test/tabu_test.cc:138-146"),
        ("tabu", "ising", "isingempty.json", 12, {}, "solver/test/tabu_test.cc:148-156"),
        ("tabu", "pubo", "puboemptymixed.json", -104, {"1": 1, "12": 1}, "solver/test/tabu_test.cc:158-170"),
        ("tabu", "ising", "isingemptymixed.json", -100, {"1": -1, "10": 1}, "solver/test/tabu_test.cc:172-184"),
        ("ssmc", "pubo", "cpupubojobstest.json", -12, {}, "solver/test/substochastic_monte_carlo_test.cc:104-112"),
        ("ssmc", "pubo", "puboempty.json", 2, {}, "solver/test/substochastic_monte_carlo_test.cc:114-122"),
        ("ssmc", "ising", "isingempty.json", 12, {}, "solver/test/substochastic_monte_carlo_test.cc:124-132"),
        ("ssmc", "ising", "ising1.json", -10, {}, "solver/test/substochastic_monte_carlo_test.cc:134-142"),
        ("ssmc", "pubo", "puboemptymixed.json", -104, {"1": 1, "12": 1}, "solver/test/substochastic_monte_carlo_test.cc:144-154"),
        ("ssmc", "ising", "isingemptymixed.json", -100, {"1": -1, "10": 1}, "solver/test/substochastic_monte_carlo_test.cc:166-176"),
        ("qmc", "pubo", "cpupubojobstest.json", -12, {}, "solver/test/quantum_monte_carlo_test.cc:86-94"),
        ("qmc", "pubo", "puboempty.json", 2, {}, "solver/test/quantum_monte_carlo_test.cc:96-104"),
        ("qmc", "ising", "isingempty.json", 12, {}, "solver/test/quantum_monte_carlo_test.cc:106-114"),
        ("qmc", "ising", "ising1.json", -10, {}, "solver/test/quantum_monte_carlo_test.cc:116-124"),
        ("qmc", "pubo", "puboemptymixed.json", -104, {"1": 1, "12": 1}, "solver/test/quantum_monte_carlo_test.cc:126-136"),
        ("qmc", "ising", "isingemptymixed.json", -100, {"1": -1, "10": 1}, "solver/test/quantum_monte_carlo_test.cc:138-148"),
        ("tabu_pf", "pubo", "cpupubojobstest.json", -12, {}, "solver/test/tabu_pf_test.cc:23-36"),
        ("tabu_pf", "pubo", "puboempty.json", 2, {}, "solver/test/tabu_pf_test.cc:38-51"),
        ("tabu_pf", "ising", "isingempty.json", 12, {}, "solver/test/tabu_pf_test.cc:53-66"),
        ("tabu_pf", "ising", "ising1.json", -10, {}, "solver/test/tabu_pf_test.cc:68-81"),
        ("tabu_pf", "pubo", "puboemptymixed.json", -104, {"1": 1, "12": 1}, "solver/test/tabu_pf_test.cc:83-98"),
        ("tabu_pf", "ising", "isingemptymixed.json", -100, {"1": -1, "10": 1}, "solver/test/tabu_pf_test.cc:100-115"),
        ("sa_pf", "pubo", "cpupubojobstest.json", -12, {}, "solver/test/sa_pf_test.cc:23-36"),
        ("sa_pf", "pubo", "puboempty.json", 2, {}, "solver/test/sa_pf_test.cc:38-51"),
        ("sa_pf", "ising", "isingempty.json", 12, {}, "solver/test/sa_pf_test.cc:53-66"),
        ("sa_pf", "ising", "ising1.json", -10, {}, "solver/test/sa_pf_test.cc:68-81"),
        ("sa_pf", "pubo", "puboemptymixed.json", -104, {"1": 1, "12": 1}, "solver/test/sa_pf_test.cc:83-98"),
        ("sa_pf", "ising", "isingemptymixed.json", -100, {"1": -1, "10": 1}, "solver/test/sa_pf_test.cc:100-115"),
        ("pt_pf", "pubo", "cpupubojobstest.json", -12, {}, "solver/test/pt_pf_test.cc:23-36"),
        ("pt_pf", "pubo", "puboempty.json", 2, {}, "solver/test/pt_pf_test.cc:38-51"),
        ("pt_pf", "ising", "isingempty.json", 12, {}, "solver/test/pt_pf_test.cc:53-66"),
        ("pt_pf", "ising", "ising1.json", -10, {}, "solver/test/pt_pf_test.cc:68-81"),
        ("pt_pf", "pubo", "puboemptymixed.json", -104, {"1": 1, "12": 1}, "solver/test/pt_pf_test.cc:83-98"),
        ("pt_pf", "ising", "isingemptymixed.json", -100, {"1": -1, "10": 1}, "solver/test/pt_pf_test.cc:100-115"),
        ("pa_pf", "pubo", "cpupubojobstest.json", -12, {}, "solver/test/pa_pf_test.cc:23-36"),
        ("pa_pf", "pubo", "puboempty.json", 2, {}, "solver/test/pa_pf_test.cc:38-51"),
        ("pa_pf", "ising", "isingempty.json", 12, {}, "solver/test/pa_pf_test.cc:53-66"),
        ("pa_pf", "ising", "ising1.json", -10, {}, "solver/test/pa_pf_test.cc:68-81"),
        ("pa_pf", "pubo", "puboemptymixed.json", -104, {"1": 1, "12": 1}, "solver/test/pa_pf_test.cc:83-98"),
        ("pa_pf", "ising", "isingemptymixed.json", -100, {"1": -1, "10": 1}, "solver/test/pa_pf_test.cc:100-115"),
        ("ssmc_pf", "pubo", "cpupubojobstest.json", -12, {}, "solver/test/ssmc_pf_test.cc:23-36"),
        ("ssmc_pf", "pubo", "puboempty.json", 2, {}, "solver/test/ssmc_pf_test.cc:38-51"),
        ("ssmc_pf", "ising", "isingempty.json", 12, {}, "solver/test/ssmc_pf_test.cc:53-65"),
        ("ssmc_pf", "ising", "ising1.json", -10, {}, "solver/test/ssmc_pf_test.cc:67-79"),
        ("ssmc_pf", "pubo", "puboemptymixed.json", -104, {"1": 1, "12": 1}, "solver/test/ssmc_pf_test.cc:81-96"),
        ("ssmc_pf", "ising", "isingemptymixed.json", -100, {"1": -1, "10": 1}, "solver/test/ssmc_pf_test.cc:98-112"),
    ]
    params_qmc = json.loads(read("params_qmc.json", DATA))["params"]
    params_pf = json.loads(read("pf5s.json", DATA))["params"]
    for solver, kind, fname, cost, conf, source in specs:
        model = terms_of(json.loads(read(fname, DATA)))
        assert model["type"] == kind
        cases.append({"solver": solver, "kind": kind, "file": fname,
                      "terms": model["terms"],
                      "params": {"qmc": params_qmc, "tabu_pf": params_pf, "sa_pf": params_pf,
                                 "pt_pf": params_pf, "pa_pf": params_pf,
                                 "ssmc_pf": params_pf}.get(solver, params1),
                      "expected_cost": cost, "configuration": conf, "source": source})
    return {"params_file": "data/params1.json", "cases": cases}


def planted():
    out = []
    for d in ("wishart_planting_N_16_alpha_0.81_qualitytest",
              "combined_4_local_N_16_qualitytest"):
        base = os.path.join(DATA, "input_e2e_pipeline", d)
        en = json.load(open(os.path.join(base, "energies.json")))
        for case in en["cases"]:
            model = terms_of(json.load(open(os.path.join(base, case["file"]))))
            out.append({"set": d, "file": case["file"], "kind": model["type"],
                        "terms": model["terms"], "energy": case["energy"]})
    return {"source": "data/input_e2e_pipeline/*/energies.json", "instances": out}


def dimacs_pins():
    """Each TEST(Dimacs, ...) block: the input text and the expected type,
    counts, variables, clauses (literals, weights) and top."""
    src = read("utils/test/dimacs_test.cc")
    cases = []
    for m in re.finditer(r'TEST\(Dimacs, (\w+)\)\s*\{(.*?)\n\}', src, re.S):
        name, body = m.group(1), m.group(2)
        t = re.search(r'read\(R"\((.*?)\)"\);', body, re.S)
        if not t:
            continue
        case = {"name": name, "text": t.group(1), "clauses": {}, "weights": {}}
        for e in re.finditer(r'EXPECT_EQ\((.*?), (.*?)\);', body):
            lhs, rhs = e.group(1).strip(), e.group(2).strip()
            if "get_type" in lhs:
                case["type"] = rhs.strip('"')
            elif "get_nvar" in lhs:
                case["nvar"] = int(rhs)
            elif "get_ncl" in lhs:
                case["ncl"] = int(rhs)
            elif "get_top" in lhs:
                case["top"] = float(rhs)
            elif "get_variables" in lhs:
                case["variables"] = [int(x) for x in re.findall(r'-?\d+', rhs)]
            else:
                c = re.match(r'clauses\[(\d+)\]\.(variables|weight)', lhs)
                if c and c.group(2) == "variables":
                    case["clauses"][c.group(1)] = [int(x) for x in re.findall(r'-?\d+', rhs)]
                elif c:
                    case["weights"][c.group(1)] = float(rhs)
        cases.append(case)
    return {"source": "utils/test/dimacs_test.cc", "cases": cases}


def proto_pins():
    """The protobuf problem folders shipped in data/, byte for byte, and the
    cost functions their writers serialised into them."""
    folders = {}
    for name in sorted(os.listdir(DATA)):
        d = os.path.join(DATA, name)
        if not (name.endswith("_pb") and os.path.isdir(d)):
            continue
        files, k = [], 0
        while os.path.exists(os.path.join(d, f"{name}_{k}.pb")):
            with open(os.path.join(d, f"{name}_{k}.pb"), "rb") as f:
                files.append(f.read().hex())
            k += 1
        folders[name] = files
    # writers (loops restated as term lists)
    stream = []  # stream_test.h:148-166: file p holds terms i = 0..p
    for p in range(4):
        stream += [[i + 2.5, [i, i + 1]] for i in range(p + 1)]
    ring = [[1.0, [i, 0 if i == 9 else i + 1]] for i in range(10)]  # test_utils.h:18-24
    ring2 = [[-9.5 if i == 9 else (-1.0 * (i + 1) if i % 2 == 0 else float(i + 1)),
              [i, 0 if i == 9 else i + 1]] for i in range(10)]  # test_utils.h:40-47
    square = [[1.0, [i, 0 if i == 3 else i + 1]] for i in range(4)]  # graph_test.cc:35-41
    body = read("utils/test/stream_proto_test.cc").split("TEST(Stream, ProtoMessagesTest)")[1]
    body = body.split("TEST(")[0]
    n_edges = int(re.search(r"edges\.size\(\), (\d+)\)", body).group(1))
    c0 = float(re.search(r"edges\[0\]\.c, ([-\d.]+)\)", body).group(1))
    nodes0 = [int(x) for x in re.search(r"edges\[0\]\.nodes, std::vector<int>\(\{(.*?)\}", body)
              .group(1).split(",")]
    return {"folders": folders,
            "expected": {
                "input_problem_pb": {"type": "ising", "version": "1.0", "terms": stream,
                                     "n_edges": n_edges, "c0": c0, "nodes0": nodes0},
                # the last writer of this folder in the reference's test order
                # is create_proto_test_problem(PUBO); proto3 leaves the type
                # (0) out of the bytes
                "models_input_problem_pb": {"type": "pubo", "version": "1.0", "terms": ring},
                "models_input_problem2_pb": {"type": "ising", "version": "1.0", "terms": ring2},
                "graph_input_problem_pb": {"type": "ising", "version": "1.0", "terms": square},
                "ex_input_problem_pb": {"type": "softspin", "version": "0.1"}}}


def estimator_pins():
    """Tests that call estimate_min_cost_diff / estimate_max_cost_diff: the
    model (inline JSON, or the test fixture's) and the expected values, with
    MIN_DELTA_DEFAULT taken from model/graph_model.h."""
    m = re.search(r"#define MIN_DELTA_DEFAULT ([0-9.]+)", read("model/graph_model.h"))
    delta = float(m.group(1))
    cases = []
    for rel in ("model/test/ising_test.cc", "model/test/pubo_test.cc"):
        src = read(rel)
        fixtures = {}
        for f in re.finditer(r"class (\w+) : public testing::Test(.*?)\n};", src, re.S):
            j = re.search(r'R"\((.*?)\)"', f.group(2), re.S)
            if j:
                fixtures[f.group(1)] = j.group(1)
        for t in re.finditer(r"TEST(_F)?\((\w+), (\w+)\)\s*\{(.*?)\n\}", src, re.S):
            fixture, suite, name, body = t.group(1), t.group(2), t.group(3), t.group(4)
            if "estimate_" not in body or "proto" in name:
                continue
            j = re.search(r'R"\((.*?)\)"', body, re.S)
            text = j.group(1) if j else fixtures.get(suite) if fixture else None
            if text is None:
                continue
            doc = json.loads(text)
            exp = {}
            for e in re.finditer(r"EXPECT_(?:DOUBLE_)?EQ\((.*?), (\w+)\);", body):
                var = e.group(2)
                call = re.search(r"double %s = \w+\.(estimate_\w+)\(\)" % var, body)
                if not call:
                    continue
                val = e.group(1).replace("MIN_DELTA_DEFAULT", repr(delta))
                exp[call.group(1)] = float(eval(val, {"__builtins__": {}}))
            if exp:
                cases.append({"source": f"{rel} {suite}.{name}", "model": terms_of(doc),
                              "expected": exp})
    return {"min_delta_default": delta, "cases": cases}


def main():
    if not os.path.isdir(CPP):
        print("reference not found at", REFERENCE, file=sys.stderr)
        sys.exit(1)
    files = {"rng_pins.json": rng_pins(), "pt_toy_pin.json": pt_toy_pin(),
             "model_pins.json": model_pins(), "solver_pins.json": solver_pins(),
             "planted.json": planted(), "dimacs_pins.json": dimacs_pins(),
             "proto_pins.json": proto_pins(), "estimator_pins.json": estimator_pins()}
    for name, obj in files.items():
        with open(os.path.join(OUT, name), "w") as f:
            json.dump(obj, f, separators=(",", ":"))
            f.write("\n")
        print("wrote", name)


if __name__ == "__main__":
    main()
