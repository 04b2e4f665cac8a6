"""DIMACS cnf / wcnf input (qio_model_create_dimacs), host side.

Pinned by the reference's own parser tests (utils/test/dimacs_test.cc,
extracted to tests/golden/dimacs_pins.json): the model built from each text
equals the MaxSat model built from the expected clauses.  Error cases follow
the reference reader's rules (utils/dimacs.cc).
"""
import pytest

import qiotoolkit_gb300 as q


def _info(m):
    i = m.info
    return (i.kind, i.n_vars, i.n_terms, i.n_incidences, i.const_cost, tuple(m.var_names()))


def test_dimacs_reference_pins(golden):
    for case in golden("dimacs_pins.json")["cases"]:
        m = q.Model.from_dimacs(case["text"])
        n = case["ncl"]
        terms = [(case["weights"][str(k)], case["clauses"][str(k)]) for k in range(n)]
        ref = q.Model("maxsat", terms)
        assert _info(m) == _info(ref), case["name"]
        assert m.n_vars == case["nvar"]


@pytest.mark.parametrize("text,msg", [
    ("1 2 0\n", "Missing problem line"),
    ("p cnf 2 2\n1 2 0\n", "Number of clauses parsed does not match: 1!=2"),
    ("p cnf 3 1\n1 2 0\n", "Number of variables found does not match: 2!=3"),
    ("p cnf 2 1\n1 1 2 0\n", "Variable name 1 appears multiple times in clause."),
    ("p cnf 2 1\n1 -1 2 0\n", "Variable name 1 appears both positive and negative in clause."),
    ("p cnf 2 2\n1 2 0\n0\n", "List of variables in a clause cannot be empty"),
    ("p dnf 2 1\n1 2 0\n", "Expected `type` to be 'cnf' or 'wcnf'"),
    ("p cnf 2 1\np cnf 2 1\n1 2 0\n", "Multiple problem lines"),
    ("p cnf 2 1\n1 x 0\n", "Expected number on line 2"),
    ("p cnf 0 1\n1 0\n", "Expected positive number"),
])
def test_dimacs_errors(text, msg):
    with pytest.raises(q.QioError, match=msg.replace("(", r"\(").replace(")", r"\)")):
        q.Model.from_dimacs(text)


def test_dimacs_wcnf_weights_and_comments():
    text = "c a comment\nc\np wcnf 3 3 10\n2.5 1 -2 0\n10 3 0\nc between\n1 -1 2 -3 0\n"
    m = q.Model.from_dimacs(text)
    ref = q.Model("maxsat", [(2.5, [1, -2]), (10.0, [3]), (1.0, [-1, 2, -3])])
    assert _info(m) == _info(ref)
