"""Protobuf problem folders (qio_model_create_proto_folder), host side.

Pinned by the folders the reference's own tests wrote (data/*_pb, bytes in
tests/golden/proto_pins.json) and the terms their writers serialised
(utils/test/stream_test.h:145-168, model/test/test_utils.h:11-55,
graph/test/graph_test.cc:28-48).  Error cases follow the reference reader
(utils/proto_reader.h:28-150) and its tests (utils/test/stream_proto_test.cc).
"""
import os
import struct

import pytest

import qiotoolkit_gb300 as q

TYPES = {"pubo": 0, "ising": 1, "maxsat": 2, "softspin": 3}


def _info(m):
    i = m.info
    return (i.kind, i.n_vars, i.n_terms, i.n_incidences, i.const_cost, tuple(m.var_names()))


def _write(tmp_path, name, files):
    d = tmp_path / name
    d.mkdir()
    for k, b in enumerate(files):
        (d / f"{name}_{k}.pb").write_bytes(b)
    return str(d)


# ---- a proto3 encoder for the Problem schema (utils/problem.proto) --------
def _varint(v):
    v &= (1 << 64) - 1
    out = bytearray()
    while True:
        b = v & 0x7F
        v >>= 7
        if v:
            out.append(b | 0x80)
        else:
            out.append(b)
            return bytes(out)


def _ld(field, payload):
    return _varint(field << 3 | 2) + _varint(len(payload)) + payload


def _term(c, ids, packed=True):
    b = _varint(1 << 3 | 1) + struct.pack("<d", c) if c != 0.0 else b""
    if packed:
        b += _ld(2, b"".join(_varint(i) for i in ids)) if ids else b""
    else:
        b += b"".join(_varint(2 << 3 | 0) + _varint(i) for i in ids)
    return b


def _problem(terms, type_=None, version=None, packed=True, extra=b""):
    cf = b""
    if type_:
        cf += _varint(1 << 3 | 0) + _varint(type_)
    if version:
        cf += _ld(2, version.encode())
    cf += b"".join(_ld(3, _term(c, ids, packed)) for c, ids in terms)
    return _ld(1, cf + extra)


def test_encoder_matches_reference_serialiser(golden):
    """The encoder writes the bytes the reference's serialiser wrote."""
    g = golden("proto_pins.json")
    for name, exp in g["expected"].items():
        if "terms" not in exp:
            continue
        files = [bytes.fromhex(h) for h in g["folders"][name]]
        if name == "input_problem_pb":
            mine, at = [], 0
            for p in range(4):
                first = p == 0
                mine.append(_problem(exp["terms"][at:at + p + 1], TYPES["ising"] if first else None,
                                     "1.0" if first else None))
                at += p + 1
        else:
            mine = [_problem(exp["terms"], TYPES[exp["type"]], exp["version"])]
        assert mine == files, name


def test_reference_folders(golden, tmp_path):
    g = golden("proto_pins.json")
    for name, exp in g["expected"].items():
        path = _write(tmp_path, name, [bytes.fromhex(h) for h in g["folders"][name]])
        if exp["type"] == "softspin":
            with pytest.raises(q.QioError, match="softspin"):
                q.Model.from_proto_folder(path)
            continue
        m = q.Model.from_proto_folder(path)
        ref = q.Model(exp["type"], [(c, ids) for c, ids in exp["terms"]])
        assert _info(m) == _info(ref), name
        if name == "input_problem_pb":  # stream_proto_test.cc ProtoMessagesTest
            assert m.n_terms == exp["n_edges"]
            assert exp["terms"][0] == [exp["c0"], exp["nodes0"]]


def test_trailing_slash_and_unpacked_ids(tmp_path):
    terms = [(1.5, [0, 3]), (-2.0, [3, 7]), (0.25, [7])]
    path = _write(tmp_path, "p_pb", [_problem(terms, TYPES["ising"], "1.1", packed=False)])
    m = q.Model.from_proto_folder(path + "/")
    assert _info(m) == _info(q.Model("ising", terms))


def test_unknown_fields_and_init_config_skipped(tmp_path):
    # init_config map entry (field 4) and a metadata Struct (field 2 of Problem)
    entry = _ld(1, b"7") + _varint(2 << 3) + _varint(1)
    extra = _ld(4, entry)
    terms = [(1.0, [0, 1]), (2.0, [1, 2, 5])]
    b = _problem(terms, TYPES["pubo"], "", extra=extra) + _ld(2, _ld(1, b""))
    m = q.Model.from_proto_folder(_write(tmp_path, "x_pb", [b]))
    assert _info(m) == _info(q.Model("pubo", terms))


def test_many_files_large(tmp_path):
    import numpy as np
    rng = np.random.default_rng(3)
    terms = [(float(rng.normal()), sorted({int(v) for v in rng.integers(0, 500, 2)}))
             for _ in range(3000)]
    terms = [(c, ids) for c, ids in terms if len(ids) == 2]
    chunks = [terms[i:i + 700] for i in range(0, len(terms), 700)]
    files = [_problem(ch, TYPES["ising"] if k == 0 else None, "1.0" if k == 0 else None)
             for k, ch in enumerate(chunks)]
    m = q.Model.from_proto_folder(_write(tmp_path, "big_pb", files))
    assert _info(m) == _info(q.Model("ising", terms))


def test_maxsat_without_terms_left_to_the_model(tmp_path):
    # the reader's "terms cannot be 0" rule covers ising and pubo only; an
    # empty maxsat problem is refused by the model, as from JSON
    with pytest.raises(q.QioError) as a:
        q.Model.from_proto_folder(_write(tmp_path, "s_pb", [_problem([], TYPES["maxsat"], "1.0")]))
    with pytest.raises(q.QioError) as b:
        q.Model.from_json({"cost_function": {"type": "maxsat", "version": "1.0", "terms": []}})
    assert str(a.value) == str(b.value)


@pytest.mark.parametrize("files,msg", [
    ([_problem([(1.0, [0, 1])], TYPES["ising"], "foo")], "Expected version to be 1.0 or 1.1. Provided: foo"),
    ([b""], "Invalid problem message. No cost function found"),
    ([_problem([], TYPES["ising"], "1.0")], "Problem terms cannot be 0. Please add problem terms"),
    ([_problem([], TYPES["pubo"], "1.0")], "Problem terms cannot be 0. Please add problem terms"),
    ([_problem([(1.0, [0, 1])], 7, "1.0")], "Expected type to be ising, pubo, maxsat or softspin"),
    ([_problem([(1.0, [0, 1])], TYPES["ising"], "1.0"), b""], "No cost function found"),
    ([_problem([(1.0, [0, 1])], TYPES["ising"], "1.0")[:-3]], "malformed"),
])
def test_errors(tmp_path, files, msg):
    path = _write(tmp_path, "e_pb", files)
    with pytest.raises(q.QioError, match=msg.replace(".", r"\.").replace("(", r"\(")):
        q.Model.from_proto_folder(path)


def test_missing_folder(tmp_path):
    path = os.path.join(str(tmp_path), "err_input_problem_pb")
    with pytest.raises(q.QioError, match="Could not open file: " + path + "/err_input_problem_pb_0.pb"):
        q.Model.from_proto_folder(path)
