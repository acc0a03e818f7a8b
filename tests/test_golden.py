"""Golden fixtures (tests/golden/oracle_golden.json, written by tests/golden/make_golden.py).

CPU: the oracle still produces them. GPU: the engine, through the C ABI and through the
`procell` CLI, produces the same bits, and the CLI's text output matches byte for byte.
"""
import hashlib
import json
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = json.load(open(os.path.join(HERE, "golden", "oracle_golden.json")))


def test_oracle_philox_vectors(oracle_lib):
    for v in GOLDEN["philox"]:
        assert oracle_lib.philox(v["ctr"], v["key"]) == v["out"]


def test_oracle_normals_and_tables(oracle_lib):
    n = GOLDEN["normals"]
    z = oracle_lib.normals(n["seed"], n["root"], n["first_parent"], len(n["bits"]))
    assert [int(x) for x in z.view(np.uint32)] == n["bits"]
    k, w, f = oracle_lib.tables()
    h = hashlib.sha256()
    for a in (k, w.view(np.uint32), f.view(np.uint32)):
        h.update(np.ascontiguousarray(a).tobytes())
    assert h.hexdigest() == GOLDEN["tables_sha256"]


def _check(values, per_type, stats, case):
    nz = [i for i in range(len(values)) if int(per_type[i].sum())]
    assert [float(values[i]).hex() for i in nz] == case["values"]
    assert [[int(x) for x in per_type[i]] for i in nz] == case["per_type"]


@pytest.mark.parametrize("name", sorted(GOLDEN["cases"]))
def test_oracle_cases(oracle_lib, name):
    c = GOLDEN["cases"][name]
    i = c["input"]
    r = oracle_lib.simulate([tuple(b) for b in i["bins"]], [tuple(t) for t in i["types"]], i["t_max"],
                            i["phi"], seed=i["seed"])
    _check(r.values, r.per_type, r.stats, c)
    assert r.stats == c["stats"]
    assert oracle_lib.format_histogram(r, True) == c["text"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(GOLDEN["cases"]))
def test_engine_cases(engine, name):
    c = GOLDEN["cases"][name]
    i = c["input"]
    g = engine.simulate([tuple(b) for b in i["bins"]], [tuple(t) for t in i["types"]], i["t_max"],
                        i["phi"], i["seed"])
    _check(g.values, g.per_type, g.stats, c)
    for k in ("roots", "divisions", "leaves", "uncounted", "vanished"):
        assert g.stats[k] == c["stats"][k]


@pytest.mark.gpu
def test_engine_tables_match_golden(engine):
    k, w, f = engine.tables()
    h = hashlib.sha256()
    for a in (k, w.view(np.uint32), f.view(np.uint32)):
        h.update(np.ascontiguousarray(a).tobytes())
    assert h.hexdigest() == GOLDEN["tables_sha256"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(GOLDEN["cases"]))
def test_cli_text_output(engine, tmp_path, name):
    from procell import _lib
    import procell.configs as cfg
    c = GOLDEN["cases"][name]
    i = c["input"]
    cfg.write_histogram(str(tmp_path / "h.txt"), [tuple(b) for b in i["bins"]])
    cfg.write_types(str(tmp_path / "c.txt"), [tuple(t) for t in i["types"]])
    args = [_lib.CLI_PATH, "-h", str(tmp_path / "h.txt"), "-c", str(tmp_path / "c.txt"),
            "-t", repr(i["t_max"]), "-s", str(i["seed"]), "-r", "-o", str(tmp_path / "out.txt")]
    if i["phi"] is not None:
        args += ["-p", repr(i["phi"])]
    r = subprocess.run(args, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert (tmp_path / "out.txt").read_text() == c["text"]
    # without -o the histogram goes to stdout; without -r only value and total
    r = subprocess.run([a for a in args if a not in ("-r", "-o", str(tmp_path / "out.txt"))],
                       capture_output=True, text=True)
    assert r.returncode == 0
    want = "".join("\t".join(line.split("\t")[:2]) + "\n" for line in c["text"].splitlines())
    assert r.stdout == want
