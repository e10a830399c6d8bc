"""KONECT converter parity with the reference's data/gen_bi.cpp: the same
graph (ids by first appearance, repeated pairs once) as the reference's own
converter writes, on committed fixtures (tests/golden/make_konect.py) and,
where the reference converter is built (oracle/_ref/gen_bi), on fresh
random inputs."""
import json
import os
import subprocess

import numpy as np
import pytest

import cumbe_gb300 as cm

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
KON = os.path.join(HERE, "golden", "konect")
REF_GEN = os.path.join(ROOT, "oracle", "_ref", "gen_bi")
GEN = os.path.join(ROOT, "cumbe_gb300", "gen_bi")
CASES = json.load(open(os.path.join(KON, "cases.json")))


def _same_graph(a, b):
    ia, ib = a.info(), b.info()
    assert (ia["n_rows"], ia["n_cols"], ia["n_edges"]) == (ib["n_rows"], ib["n_cols"], ib["n_edges"])
    assert all(np.array_equal(x, y) for x, y in zip(a.csr()[2:], b.csr()[2:]))


@pytest.mark.parametrize("name", sorted(CASES))
def test_loader_matches_reference_converter(built, name):
    c = CASES[name]
    ours = cm.Graph.load_konect(os.path.join(KON, c["input"]), c["skip_words"], c["skip_words_per_edge"])
    ref = cm.Graph.load_bi(os.path.join(KON, c["reference_bi"]))
    _same_graph(ours, ref)


@pytest.mark.parametrize("name", sorted(CASES))
def test_gen_bi_program_matches_reference_converter(built, tmp_path, name):
    c = CASES[name]
    out = tmp_path / "g.bi"
    r = subprocess.run([GEN, os.path.join(KON, c["input"]), str(out), str(c["skip_words"]),
                        str(c["skip_words_per_edge"])], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "Loading... Done" in r.stdout and "Writing... Done" in r.stdout
    ref_text = open(os.path.join(KON, c["reference_bi"])).read().split("\n")
    assert out.read_text().split("\n")[0] == ref_text[0]  # "R L E" header line
    _same_graph(cm.Graph.load_bi(str(out)), cm.Graph.load_bi(os.path.join(KON, c["reference_bi"])))


def test_gen_bi_prompts_for_missing_counts(built, tmp_path):
    c = CASES["unweighted"]
    out = tmp_path / "g.bi"
    r = subprocess.run([GEN, os.path.join(KON, c["input"]), str(out)], input="7\n0\n", capture_output=True, text=True)
    assert r.returncode == 0 and "Number of passed words: " in r.stdout
    _same_graph(cm.Graph.load_bi(str(out)), cm.Graph.load_bi(os.path.join(KON, c["reference_bi"])))
    r = subprocess.run([GEN, "x"], capture_output=True, text=True)
    assert r.stdout.strip() == "Wrong Dataset :("


@pytest.mark.skipif(not os.path.exists(REF_GEN), reason="reference converter not built here")
def test_random_inputs_against_live_reference_converter(built, tmp_path):
    rng = np.random.default_rng(77)
    for trial in range(6):
        n = int(rng.integers(1, 3000))
        s = rng.integers(-50, 400, n)
        d = rng.integers(0, 700, n)
        extra = int(rng.integers(0, 3))
        rows = [" ".join([str(a), str(b)] + ["1"] * extra) for a, b in zip(s.tolist(), d.tolist())]
        text = "% bip\n% x y z\n" + "\n".join(rows) + ("\n" if trial % 2 else "")
        src = tmp_path / f"in{trial}.tsv"
        src.write_text(text)
        ref_out = tmp_path / f"ref{trial}.bi"
        subprocess.run([REF_GEN, str(src), str(ref_out), "5", str(extra)], check=True, capture_output=True)
        ours = cm.Graph.load_konect(str(src), 5, extra)
        _same_graph(ours, cm.Graph.load_bi(str(ref_out)))
