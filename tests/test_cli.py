"""The `mbe` CLI keeps the reference's argv and output lines
(src/main.cu:9,121-141,207-234)."""
import json
import os
import re
import subprocess

import pytest

import cumbe_gb300 as cm

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


def test_usage_and_bad_file(built, tmp_path):
    r = subprocess.run([cm.CLI_PATH], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
    bad = tmp_path / "bad.bi"
    bad.write_text("2 2 5\n0 1\n")
    r = subprocess.run([cm.CLI_PATH, str(bad), "cuMBE"], capture_output=True, text=True)
    assert r.returncode == 1 and "loading the graph" in r.stderr and r.stdout == ""


@pytest.mark.gpu
@pytest.mark.parametrize("variant", ["cuMBE", "noRS", "noES", "noWS", "bogus"])
def test_cli_lines_and_result_file(built, tmp_path, variant):
    exp = json.load(open(os.path.join(GOLD, "expected.json")))["power_law_2k_1k"]
    path = os.path.join(GOLD, exp["file"])
    (tmp_path / "result").mkdir()
    r = subprocess.run([cm.CLI_PATH, path, variant], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.splitlines()
    algo = variant if variant != "bogus" else "cuMBE"  # unknown names fall back (src/main.cu:122)
    assert lines[0].startswith("date/time: ")
    assert lines[1] == f"algorithm: {algo}"
    assert lines[2] == "dataset: power_law_2k_1k.bi"
    assert lines[3] == "|R|: 1000, |L|: 2000, |E|: 10000"
    assert re.fullmatch(r"grid_size: \d+, block_size: \d+", lines[4])
    assert lines[5] == f"maximal bicliques: {exp['count']}"
    assert re.fullmatch(r"runtime \(s\): [0-9.e+-]+", lines[6])
    assert lines[7] == f"hash: {exp['hash']}"
    saved = (tmp_path / "result" / f"power_law_2k_1k_{algo}").read_text().splitlines()
    assert saved[1:6] == lines[1:6]


@pytest.mark.gpu
def test_cli_emit_file(built, tmp_path):
    """`--emit FILE` writes every maximal biclique once: rows | cols, ascending
    file ids; stdout keeps the reference's lines."""
    exp = json.load(open(os.path.join(GOLD, "expected.json")))["power_law_2k_1k"]
    path = os.path.join(GOLD, exp["file"])
    out = tmp_path / "bicliques.txt"
    r = subprocess.run([cm.CLI_PATH, path, "cuMBE", "--emit", str(out)], capture_output=True, text=True,
                       cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    assert r.stdout.splitlines()[5] == f"maximal bicliques: {exp['count']}"
    h, n = 0, 0
    seen = set()
    for line in out.read_text().splitlines():
        a, b = line.split(" | ")
        rows = [int(v) for v in a.split()]
        cols = [int(v) for v in b.split()]
        assert rows == sorted(rows) and cols == sorted(cols)
        seen.add((tuple(rows), tuple(cols)))
        h = (h + cm.biclique_hash(rows, cols)) & (2 ** 64 - 1)
        n += 1
    assert n == exp["count"] == len(seen)
    assert f"0x{h:016x}" == exp["hash"]


@pytest.mark.gpu
def test_cli_takes_a_binary_image(built, tmp_path):
    exp = json.load(open(os.path.join(GOLD, "expected.json")))["power_law_2k_1k"]
    img = tmp_path / "power_law_2k_1k.mbeg"
    cm.Graph.load_bi(os.path.join(GOLD, exp["file"])).write_bin(str(img))
    r = subprocess.run([cm.CLI_PATH, str(img)], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.splitlines()
    assert lines[5] == f"maximal bicliques: {exp['count']}"
    assert lines[7] == f"hash: {exp['hash']}"
