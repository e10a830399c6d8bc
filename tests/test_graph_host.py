"""Host-side graph handling of libmbe (no GPU): .bi I/O, ingest, generator,
and the exported C ABI."""
import ctypes
import os
import re

import numpy as np
import pytest

import cumbe_gb300 as cm
import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol(built):
    hdr = open(os.path.join(ROOT, "include", "mbe.h")).read()
    declared = set(re.findall(r"MBE_API\s+[\w\s\*]+?\b(mbe_\w+)\s*\(", hdr))
    assert declared, "no declarations parsed"
    lib = ctypes.CDLL(cm.LIB_PATH)
    for name in sorted(declared):
        assert hasattr(lib, name), name
    assert declared == set(cm.SIGNATURES), declared ^ set(cm.SIGNATURES)


def test_bi_round_trip_and_normalisation(built, tmp_path):
    # unsorted rows with a duplicate, as data/gen_bi.cpp writes them
    text = "3 4 6\n\n0 3\n3 2\n5 1\n\n2 1\n0 1\n2 1\n3 1\n1 1\n0 1"
    p = tmp_path / "g.bi"
    p.write_text(text)
    g = cm.Graph.load_bi(str(p))
    info = g.info()
    assert info["n_rows"] == 3 and info["n_cols"] == 4 and info["n_edges"] == 5
    assert info["n_dup_dropped"] == 1
    nr, nc, rp, ci = g.csr()
    assert rp.tolist() == [0, 2, 4, 5]
    assert ci.tolist() == [0, 2, 1, 3, 0]
    q = tmp_path / "h.bi"
    g.write_bi(str(q))
    g2 = cm.Graph.load_bi(str(q))
    assert [a.tolist() for a in g2.csr()[2:]] == [rp.tolist(), ci.tolist()]


@pytest.mark.parametrize("text,err", [
    ("", "FORMAT"), ("2 2 1\n0 1\n", "FORMAT"), ("1 2 1\n0 1\n5 1", "FORMAT"),
    ("1 2 2\n0 3\n0 1\n1 1", "FORMAT"), ("1 -2 1\n0 1\n0 1", "FORMAT")])
def test_bad_bi_files_fail_cleanly(built, tmp_path, text, err):
    p = tmp_path / "bad.bi"
    p.write_text(text)
    with pytest.raises(cm.MBEError) as ei:
        cm.Graph.load_bi(str(p))
    assert err in str(ei.value)


def test_missing_file(built):
    with pytest.raises(cm.MBEError) as ei:
        cm.Graph.load_bi("/nonexistent/x.bi")
    assert "IO" in str(ei.value)


def test_generator_is_deterministic(built):
    a = cm.Graph.generate(2000, 1000, 10000, 2.1, 2.1, 0, 1).csr()
    b = cm.Graph.generate(2000, 1000, 10000, 2.1, 2.1, 0, 1).csr()
    c = cm.Graph.generate(2000, 1000, 10000, 2.1, 2.1, 0, 2).csr()
    assert all(np.array_equal(x, y) for x, y in zip(a[2:], b[2:]))
    assert not np.array_equal(a[3], c[3])
    assert a[3].size == 10000


def test_generator_cap_and_planted(built):
    g = cm.Graph.generate(5000, 2000, 20000, 2.0, 2.0, 50, 3, planted=5, planted_rows=6, planted_cols=8,
                          planted_density=1.0)
    i = g.info()
    # the cap binds the Chung-Lu draws; each planted block adds at most its width
    assert i["max_row_deg"] <= 50 + 5 * 8 and i["max_col_deg"] <= 50 + 5 * 6
    assert i["n_edges"] >= 20000


def test_library_hash_matches_oracle(built):
    rng = np.random.default_rng(1)
    for _ in range(50):
        r = rng.integers(0, 1 << 20, rng.integers(0, 9))
        c = rng.integers(0, 1 << 20, rng.integers(0, 9))
        assert cm.biclique_hash(r, c) == oracle.biclique_hash(r, c)


def test_no_device_raises(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(cm.MBEError) as ei:
        cm.Engine(0)
    assert "NO_DEVICE" in str(ei.value)
