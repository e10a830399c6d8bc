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


def test_python_option_flags_and_variants_match_the_header():
    hdr = open(os.path.join(ROOT, "include", "mbe.h")).read()
    flags = {n: 1 << int(k) for n, k in re.findall(r"MBE_OPT_(\w+)\s*=\s*1u\s*<<\s*(\d+)", hdr)}
    assert flags, "no option flags parsed"
    for name, value in flags.items():
        assert getattr(cm, "OPT_" + name) == value, name
    variants = {n: int(v) for n, v in re.findall(r"MBE_(CUMBE|NORS|NOES|NOWS)\s*=\s*(\d+)", hdr)}
    assert {k.upper(): v for k, v in cm.VARIANTS.items()} == variants


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


def _big_bi(rng, nr, nc, ne):
    """A `.bi` text large enough for the threaded parser: unsorted rows with
    duplicates, rows stored out of order in the edge list."""
    lens = rng.multinomial(ne, np.ones(nr) / nr)
    starts = np.zeros(nr, np.int64)
    order = rng.permutation(nr)  # row blocks laid out in a shuffled order
    pos = 0
    for r in order:
        starts[r] = pos
        pos += lens[r]
    cols = rng.integers(0, nc, ne, dtype=np.int64)
    head = f"{nr} {nc} {ne}\n\n"
    table = "\n".join(f"{s} {l}" for s, l in zip(starts.tolist(), lens.tolist()))
    edges = "\n".join(f"{c} 1" for c in cols.tolist())
    return head + table + "\n\n" + edges, starts, lens, cols


def _expected_csr(nr, starts, lens, cols):
    rows = np.concatenate([np.full(l, r, np.int64) for r, l in enumerate(lens.tolist())]) if nr else np.zeros(0)
    vals = np.concatenate([cols[s:s + l] for s, l in zip(starts.tolist(), lens.tolist())])
    pairs = np.unique(rows * (1 << 32) + vals)
    r, c = pairs >> 32, pairs & 0xFFFFFFFF
    rp = np.zeros(nr + 1, np.uint64)
    np.add.at(rp, r + 1, 1)
    return np.cumsum(rp).astype(np.uint64), c.astype(np.uint32), len(vals) - len(pairs)


def test_threaded_parser_matches_definition(built, tmp_path):
    rng = np.random.default_rng(3)
    text, starts, lens, cols = _big_bi(rng, 150000, 40000, 1500000)
    assert len(text) > (12 << 20)  # above the threaded-parse threshold
    p = tmp_path / "big.bi"
    p.write_text(text)
    g = cm.Graph.load_bi(str(p))
    nr, nc, rp, ci = g.csr()
    erp, eci, dups = _expected_csr(150000, starts, lens, cols)
    assert np.array_equal(rp, erp) and np.array_equal(ci, eci)
    info = g.info()
    assert info["n_dup_dropped"] == dups
    assert info["max_row_deg"] == int(np.diff(erp).max())
    assert info["max_col_deg"] == int(np.bincount(eci, minlength=40000).max())


def test_threaded_parser_reports_the_first_bad_edge(built, tmp_path):
    rng = np.random.default_rng(4)
    text, starts, lens, cols = _big_bi(rng, 100000, 30000, 1200000)
    lines = text.split("\n")
    first_edge_line = 2 + 100000 + 1
    bad = lines.copy()
    bad[first_edge_line + 900000] = "12x 1"
    bad[first_edge_line + 1000000] = "99999999 1"
    p = tmp_path / "bad.bi"
    p.write_text("\n".join(bad))
    with pytest.raises(cm.MBEError, match="truncated edge list at edge 900000"):
        cm.Graph.load_bi(str(p))
    bad = lines.copy()
    bad[first_edge_line + 700000] = "30000 1"
    p.write_text("\n".join(bad))
    with pytest.raises(cm.MBEError, match="neighbour id out of range at edge 700000"):
        cm.Graph.load_bi(str(p))
    bad = lines.copy()
    bad[2 + 60000] = f"{1200000} 5"
    p.write_text("\n".join(bad))
    with pytest.raises(cm.MBEError, match="row 60000 range outside edge list"):
        cm.Graph.load_bi(str(p))


def test_binary_image_round_trip_and_corruption(built, tmp_path):
    g = cm.Graph.generate(3000, 1200, 20000, 2.1, 2.1, 0, 7)
    b = tmp_path / "g.mbeg"
    g.write_bin(str(b))
    h = cm.Graph.load_bin(str(b))
    assert g.info() == h.info()
    assert all(np.array_equal(x, y) for x, y in zip(g.csr()[2:], h.csr()[2:]))
    raw = bytearray(b.read_bytes())
    for off in (10, 60, len(raw) - 3):  # header, row offsets, column ids
        bad = bytearray(raw)
        bad[off] ^= 0x40
        q = tmp_path / "bad.mbeg"
        q.write_bytes(bytes(bad))
        with pytest.raises(cm.MBEError, match="FORMAT"):
            cm.Graph.load_bin(str(q))
    q.write_bytes(bytes(raw[:-4]))
    with pytest.raises(cm.MBEError, match="FORMAT"):
        cm.Graph.load_bin(str(q))
    with pytest.raises(cm.MBEError, match="FORMAT"):
        cm.Graph.load_bin(os.path.join(ROOT, "tests", "golden", "graphs", os.listdir(
            os.path.join(ROOT, "tests", "golden", "graphs"))[0]))


def test_cached_load_writes_then_reuses_the_image(built, tmp_path):
    g = cm.Graph.generate(2000, 1000, 10000, 2.1, 2.1, 0, 1)
    bi, cache = tmp_path / "g.bi", tmp_path / "g.mbeg"
    g.write_bi(str(bi))
    a = cm.Graph.load_cached(str(bi), str(cache))
    assert cache.exists()
    m0 = cache.stat().st_mtime_ns
    b = cm.Graph.load_cached(str(bi), str(cache))
    assert cache.stat().st_mtime_ns == m0  # reused, not rewritten
    assert all(np.array_equal(x, y) for x, y in zip(a.csr()[2:], b.csr()[2:]))
    assert all(np.array_equal(x, y) for x, y in zip(g.csr()[2:], b.csr()[2:]))
    cache.write_bytes(b"junk")  # a broken cache is replaced
    os.utime(cache, ns=(m0 + 10 ** 9, m0 + 10 ** 9))
    c = cm.Graph.load_cached(str(bi), str(cache))
    assert all(np.array_equal(x, y) for x, y in zip(g.csr()[2:], c.csr()[2:]))
    assert cm.Graph.load_bin(str(cache)).info()["n_edges"] == g.info()["n_edges"]
