"""CPU oracle self-checks: the restatement of the reference's search agrees
with brute force from the definition, for every variant, list by list."""
import numpy as np
import pytest

import oracle
from conftest import random_csr

VARIANTS = ["cuMBE", "noRS", "noES", "noWS"]


@pytest.mark.parametrize("seed", range(4))
def test_restatement_matches_brute_force(built, seed):
    rng = np.random.default_rng(seed)
    for _ in range(150):
        nr, nc = int(rng.integers(1, 12)), int(rng.integers(1, 12))
        g = random_csr(rng, nr, nc, rng.uniform(0.05, 0.95))
        b = oracle.brute(*g, emit_cap=10000)
        for v in VARIANTS:
            r = oracle.ref_enumerate(*g, variant=v, emit_cap=10000)
            assert (r.count, r.hash) == (b.count, b.hash)
            assert r.bicliques == b.bicliques


def test_threads_do_not_change_results(built):
    rng = np.random.default_rng(7)
    g = random_csr(rng, 60, 40, 0.15)
    one = oracle.ref_enumerate(*g, threads=1)
    many = oracle.ref_enumerate(*g, threads=4)
    assert (one.count, one.hash) == (many.count, many.hash)


def test_thresholds_are_a_filter(built):
    rng = np.random.default_rng(3)
    for _ in range(40):
        g = random_csr(rng, 10, 9, 0.5)
        full = oracle.brute(*g, emit_cap=10000).bicliques
        for a, b in [(1, 1), (2, 1), (1, 3), (3, 3)]:
            t = oracle.ref_enumerate(*g, min_rows=a, min_cols=b, emit_cap=10000)
            want = [x for x in full if len(x[0]) >= a and len(x[1]) >= b]
            assert t.bicliques == want


def test_edge_cases(built):
    # empty graph, single edge, complete bipartite, isolated vertices, one side empty
    cases = [
        (3, 4, np.zeros(4, np.uint64), np.zeros(0, np.uint32), 0),
        (1, 1, np.array([0, 1], np.uint64), np.array([0], np.uint32), 1),
        (3, 5, np.array([0, 5, 10, 15], np.uint64), np.tile(np.arange(5, dtype=np.uint32), 3), 1),
        (4, 3, np.array([0, 1, 1, 2, 2], np.uint64), np.array([0, 2], np.uint32), 2),
        (0, 3, np.zeros(1, np.uint64), np.zeros(0, np.uint32), 0),
    ]
    for nr, nc, rp, ci, want in cases:
        for v in VARIANTS:
            assert oracle.ref_enumerate(nr, nc, rp, ci, variant=v).count == want
        if nr and nc:
            assert oracle.brute(nr, nc, rp, ci).count == want


def test_hash_is_order_free(built):
    h1 = oracle.biclique_hash([3, 1, 2], [9, 7])
    h2 = oracle.biclique_hash([1, 2, 3], [7, 9])
    assert h1 == h2
    assert h1 != oracle.biclique_hash([7, 9], [1, 2, 3])


def test_oracle_generator_matches_the_library(built):
    """The oracle's restatement of the synthetic generator (used by the
    CPU baseline, which must not load the product library) builds the same
    graph as mbe_graph_generate: Chung-Lu, capped, uniform and planted."""
    import cumbe_gb300 as cm
    from cumbe_gb300 import workloads
    cases = [workloads.SINGLE["power_law_2k_1k"], workloads.SINGLE["power_law_94k_30k"],
             dict(n_rows=28000, n_cols=10000, n_edges=160000, gamma_rows=1.9, gamma_cols=1.9, max_deg=0, seed=3,
                  planted=4, planted_rows=20, planted_cols=30, planted_density=0.9)] + workloads.batch(6)
    for p in cases:
        a = oracle.generate(**p)
        b = cm.Graph.generate(**p).csr()
        assert a[:2] == b[:2]
        assert np.array_equal(a[2], b[2]) and np.array_equal(a[3], b[3]), p


def test_root_samples_partition_the_roots(built):
    csr = oracle.generate(2000, 1000, 10000, 2.1, 2.1, 0, 1)
    full = oracle.ref_enumerate(*csr, threads=4)
    parts = [oracle.ref_enumerate_roots(*csr, root_begin=k, root_stride=3, threads=4) for k in range(3)]
    assert sum(p.count for p in parts) == full.count
    assert sum(p.hash for p in parts) % (1 << 64) == full.hash
    lo = oracle.ref_enumerate_roots(*csr, root_end=400, threads=4)
    hi = oracle.ref_enumerate_roots(*csr, root_begin=400, threads=4)
    assert (lo.count + hi.count, (lo.hash + hi.hash) % (1 << 64)) == (full.count, full.hash)
