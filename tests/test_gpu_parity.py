"""GPU parity: libmbe's sm_103a kernels against the CPU oracle (count and
canonical hash bit-exact), through the C ABI."""
import os

import numpy as np
import pytest

import cumbe_gb300 as cm
import oracle
from conftest import random_csr

pytestmark = pytest.mark.gpu
VARIANTS = ["cuMBE", "noRS", "noES", "noWS"]


def _check(engine, g, variant="cuMBE", **kw):
    nr, nc, rp, ci = g
    want = oracle.ref_enumerate(nr, nc, rp, ci, threads=4, **kw)
    G = cm.Graph.from_csr(nr, nc, rp, ci)
    got = engine.enumerate(G, variant, **kw)
    assert (got.count, got.hash) == (want.count, want.hash), (variant, kw, got, want)
    return got


def test_tiny_random_all_variants(engine):
    rng = np.random.default_rng(11)
    for _ in range(60):
        g = random_csr(rng, int(rng.integers(1, 14)), int(rng.integers(1, 14)), rng.uniform(0.05, 0.95))
        for v in VARIANTS:
            _check(engine, g, v)


@pytest.mark.parametrize("shape", [(60, 40, 0.12), (40, 60, 0.2), (120, 90, 0.05), (33, 70, 0.5)])
def test_medium_random(engine, shape):
    rng = np.random.default_rng(hash(shape) & 0xFFFF)
    g = random_csr(rng, *shape)
    for v in VARIANTS:
        _check(engine, g, v)


def test_edge_cases(engine):
    cases = [
        (3, 4, np.zeros(4, np.uint64), np.zeros(0, np.uint32)),
        (1, 1, np.array([0, 1], np.uint64), np.array([0], np.uint32)),
        (3, 5, np.array([0, 5, 10, 15], np.uint64), np.tile(np.arange(5, dtype=np.uint32), 3)),
        (4, 3, np.array([0, 1, 1, 2, 2], np.uint64), np.array([0, 2], np.uint32)),
        (0, 3, np.zeros(1, np.uint64), np.zeros(0, np.uint32)),
        (40, 1, np.arange(41, dtype=np.uint64), np.zeros(40, np.uint32)),
    ]
    for g in cases:
        for v in VARIANTS:
            _check(engine, g, v)


def test_config0_synthetic(engine):
    """|U|=2000, |V|=1000, 10,000 Chung-Lu edges (gamma 2.1), seed 1."""
    G = cm.Graph.generate(2000, 1000, 10000, 2.1, 2.1, 0, 1)
    nr, nc, rp, ci = G.csr()
    want = oracle.ref_enumerate(nr, nc, rp, ci, threads=8)
    for v in VARIANTS:
        got = engine.enumerate(G, v)
        assert (got.count, got.hash) == (want.count, want.hash), v


def test_thresholds(engine):
    rng = np.random.default_rng(5)
    g = random_csr(rng, 80, 50, 0.15)
    for a, b in [(1, 1), (2, 2), (3, 1), (1, 4), (4, 4)]:
        _check(engine, g, "cuMBE", min_rows=a, min_cols=b)


def test_batch_matches_single(engine):
    rng = np.random.default_rng(9)
    gs, want = [], []
    for i in range(40):
        g = random_csr(rng, int(rng.integers(2, 70)), int(rng.integers(2, 70)), rng.uniform(0.02, 0.3))
        gs.append(cm.Graph.from_csr(*g))
        want.append(oracle.ref_enumerate(*g))
    res, ms = engine.batch(gs)
    for r, w in zip(res, want):
        assert (r.count, r.hash) == (w.count, w.hash)


def test_small_pool_forces_chunks(engine):
    """A tiny node pool makes the root expansion run in many chunks with
    retries; results must not change."""
    G = cm.Graph.generate(2000, 1000, 10000, 2.1, 2.1, 0, 1)
    nr, nc, rp, ci = G.csr()
    want = oracle.ref_enumerate(nr, nc, rp, ci, threads=8)
    old = os.environ.get("MBE_POOL_MB")
    os.environ["MBE_POOL_MB"] = "2"
    try:
        got = engine.enumerate(G)
    finally:
        if old is None:
            del os.environ["MBE_POOL_MB"]
        else:
            os.environ["MBE_POOL_MB"] = old
    assert (got.count, got.hash) == (want.count, want.hash)


def test_small_arena_spills_to_pool(engine):
    """A 4096-word DFS arena forces child records into the shared node pool
    and donations to replay deep paths; results must not change."""
    G = cm.Graph.generate(2000, 1000, 10000, 2.1, 2.1, 0, 1)
    nr, nc, rp, ci = G.csr()
    want = oracle.ref_enumerate(nr, nc, rp, ci, threads=8)
    got = engine.enumerate(G, stack_words=4096)
    assert (got.count, got.hash) == (want.count, want.hash)


def test_donation_granularity_does_not_change_results(engine):
    G = cm.Graph.generate(3000, 1500, 16000, 2.0, 2.2, 0, 4)
    base = engine.enumerate(G, "noWS")
    for dm in (2, 3, 8, 64):
        got = engine.enumerate(G, "cuMBE", donate_min=dm)
        assert (got.count, got.hash) == (base.count, base.hash), dm


def test_stress_graph_shape_small_scale(engine):
    """The load-imbalance stress graph's shape (Chung-Lu gamma 1.9 on both
    sides, no degree cap, a planted K_{20,30} block at density 0.9 over hubs)
    at 1/250 of its size: 5,600 x 2,000, 32,000 edges, 920,386 bicliques."""
    G = cm.Graph.generate(5600, 2000, 32000, 1.9, 1.9, 0, 3, planted=1, planted_rows=20, planted_cols=30,
                          planted_density=0.9)
    nr, nc, rp, ci = G.csr()
    want = oracle.ref_enumerate(nr, nc, rp, ci, threads=os.cpu_count() or 8)
    assert want.count == 920386
    for v in ("cuMBE", "noWS"):
        got = engine.enumerate(G, v)
        assert (got.count, got.hash) == (want.count, want.hash), v


@pytest.mark.parametrize("env", [{"MBE_SOLVE_ROWS": "0"}, {"MBE_SOLVE_ROWS": "16"}, {"MBE_DONATE_COPY": "0"},
                                 {"MBE_SOLVE_ROWS": "0", "MBE_DONATE_COPY": "0"}])
def test_alternative_paths_give_the_same_bicliques(engine, env):
    """The record path instead of the register search, and path-replay
    donation instead of pool copies, must not change any result."""
    G = cm.Graph.generate(3000, 1500, 16000, 2.0, 2.2, 0, 4)
    rng = np.random.default_rng(8)
    H = cm.Graph.from_csr(*random_csr(rng, 90, 60, 0.15))
    base = [engine.enumerate(x) for x in (G, H)]
    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        got = [engine.enumerate(x) for x in (G, H)]
        em = engine.enumerate(H, emit_cap=base[1].count)
    finally:
        for k, v in old.items():
            if v is None:
                del os.environ[k]
            else:
                os.environ[k] = v
    assert [(r.count, r.hash) for r in got] == [(r.count, r.hash) for r in base], env
    assert (em.count, em.hash, len(em.bicliques)) == (base[1].count, base[1].hash, base[1].count)


def test_randomized_sweep_against_the_oracle(engine):
    """150 random graphs: sizes 5..150 per side, densities 0.02..0.5, both
    orientations.  On graphs this small thousands of warps wait for work,
    so donation (pool copies and path replays) and the register search run
    constantly."""
    rng = np.random.default_rng(2026)
    for i in range(150):
        nr, nc = int(rng.integers(5, 151)), int(rng.integers(5, 151))
        p = float(np.exp(rng.uniform(np.log(0.02), np.log(0.5))))
        if nr * nc * p > 2500:  # keep the oracle's share of the test time small
            p = 2500.0 / (nr * nc)
        g = random_csr(rng, nr, nc, p)
        _check(engine, g, "cuMBE" if i % 3 else "noRS")
