"""Output stream (MBE_OPT_EMIT): the bicliques themselves, not just their
count, against the CPU oracle's lists -- every maximal biclique exactly once,
in file ids, rows then cols."""
import ctypes
import os

import numpy as np
import pytest

import cumbe_gb300 as cm
import oracle
from conftest import random_csr

pytestmark = pytest.mark.gpu
VARIANTS = ["cuMBE", "noRS", "noES", "noWS"]


def _canon(bl):
    return sorted((tuple(sorted(a)), tuple(sorted(b))) for a, b in bl)


def _check_emit(engine, g, variant="cuMBE", min_rows=0, min_cols=0, **tuning):
    nr, nc, rp, ci = g
    want = oracle.ref_enumerate(nr, nc, rp, ci, threads=1, min_rows=min_rows, min_cols=min_cols,
                                emit_cap=4 * 10 ** 5, emit_ids_cap=32 * 10 ** 6)
    G = cm.Graph.from_csr(nr, nc, rp, ci)
    got = engine.enumerate(G, variant, min_rows=min_rows, min_cols=min_cols, emit_cap=max(1, want.count),
                           emit_ids_cap=sum(len(a) + len(b) for a, b in want.bicliques) or 1, **tuning)
    assert (got.count, got.hash) == (want.count, want.hash), (variant, got, want)
    assert len(got.bicliques) == got.count
    assert _canon(got.bicliques) == _canon(want.bicliques), variant
    h = 0
    for a, b in got.bicliques:
        h = (h + cm.biclique_hash(a, b)) & (2 ** 64 - 1)
    assert h == got.hash
    return got


def test_emit_tiny_random_all_variants(engine):
    rng = np.random.default_rng(21)
    for _ in range(25):
        g = random_csr(rng, int(rng.integers(1, 12)), int(rng.integers(1, 12)), rng.uniform(0.1, 0.9))
        for v in VARIANTS:
            _check_emit(engine, g, v)


@pytest.mark.parametrize("shape", [(60, 40, 0.12), (40, 60, 0.2), (33, 70, 0.5)])
def test_emit_medium_both_orientations(engine, shape):
    rng = np.random.default_rng(sum(int(x * 100) for x in shape))
    g = random_csr(rng, *shape)
    for v in ("cuMBE", "noWS"):
        _check_emit(engine, g, v)


def test_emit_power_law(engine):
    """2,000 x 1,000 Chung-Lu graph (gamma 2.1, 10,000 edges, seed 1): deep
    trees, packed records, the register-resident search and donation."""
    G = cm.Graph.generate(2000, 1000, 10000, 2.1, 2.1, 0, 1)
    _check_emit(engine, G.csr())


def test_emit_thresholds(engine):
    rng = np.random.default_rng(9)
    g = random_csr(rng, 70, 45, 0.18)
    for a, b in [(2, 2), (3, 1), (1, 4)]:
        _check_emit(engine, g, "cuMBE", min_rows=a, min_cols=b)


def test_emit_through_pool_records_and_replays(engine):
    """Tiny arenas put child records (with their R lists) in the shared pool
    and make donations replay paths; a tiny pool forces chunked roots."""
    G = cm.Graph.generate(2000, 1000, 10000, 2.1, 2.1, 0, 1)
    _check_emit(engine, G.csr(), stack_words=4096)
    old = os.environ.get("MBE_POOL_MB")
    os.environ["MBE_POOL_MB"] = "2"
    try:
        _check_emit(engine, G.csr())
    finally:
        if old is None:
            del os.environ["MBE_POOL_MB"]
        else:
            os.environ["MBE_POOL_MB"] = old


def test_emit_overflow_is_an_error(engine):
    G = cm.Graph.generate(2000, 1000, 10000, 2.1, 2.1, 0, 1)
    with pytest.raises(RuntimeError, match="emit buffers full"):
        engine.enumerate(G, emit_cap=100)
    # the context stays usable
    full = engine.enumerate(G)
    assert full.count == 28539


def test_emit_rejected_for_batches(engine):
    G = cm.Graph.generate(200, 100, 900, 2.1, 2.1, 0, 1)
    o = cm._opts(flags=cm.OPT_EMIT)
    arr = (ctypes.c_void_p * 2)(G.handle, G.handle)
    res = (cm._Result * 2)()
    tot = ctypes.c_float(0)
    st = cm.lib().mbe_batch_run(engine._h, arr, 2, 0, ctypes.byref(o), res, ctypes.byref(tot))
    assert st == 1  # MBE_ERR_INVALID_ARG
