"""GPU: root samples and bounded device waits, through the C ABI.

Root samples (mbe_opts.root_begin / root_end / root_stride) select roots by
their position in the processing order (degree ascending, id ascending);
the engine's result must equal the oracle's over the same sample, and
disjoint samples must add up to the whole graph's count and hash.

The bounded waits: every device-side wait of the enumeration kernels ends,
after wait_timeout_ns without progress anywhere on the device, in an error
status the host reads (MBE_ERR_DEVICE_TIMEOUT), never a trap.  A limit of
1 ns makes the idle warps' waits for a task run out; the call must fail
with that status, the kernels must have exited, and the same context must
then enumerate correctly."""
import numpy as np
import pytest

import cumbe_gb300 as cm
import oracle
from conftest import random_csr

pytestmark = pytest.mark.gpu


def _graphs():
    rng = np.random.default_rng(77)
    return {
        "power_law_2k_1k": cm.Graph.generate(2000, 1000, 10000, 2.1, 2.1, 0, 1).csr(),  # rows > cols: swapped
        "random_90x160": random_csr(rng, 90, 160, 0.08),                                # not swapped
    }


SAMPLES = [dict(root_begin=0, root_stride=3), dict(root_begin=1, root_stride=3), dict(root_begin=2, root_stride=3),
           dict(root_begin=100, root_end=700), dict(root_begin=5, root_stride=7), dict(root_begin=0, root_end=1)]


@pytest.mark.parametrize("name", ["power_law_2k_1k", "random_90x160"])
@pytest.mark.parametrize("variant", ["cuMBE", "noWS"])
def test_root_sample_matches_oracle(engine, name, variant):
    nr, nc, rp, ci = _graphs()[name]
    G = cm.Graph.from_csr(nr, nc, rp, ci)
    for smp in SAMPLES:
        want = oracle.ref_enumerate_roots(nr, nc, rp, ci, variant=variant, threads=4, **smp)
        got = engine.enumerate(G, variant, **smp)
        assert (got.count, got.hash) == (want.count, want.hash), (name, variant, smp)


def test_disjoint_samples_add_up_to_the_whole_graph(engine):
    nr, nc, rp, ci = _graphs()["power_law_2k_1k"]
    G = cm.Graph.from_csr(nr, nc, rp, ci)
    full = engine.enumerate(G)
    parts = [engine.enumerate(G, root_begin=k, root_stride=4) for k in range(4)]
    assert sum(p.count for p in parts) == full.count
    assert sum(p.hash for p in parts) % (1 << 64) == full.hash


def test_root_sample_in_a_batch(engine):
    gs = [cm.Graph.generate(**p) for p in
          [dict(n_rows=300, n_cols=150, n_edges=2500, seed=s, gamma_rows=0.0, gamma_cols=0.0) for s in range(6)]]
    res, _ = engine.batch(gs, root_begin=3, root_stride=2)
    for g, r in zip(gs, res):
        want = oracle.ref_enumerate_roots(*g.csr(), root_begin=3, root_stride=2, threads=4)
        assert (r.count, r.hash) == (want.count, want.hash)


def test_bad_options_are_rejected(engine):
    G = cm.Graph.generate(200, 100, 800, 2.1, 2.1, 0, 1)
    for bad in [dict(warps_per_block=3), dict(root_begin=10, root_end=10)]:
        with pytest.raises(cm.MBEError) as e:
            engine.enumerate(G, **bad)
        assert e.value.status == 1  # MBE_ERR_INVALID_ARG
    engine.enumerate(G, warps_per_block=4)  # the compiled shape is accepted


def test_device_wait_timeout_is_an_error_status_and_the_context_recovers(engine):
    g = cm.Graph.generate(2000, 1000, 10000, 2.1, 2.1, 0, 1)
    want = oracle.ref_enumerate(*g.csr(), threads=4)
    with pytest.raises(cm.MBEError) as e:
        engine.enumerate(g, wait_timeout_ns=1)
    assert e.value.status == 6  # MBE_ERR_DEVICE_TIMEOUT
    assert "timed out" in str(e.value)
    for _ in range(2):
        got = engine.enumerate(g)
        assert (got.count, got.hash) == (want.count, want.hash)


def test_l2_persisting_window_gives_the_same_result(engine):
    """MBE_OPT_L2_PIN (an access-policy window keeping the L-side adjacency
    persisting in L2 for a one-graph run) changes no result, and the window
    is cleared afterwards (a later plain run is exact too)."""
    g = cm.Graph.generate(2000, 1000, 10000, 2.1, 2.1, 0, 1)
    want = oracle.ref_enumerate(*g.csr(), threads=4)
    for pin in (True, False, True):
        got = engine.enumerate(g, l2_pin=pin)
        assert (got.count, got.hash) == (want.count, want.hash), pin


def test_one_batch_with_different_thresholds_per_entry(engine):
    """Thresholds travel per entry of a launch (the server batches requests
    with different thresholds together): the same graph twice, and graphs of
    both orientations, each with its own |A| >= a, |B| >= b, in one batched
    launch, against the oracle."""
    import ctypes
    rng = np.random.default_rng(3)
    gs = [cm.Graph.from_csr(*random_csr(rng, 40, 70, 0.12)), cm.Graph.from_csr(*random_csr(rng, 80, 35, 0.15))]
    entries = [(gs[0], 0, 0), (gs[0], 2, 3), (gs[1], 3, 2), (gs[1], 0, 0), (gs[0], 4, 1)]
    blocker = cm.Graph.generate(2000, 1000, 10000, 2.1, 2.1, 0, 1)  # keeps the slot busy while the rest queue
    srv = cm.Server(0, slots=1, max_batch=64)
    try:
        gids = [srv.add_graph(g) for g in gs]
        srv.submit(srv.add_graph(blocker))
        rids = [srv.submit(gids[gs.index(g)], a, b) for g, a, b in entries]
        out, t0 = [], __import__("time").time()
        while len(out) < len(rids) + 1 and __import__("time").time() - t0 < 60:
            out += srv.poll()
    finally:
        srv.stop()
    res = {r["request"]: r for r in out}
    for rid, (g, a, b) in zip(rids, entries):
        want = oracle.ref_enumerate(*g.csr(), threads=2, min_rows=a, min_cols=b)
        assert (res[rid]["count"], res[rid]["hash"]) == (want.count, want.hash), (a, b)
