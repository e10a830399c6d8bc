"""GPU: the batched mode with its chunk loop inside a captured CUDA graph
(the default; MBE_OPT_HOST_CHUNKS drives it from the host).  The 885 graphs of the batch oracle fixture run in one
mbe_batch_run with the default chunks, and again with 32 MiB chunks and
one chunk per launch of the captured graph (MBE_GRAPH_CHUNKS=1), so the
graph is launched again and again; and a graph whose root records crowd a
1 MiB pool, where a record that does not fit hands the run to the
host-driven chunk loop (which re-queues it).  Every result must equal the
oracle's (or, with the small pool, the host-driven loop's, itself pinned to
the oracle elsewhere).  A run that stayed in graph mode reports its whole
device time in ms (ms_prep 0)."""
import json
import os

import pytest

import cumbe_gb300 as cm
from cumbe_gb300 import workloads

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
FIX = json.load(open(os.path.join(HERE, "golden", "batch_oracle.json")))


class env:
    """Environment variables set for the duration of a with-block."""

    def __init__(self, **kv):
        self.kv, self.old = {k: str(v) for k, v in kv.items()}, {}

    def __enter__(self):
        for k, v in self.kv.items():
            self.old[k] = os.environ.get(k)
            os.environ[k] = v

    def __exit__(self, *exc):
        for k, v in self.old.items():
            if v is None:
                del os.environ[k]
            else:
                os.environ[k] = v


@pytest.fixture(scope="module")
def fixture_graphs():
    seeds = sorted(int(k) for k in FIX["graphs"])
    return seeds, [cm.Graph.generate(**workloads.batch_params(s)) for s in seeds]


def _mismatches(seeds, res):
    return [(s, r.count, f"{r.hash:#018x}", FIX["graphs"][str(s)]) for s, r in zip(seeds, res)
            if [r.count, f"{r.hash:#018x}"] != FIX["graphs"][str(s)]]


def test_graph_mode_batch_matches_the_oracle_fixture(engine, fixture_graphs):
    seeds, gs = fixture_graphs
    res, ms = engine.batch(gs)
    assert not _mismatches(seeds, res)
    assert ms > 0 and all(r.ms_prep == 0 for r in res)  # the chunk loop ran as a captured graph


def test_host_driven_chunk_loop_matches_the_oracle_fixture(engine, fixture_graphs):
    seeds, gs = fixture_graphs
    res, _ = engine.batch(gs, host_chunks=True)
    assert not _mismatches(seeds, res)
    assert all(r.ms_prep > 0 for r in res)  # root expansion timed apart: the host loop ran


def test_graph_mode_over_many_launches_of_the_captured_chunks(engine, fixture_graphs):
    seeds, gs = fixture_graphs
    # a 64 MiB pool: 32 MiB of root records per chunk, and room beside them
    # for the records of every root expansion block in flight (the largest
    # of these graphs' records is under 13k words)
    with env(MBE_POOL_MB=64, MBE_GRAPH_CHUNKS=1):
        res, _ = engine.batch(gs)
    assert not _mismatches(seeds, res)
    assert all(r.ms_prep == 0 for r in res)


def test_graph_mode_with_a_pool_too_small_for_records_side_by_side(engine):
    # the stress shape at 1/250 has root records of up to ~0.5 MB: in a
    # 1 MiB pool, records claimed side by side at a chunk's start can
    # overflow it, and those roots must be re-queued, not lost
    gs = [cm.Graph.generate(**workloads.stress_params(250))] + \
         [cm.Graph.generate(**workloads.batch_params(s)) for s in (0, 3, 17)]
    want, _ = engine.batch(gs, host_chunks=True)
    with env(MBE_POOL_MB=1):
        got, _ = engine.batch(gs)
    assert [(r.count, r.hash) for r in got] == [(r.count, r.hash) for r in want]
    assert got[0].count == 920386  # the oracle's count for this graph
