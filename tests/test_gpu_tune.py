"""GPU: the batched mode's autotuner (mbe_batch_tune).  It times engine
configurations per graph-size bucket and caches the fastest; mbe_batch_run
then runs each group of graphs that share a choice with it.  Results must
not depend on the choice: they are checked against the committed oracle
fixture of the batch workload."""
import json
import os

import pytest

import cumbe_gb300 as cm
from cumbe_gb300 import workloads

pytestmark = pytest.mark.gpu
FIX = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "batch_oracle.json")))


def test_tuned_batch_matches_the_oracle_fixture(engine):
    seeds = sorted(int(k) for k in FIX["graphs"])[:160]
    gs = [cm.Graph.generate(**workloads.batch_params(s)) for s in seeds]
    try:
        choices = engine.batch_tune(gs)
        assert choices and sum(c["n_graphs"] for c in choices) == len(gs)
        for c in choices:
            assert c["trials"] >= 9 and 0 < c["sample_graphs"] <= 32
            assert c["ms_tuned"] <= c["ms_default"]
            assert c["solve_rows"] in (0, 16, 32) and c["donate_min"] in (0, 3, 4)
        res, _ = engine.batch(gs)
        for s, r in zip(seeds, res):
            assert [r.count, f"{r.hash:#018x}"] == FIX["graphs"][str(s)], s
    finally:
        engine.batch_tune_reset()


def test_tuning_rejects_explicit_knobs(engine):
    g = cm.Graph.generate(**workloads.batch_params(0))
    with pytest.raises(cm.MBEError):
        cm.lib()  # loaded
        o = cm._opts(blocks_per_sm=2)
        import ctypes
        arr = (cm._VP * 1)(g.handle)
        out = (cm._TuneChoice * 4)()
        k = ctypes.c_uint32()
        cm._check(cm.lib().mbe_batch_tune(engine._h, arr, 1, 0, ctypes.byref(o), out, 4, ctypes.byref(k)),
                  "mbe_batch_tune")
