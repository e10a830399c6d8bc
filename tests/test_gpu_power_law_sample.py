"""GPU: the headline graph (94,000 x 30,000, 293,000 Chung-Lu edges, gammas
2.0 / 2.3, degree cap 7,500, seed 2) enumerated on two fixed root samples
by all four variants.  Count and hash must equal the CPU oracle's over the
same roots, committed in tests/golden/power_law_sample_oracle.json
(make_power_law_sample.py): the whole graph's count is pinned by the
reference's own kernel, and these samples pin the hash on the same
full-size graph."""
import json
import os

import pytest

import cumbe_gb300 as cm
from cumbe_gb300 import workloads

pytestmark = pytest.mark.gpu
FIX_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "power_law_sample_oracle.json")


def test_headline_graph_root_samples_match_the_oracle(engine):
    fix = json.load(open(FIX_PATH))
    g = cm.Graph.generate(**workloads.SINGLE["power_law_94k_30k"])
    assert g.info()["n_edges"] == fix["n_edges"]
    try:
        for smp in fix["samples"]:
            kw = dict(root_begin=smp["root_begin"], root_end=smp["root_end"], root_stride=smp["root_stride"])
            for v in ("cuMBE", "noRS", "noES", "noWS"):
                r = engine.enumerate(g, v, **kw)
                assert (r.count, f"{r.hash:#018x}") == (smp["count"], smp["hash"]), (v, kw)
    finally:
        engine.release(g)
