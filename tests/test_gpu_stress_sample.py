"""GPU: the stress graph at its full stated size (1.4M x 500k, 8M Chung-Lu
edges with gamma 1.9, 200 planted K_{20,30} blocks at density 0.9 over
hubs), generated, uploaded and transposed on the device, then enumerated on
fixed root samples (its full enumeration is out of reach for any engine).
Count and hash must equal the CPU oracle's over the same roots, committed
in tests/golden/stress_sample_oracle.json (make_stress_sample.py)."""
import json
import os

import pytest

import cumbe_gb300 as cm
from cumbe_gb300 import workloads

pytestmark = pytest.mark.gpu
FIX_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "stress_sample_oracle.json")


@pytest.fixture(scope="module")
def stress_graph():
    return cm.Graph.generate(**workloads.SINGLE["power_law_1400k_500k"])


def test_full_size_stress_graph_samples_match_the_oracle(engine, stress_graph):
    fix = json.load(open(FIX_PATH))
    assert stress_graph.info()["n_edges"] == fix["n_edges"]
    try:
        for smp in fix["samples"]:
            kw = dict(root_begin=smp["root_begin"], root_end=smp["root_end"], root_stride=smp["root_stride"])
            for v in ("cuMBE", "noWS"):
                r = engine.enumerate(stress_graph, v, **kw)
                assert (r.count, f"{r.hash:#018x}") == (smp["count"], smp["hash"]), (v, kw)
    finally:
        engine.release(stress_graph)
