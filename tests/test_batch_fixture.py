"""The batched workload against committed oracle results.

tests/golden/batch_oracle.json holds the CPU oracle's count and canonical
hash for the batch workload's graphs with seed < 1024 and at most 40,000
edges (885 graphs; tests/golden/make_batch_fixture.py writes it).  The GPU
test enumerates all of them in ONE mbe_batch_run and checks every graph's
result against the file; the CPU tests pin the file itself."""
import json
import os
import sys

import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
FIX = json.load(open(os.path.join(HERE, "golden", "batch_oracle.json")))


def test_fixture_covers_exactly_the_stated_subset(built):
    import make_batch_fixture
    assert sorted(int(k) for k in FIX["graphs"]) == make_batch_fixture.selected_seeds()


@pytest.mark.parametrize("seed", [0, 3, 17, 101, 517, 1000])
def test_fixture_entries_match_the_oracle(built, seed):
    from cumbe_gb300 import workloads
    if str(seed) not in FIX["graphs"]:
        pytest.skip("seed outside the subset")
    r = oracle.ref_enumerate(*oracle.generate(**workloads.batch_params(seed)), threads=4)
    assert [r.count, f"{r.hash:#018x}"] == FIX["graphs"][str(seed)]


@pytest.mark.gpu
def test_one_batched_launch_matches_the_oracle_fixture(engine):
    import cumbe_gb300 as cm
    from cumbe_gb300 import workloads
    seeds = sorted(int(k) for k in FIX["graphs"])
    gs = [cm.Graph.generate(**workloads.batch_params(s)) for s in seeds]
    res, _ = engine.batch(gs)
    bad = [(s, r.count, f"{r.hash:#018x}", FIX["graphs"][str(s)]) for s, r in zip(seeds, res)
           if [r.count, f"{r.hash:#018x}"] != FIX["graphs"][str(s)]]
    assert not bad, bad[:5]
