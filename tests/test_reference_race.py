"""The reference's own kernels against the oracle on the 9 small fixtures
where its work-stealing variants undercount (reference_counts.json).

tests/golden/reference_counts_repeat.json holds three runs of each variant
per fixture, in device memory and in managed memory (the reference's own
allocation, src/main.cu:41-47,88-110), made by `ref_counts.py --repeat 3`
with the reference's kernels compiled from its sources (oracle/_ref).  The
host steps are deterministic, so counts that differ between runs of one
input come from the kernels themselves: the work-stealing variants race
(src/mbe_cuMBE.cuh:643-1257), while noWS, which only differs by not
stealing, returns the oracle's count on every run in both memories."""
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))
REP = json.load(open(os.path.join(HERE, "golden", "reference_counts_repeat.json")))
EXPECTED = json.load(open(os.path.join(HERE, "golden", "expected.json")))


def test_nows_matches_the_oracle_on_every_run():
    for name, runs in REP.items():
        assert runs["oracle"] == EXPECTED[name]["count"]
        for mem in ("device", "managed"):
            assert runs[f"noWS_{mem}"] == [runs["oracle"]] * len(runs[f"noWS_{mem}"]), name


def test_stealing_variants_never_overcount_and_vary_between_runs():
    varied = 0
    for name, runs in REP.items():
        for v in ("cuMBE", "noES", "noRS"):
            for mem in ("device", "managed"):
                counts = runs[f"{v}_{mem}"]
                assert max(counts) <= runs["oracle"], (name, v, mem)
                varied += len(set(counts)) > 1
    assert varied >= 10  # the same input, different counts: a race in the kernels
