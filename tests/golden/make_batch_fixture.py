"""Writes batch_oracle.json: the CPU oracle's count and canonical hash for
the batched workload's graphs (cumbe_gb300.workloads.batch_params(seed))
with seed < 1024 and at most 40,000 edges, the subset the oracle finishes
in about a minute.  The graphs come from the oracle's own copy of the
generator.  tests/test_batch_fixture.py runs them as one mbe_batch_run and
checks every graph's result against this file.

    python tests/golden/make_batch_fixture.py [--threads N]
"""
import argparse
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

MAX_SEED = 1024
MAX_EDGES = 40000


def selected_seeds():
    from cumbe_gb300 import workloads
    return [s for s in range(MAX_SEED) if workloads.batch_params(s)["n_edges"] <= MAX_EDGES]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 4)
    args = ap.parse_args()
    import oracle
    from cumbe_gb300 import workloads
    out = {"rule": f"seeds < {MAX_SEED} with n_edges <= {MAX_EDGES}", "graphs": {}}
    for s in selected_seeds():
        p = workloads.batch_params(s)
        r = oracle.ref_enumerate(*oracle.generate(**p), threads=args.threads)
        out["graphs"][str(s)] = [r.count, f"{r.hash:#018x}"]
    with open(os.path.join(HERE, "batch_oracle.json"), "w") as f:
        json.dump(out, f, indent=0, sort_keys=True)
    print(len(out["graphs"]), "graphs,", sum(v[0] for v in out["graphs"].values()), "bicliques")


if __name__ == "__main__":
    main()
