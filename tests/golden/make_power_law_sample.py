"""Writes power_law_sample_oracle.json: the CPU oracle's count and canonical
hash for fixed root samples of the headline graph
(cumbe_gb300.workloads.SINGLE["power_law_94k_30k"]: 94,000 x 30,000 rows x
cols, 293,000 Chung-Lu edges, gammas 2.0 / 2.3, degree cap 7,500, seed 2).
The oracle's restatement of the reference's search needs hours for the
whole graph (its count alone is pinned by the reference's own kernel,
reference_generated.json); stride samples of the roots (mbe_opts.root_begin
/ root_end / root_stride over the processing order, degree ascending) take
minutes and pin the hash on the full-size graph too.
tests/test_gpu_power_law_sample.py compares the GPU engine with them.

    python tests/golden/make_power_law_sample.py [--threads N]
"""
import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

# (root_begin, root_end, root_stride): every 1000th root (the bench's CPU
# baseline sample) and every 250th from an odd offset, both spanning light
# and heavy roots of the processing order.
SAMPLES = [(0, 30000, 1000), (7, 30000, 250)]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 4)
    args = ap.parse_args()
    import oracle
    from cumbe_gb300 import workloads
    p = workloads.SINGLE["power_law_94k_30k"]
    g = oracle.generate(**p)
    out = {"graph": "power_law_94k_30k", "params": p, "n_edges": int(len(g[3])), "samples": []}
    for b, e, s in SAMPLES:
        t0 = time.time()
        r = oracle.ref_enumerate_roots(*g, root_begin=b, root_end=e, root_stride=s, threads=args.threads)
        out["samples"].append({"root_begin": b, "root_end": e, "root_stride": s, "count": r.count,
                               "hash": f"{r.hash:#018x}", "oracle_nodes": r.nodes,
                               "oracle_s": round(time.time() - t0, 1), "oracle_threads": args.threads})
        print(out["samples"][-1], flush=True)
    with open(os.path.join(HERE, "power_law_sample_oracle.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
