"""Writes stress_sample_oracle.json: the CPU oracle's count and canonical
hash for fixed root samples of the full-size stress graph
(cumbe_gb300.workloads.SINGLE["power_law_1400k_500k"]: 1.4M x 500k rows x
cols, 8M Chung-Lu edges with gamma 1.9, 200 planted K_{20,30} blocks at
density 0.9 over hubs; 8,107,119 distinct edges).  Its full enumeration is
out of reach for any engine; a sample of roots (mbe_opts.root_begin /
root_end / root_stride over the processing order) is not.  The oracle's
restatement of the reference's search spends minutes on these samples
(each root next to a hub scans the hub's ~287k-entry list per child), so
the results are committed and tests/test_gpu_stress_sample.py compares the
GPU engine with them.

    python tests/golden/make_stress_sample.py [--threads N]
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

# (root_begin, root_end, root_stride): roots of degree 1..2, and of degree
# 2..5 further along the processing order.  Roots of higher degree next to
# several hubs are out of the oracle's reach (each of their children rescans
# the hubs' lists); the GPU engine enumerates them in the bench sample.
SAMPLES = [(0, 100000, 1000), (100000, 300000, 5000)]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 4)
    args = ap.parse_args()
    import oracle
    from cumbe_gb300 import workloads
    p = workloads.SINGLE["power_law_1400k_500k"]
    g = oracle.generate(**p)
    out = {"graph": "power_law_1400k_500k", "params": p, "n_edges": int(len(g[3])), "samples": []}
    for b, e, s in SAMPLES:
        t0 = time.time()
        r = oracle.ref_enumerate_roots(*g, root_begin=b, root_end=e, root_stride=s, threads=args.threads)
        out["samples"].append({"root_begin": b, "root_end": e, "root_stride": s, "count": r.count,
                               "hash": f"{r.hash:#018x}", "oracle_nodes": r.nodes,
                               "oracle_s": round(time.time() - t0, 1), "oracle_threads": args.threads})
        print(out["samples"][-1], flush=True)
    with open(os.path.join(HERE, "stress_sample_oracle.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
