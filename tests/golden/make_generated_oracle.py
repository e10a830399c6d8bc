"""Adds the CPU oracle's count and canonical hash to an entry of
reference_generated.json (the synthetic graphs whose counts the reference's
own kernels printed), so that the GPU test pins the hash as well as the
count there.  The graph comes from the oracle's copy of the generator.

    python tests/golden/make_generated_oracle.py power_law_94k_30k_e100k [--threads N]
"""
import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("name")
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 4)
    args = ap.parse_args()
    import oracle
    path = os.path.join(HERE, "reference_generated.json")
    doc = json.load(open(path))
    rec = doc[args.name]
    t0 = time.time()
    r = oracle.ref_enumerate(*oracle.generate(**rec["generator"]), threads=args.threads)
    rec["oracle"] = {"count": r.count, "hash": f"{r.hash:#018x}", "oracle_s": round(time.time() - t0, 1),
                     "oracle_threads": args.threads}
    print(args.name, rec["oracle"], flush=True)
    with open(path, "w") as f:
        json.dump(doc, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
