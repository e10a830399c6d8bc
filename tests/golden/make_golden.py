"""Generates the golden fixtures: small .bi graphs plus the oracle's
expected count and canonical hash for each (expected.json).

    python tests/golden/make_golden.py

The reference's own counts for the same files come from
tests/golden/ref_counts.py, run on a GPU machine (reference_counts.json).
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import cumbe_gb300 as cm  # noqa: E402
import oracle  # noqa: E402


def random_graph(rng, nr, nc, p):
    M = rng.random((nr, nc)) < p
    rp = np.zeros(nr + 1, np.uint64)
    rp[1:] = np.cumsum(M.sum(1))
    return nr, nc, rp, np.nonzero(M)[1].astype(np.uint32)


def fixtures():
    rng = np.random.default_rng(20261203)
    out = []
    for i in range(16):
        nr = int(rng.integers(20, 90))
        nc = int(rng.integers(20, 90))
        p = float(rng.uniform(0.04, 0.22))
        out.append((f"random_{i:02d}_{nr}x{nc}", random_graph(rng, nr, nc, p)))
    g = cm.Graph.generate(2000, 1000, 10000, 2.1, 2.1, 0, 1)
    out.append(("power_law_2k_1k", g.csr()))
    g = cm.Graph.generate(20000, 6000, 30000, 2.0, 2.3, 1500, 7)
    out.append(("power_law_20k_6k", g.csr()))
    return out


def main():
    expected = {}
    for name, (nr, nc, rp, ci) in fixtures():
        if ci.size == 0:
            continue
        path = os.path.join(HERE, "graphs", name + ".bi")
        cm.Graph.from_csr(nr, nc, rp, ci).write_bi(path)
        r = oracle.ref_enumerate(nr, nc, rp, ci, threads=8)
        expected[name] = {"file": f"graphs/{name}.bi", "n_rows": int(nr), "n_cols": int(nc),
                          "n_edges": int(ci.size), "count": int(r.count), "hash": f"{r.hash:#018x}"}
        print(name, expected[name])
    with open(os.path.join(HERE, "expected.json"), "w") as f:
        json.dump(expected, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
