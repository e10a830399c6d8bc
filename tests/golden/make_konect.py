"""Makes the KONECT-converter fixtures in tests/golden/konect/: seeded
synthetic edge-pair files in the KONECT layout ("%" header lines, then
"source target [weight [time]]" lines) and the `.bi` files the reference's
own converter (data/gen_bi.cpp, built unmodified into oracle/_ref/gen_bi by
oracle/build_ref.py) writes for them.  Run from the repository root where
the reference sources are present:  python tests/golden/make_konect.py"""
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "konect")
GEN = os.path.join(ROOT, "oracle", "_ref", "gen_bi")


def konect_text(rng, n_src, n_dst, n_edges, extra, negative=False, tail=""):
    src_ids = rng.choice(10 ** 6, n_src, replace=False) - (5 * 10 ** 5 if negative else 0)
    dst_ids = rng.choice(10 ** 6, n_dst, replace=False)
    s = rng.choice(src_ids, n_edges)
    d = rng.choice(dst_ids, n_edges)
    dup = rng.integers(0, n_edges, n_edges // 10)  # repeated pairs
    s = np.concatenate([s, s[dup]])
    d = np.concatenate([d, d[dup]])
    head = f"% bip {'weighted' if extra else 'unweighted'}\n% {len(s)} {n_src} {n_dst}\n"
    lines = []
    for a, b in zip(s.tolist(), d.tolist()):
        cols = [str(a), str(b)] + [str(int(x)) for x in rng.integers(1, 10 ** 9, extra)]
        lines.append(("\t" if rng.random() < 0.5 else " ").join(cols))
    return head + "\n".join(lines) + "\n" + tail, 7, extra


def main():
    if not os.path.exists(GEN):
        sys.exit("oracle/_ref/gen_bi is missing: run oracle/build_ref.py where the reference sources are present")
    os.makedirs(OUT, exist_ok=True)
    rng = np.random.default_rng(2024)
    cases = {
        "unweighted": konect_text(rng, 60, 25, 400, 0),
        "weighted_timed": konect_text(rng, 40, 90, 700, 2),
        "negative_ids_ragged_tail": konect_text(rng, 30, 30, 300, 1, negative=True, tail="17"),
    }
    meta = {}
    for name, (text, skip, skip_edge) in cases.items():
        src = os.path.join(OUT, name + ".tsv")
        dst = os.path.join(OUT, name + ".ref.bi")
        with open(src, "w") as f:
            f.write(text)
        subprocess.run([GEN, src, dst, str(skip), str(skip_edge)], check=True, capture_output=True)
        meta[name] = {"input": name + ".tsv", "reference_bi": name + ".ref.bi", "skip_words": skip,
                      "skip_words_per_edge": skip_edge}
    with open(os.path.join(OUT, "cases.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(json.dumps(meta, indent=1))


if __name__ == "__main__":
    main()
