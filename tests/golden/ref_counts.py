"""Runs the reference's own kernels (oracle/_ref: the cubin compiled from
its sources and ref_runner) on every golden fixture and variant, and writes
the counts it prints to reference_counts.json.  Needs a GPU.

    python tests/golden/ref_counts.py [--out path]
"""
import argparse
import json
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def repeat_runs(built, expected, names, repeat, out_path):
    """Runs the reference's work-stealing variants `repeat` times on each
    fixture named, in device and in managed memory, and records every count:
    the host steps are deterministic, so counts that differ between runs of
    the same input come from the reference's kernels themselves."""
    out = {}
    for name in names:
        e = expected[name]
        out[name] = {"oracle": e["count"]}
        for variant in ["cuMBE", "noES", "noRS", "noWS"]:
            for mem in ["device", "managed"]:
                counts = []
                for _ in range(repeat):
                    r = subprocess.run([built["runner"], built["cubin"], os.path.join(HERE, e["file"]), variant, mem],
                                       capture_output=True, text=True, timeout=600)
                    if r.returncode != 0:
                        raise SystemExit(f"{name} {variant} {mem}: runner failed: {r.stderr}")
                    counts.append(int(re.search(r"maximal bicliques: (-?\d+)", r.stdout).group(1)))
                out[name][f"{variant}_{mem}"] = counts
        print(name, out[name], flush=True)
    with open(out_path, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "reference_counts.json"))
    ap.add_argument("--repeat", type=int, default=0,
                    help="instead: rerun the fixtures where a stealing variant undercounts, N times each")
    args = ap.parse_args()
    import build_ref
    built = build_ref.build()
    if not built["cubin"] or not built["runner"]:
        raise SystemExit(f"reference build incomplete: {built}")
    expected = json.load(open(os.path.join(HERE, "expected.json")))
    if args.repeat:
        known = json.load(open(os.path.join(HERE, "reference_counts.json")))
        names = sorted(n for n, v in known.items()
                       if any(v[x]["count"] != expected[n]["count"] for x in ("cuMBE", "noES", "noRS")))
        repeat_runs(built, expected, names, args.repeat, os.path.join(HERE, "reference_counts_repeat.json"))
        return
    out = {}
    for name, e in sorted(expected.items()):
        out[name] = {}
        for variant in ["cuMBE", "noRS", "noES", "noWS"]:
            r = subprocess.run([built["runner"], built["cubin"], os.path.join(HERE, e["file"]), variant],
                               capture_output=True, text=True, timeout=600)
            if r.returncode != 0:
                raise SystemExit(f"{name} {variant}: runner failed: {r.stderr}")
            m = re.search(r"maximal bicliques: (-?\d+)", r.stdout)
            t = re.search(r"runtime \(s\): ([0-9.eE+-]+)", r.stdout)
            g = re.search(r"grid_size: (\d+)", r.stdout)
            out[name][variant] = {"count": int(m.group(1)), "runtime_s": float(t.group(1)),
                                  "grid_size": int(g.group(1))}
            print(name, variant, out[name][variant], flush=True)
    with open(args.out, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
