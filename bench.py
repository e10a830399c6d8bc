"""Throughput benchmark: maximal biclique enumeration on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--workload power_law_94k_30k]

A step is one full enumeration (count + canonical hash) of the workload
graph.  Prints ONE JSON line (rank 0).

  value      maximal bicliques/sec with the graph resident in HBM: the sum
             of counts over the K timed steps / the sum of the steps' device
             time (CUDA events on the library's stream around the root
             expansion and DFS kernels); L2 is flushed (a 512 MiB write)
             before every timed step.
  e2e        the same metric through the public C ABI from host buffers:
             every step drops the device copy, then mbe_enumerate uploads
             (host->device copies, transpose, root order), enumerates and
             copies the result back; wall-clock per step.
  roofline   dfs_kernel's algorithmic bytes (4 B x 32-bit words of bit rows
             and candidate data it streams, as the kernel's word counter
             counted them when the per-workload figure was frozen) / its
             event time, against the measured HBM copy bandwidth.
  cpu_baseline  the CPU oracle (a restatement of the reference's search) on
             the host cores over a stride sample of the same graph's roots.

`--impl reference` times that CPU restatement alone (the reference ships
no CPU implementation of this path; its GPU kernels cannot be installed
as a package), on the same metric, one stride sample per step.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# The workloads (synthetic, seeded).  The default is the one the headline
# metric is quoted on: a 94,000 x 30,000 power-law bipartite graph.
WORKLOADS = {
    "power_law_94k_30k": dict(n_rows=94000, n_cols=30000, n_edges=293000, gamma_rows=2.0, gamma_cols=2.3,
                              max_deg=7500, seed=2, cpu_stride=1000),
    # same generator with 100k edges: the small case ncu captures run on
    "power_law_94k_30k_e100k": dict(n_rows=94000, n_cols=30000, n_edges=100000, gamma_rows=2.0, gamma_cols=2.3,
                                    max_deg=7500, seed=2, cpu_stride=100),
    "power_law_2k_1k": dict(n_rows=2000, n_cols=1000, n_edges=10000, gamma_rows=2.1, gamma_cols=2.1,
                            max_deg=0, seed=1, cpu_stride=1),
}
DEFAULT_WORKLOAD = "power_law_94k_30k"
FALLBACK_HBM_GBS = 6800.0


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x, world, device):
    """The largest of the ranks' values of x (the slowest replica's step
    time); x itself on one rank."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x, world, device):
    """The sum of the ranks' integer values of x (each rank's share of the
    bicliques); x itself on one rank."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.int64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return int(t.item())


def shard_of(rank, world):
    """Root sample of one rank: processing positions rank, rank + world, ...
    (round-robin over the degree order, so every rank gets the same mix of
    light and heavy roots).  The shards partition the roots, so the ranks'
    counts (and hashes, a wrapping sum) add up to the whole graph's."""
    if world <= 1:
        return {}
    return {"root_begin": rank, "root_stride": world}


def sharded_value(total_count_per_step, ms_per_step):
    """Whole-job bicliques/s: the bicliques all ranks found in one step,
    divided by the slowest rank's step time."""
    return total_count_per_step / (ms_per_step / 1000.0)


def peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def profile_value(workload, key):
    """A figure of dfs_kernel from the committed ncu summary
    (profiles/dfs_kernel_<workload>.md, a line '<key>: N')."""
    p = os.path.join(ROOT, "profiles", f"dfs_kernel_{workload}.md")
    try:
        for line in open(p):
            if line.strip().startswith(key + ":"):
                return float(line.split(":", 1)[1].strip())
    except OSError:
        pass
    return None


def profile_traffic(workload):
    """Per-launch DRAM bytes of dfs_kernel (line 'traffic_bytes_per_launch: N')."""
    return profile_value(workload, "traffic_bytes_per_launch")


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.rows.append(parts)

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if not self.rows:
            return None
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def cpu_baseline(csr, wl, threads, stride_mult=1):
    """The oracle port on the host cores over a stride sample of the roots."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    nr, nc, rp, ci = csr
    stride = wl["cpu_stride"] * stride_mult
    t0 = time.perf_counter()
    r = oracle.ref_enumerate_sampled(nr, nc, rp, ci, stride, threads=threads)
    dt = time.perf_counter() - t0
    return r, dt, stride


def batched_leg(eng, n_graphs=4096):
    """Batched workload: n_graphs graphs (workloads.batch) through
    mbe_batch_run with the engine defaults (chunks launched as a captured
    CUDA graph), the same with the host-driven chunk loop, then autotuned
    (mbe_batch_tune on the same graphs, its wall time reported apart), vs one
    launch pair per graph.  Per-graph counts and hashes must agree between
    all four and with the committed oracle results for the graphs they
    cover."""
    import cumbe_gb300 as cm
    from cumbe_gb300 import workloads
    ps = workloads.batch(n_graphs)
    gs = [cm.Graph.generate(**p) for p in ps]
    for g in gs:
        eng.upload(g)
    eng.batch_tune_reset()
    eng.batch(gs[:64])  # warm-up
    t0 = time.perf_counter()
    res, ms = eng.batch(gs)
    batched_wall = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    res_h, ms_h = eng.batch(gs, host_chunks=True)
    host_wall = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    choices = eng.batch_tune(gs)
    tune_wall = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    res_t, ms_t = eng.batch(gs)
    tuned_wall = (time.perf_counter() - t0) * 1e3
    eng.batch_tune_reset()
    plain_ms = 0.0
    mismatches = 0
    t0 = time.perf_counter()
    for g, r, rt in zip(gs, res, res_t):
        q = eng.enumerate(g)
        plain_ms += q.ms
        mismatches += (q.count, q.hash) != (r.count, r.hash) or (rt.count, rt.hash) != (r.count, r.hash)
    mismatches += sum((rh.count, rh.hash) != (r.count, r.hash) for r, rh in zip(res, res_h))
    plain_wall = (time.perf_counter() - t0) * 1e3
    fix = json.load(open(os.path.join(ROOT, "tests", "golden", "batch_oracle.json")))["graphs"]
    fixture_checked = fixture_mismatches = 0
    for seed, r in enumerate(res_t):
        if str(seed) in fix:
            fixture_checked += 1
            fixture_mismatches += [r.count, f"{r.hash:#018x}"] != fix[str(seed)]
    total = sum(r.count for r in res)
    for g in gs:
        eng.release(g)
    return {"graphs": n_graphs, "bicliques": total, "batched_ms": ms, "tuned_ms": ms_t, "plain_ms": plain_ms,
            "host_chunks_ms": ms_h,
            "batched_wall_ms": batched_wall, "tuned_wall_ms": tuned_wall, "plain_wall_ms": plain_wall,
            "host_chunks_wall_ms": host_wall,
            "tuning_wall_ms": tune_wall,
            "batched_bicliques_per_s": total / (ms / 1e3), "tuned_bicliques_per_s": total / (ms_t / 1e3),
            "plain_bicliques_per_s": total / (plain_ms / 1e3),
            "tune_choices": [{k: (round(v, 3) if isinstance(v, float) else v) for k, v in c.items()} for c in choices],
            "note": "_ms = device time of the enumeration kernels (CUDA events); _wall_ms = host wall clock "
                    "of the whole call(s), graphs resident; batched/tuned: chunks launched as a captured CUDA "
                    "graph (8 per launch); host_chunks: the host-driven chunk loop; tuning = mbe_batch_tune's "
                    "sweep, untimed",
            "per_graph_mismatches": mismatches,
            "oracle_fixture": {"graphs_checked": fixture_checked, "mismatches": fixture_mismatches},
            "workload": "4,096 uniform random graphs, |U| log-uniform [50,5000], |V|=|U|/2, "
                        "density log-uniform [0.002,0.05], seeds 0..4095"}


_SERVED_POOL = None


def served_leg(rate=2000.0, n_requests=8000, seed=11):
    """Poisson request stream against a device-resident pool drawn from the
    four other workloads (workloads.served_pool: the 2,000 x 1,000 graph, the
    94,000 x 30,000 graph, the stress shape at 1/250 and 1/100, the batch
    graphs with |U| <= 1000), each request on a uniformly drawn pool graph,
    half of them thresholded (|A| >= a, |B| >= b, a, b uniform in 1..5).
    Continuous batching (2 slots of 3 DFS blocks per SM, up to 256 requests
    per launch) vs one request per launch on the whole GPU; both arms are
    warmed up (buffers sized for the pool) before the stream starts."""
    global _SERVED_POOL
    import numpy as np
    import cumbe_gb300 as cm
    from cumbe_gb300 import workloads
    if _SERVED_POOL is None:
        spec = workloads.served_pool()
        _SERVED_POOL = ([name for name, _ in spec], [cm.Graph.generate(**p) for _, p in spec])
    names, pool = _SERVED_POOL
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, n_requests)
    picks = rng.integers(0, len(pool), n_requests)
    thr = [(0, 0) if rng.random() < 0.5 else (int(rng.integers(1, 6)), int(rng.integers(1, 6)))
           for _ in range(n_requests)]
    mix = {}
    for k in picks:
        mix[names[k]] = mix.get(names[k], 0) + 1

    def run(slots, max_batch, bpsm):
        srv = cm.Server(0, slots=slots, max_batch=max_batch, blocks_per_sm=bpsm)
        try:
            gids = [srv.add_graph(g) for g in pool]
            srv.warmup()
            t0 = time.perf_counter()
            due = 0.0
            for i in range(n_requests):
                due += gaps[i]
                while time.perf_counter() - t0 < due:
                    pass
                a, b = thr[i]
                srv.submit(gids[picks[i]], a, b)
            out = []
            while len(out) < n_requests:
                out += srv.poll()
                time.sleep(0.001)
            mem = srv.memory()
        finally:
            srv.stop()
        lat = np.array([r["done_s"] - r["submit_s"] for r in out]) * 1e3
        by_req = {r["request"]: r for r in out}
        classes = {}
        for k, rid in enumerate(sorted(by_req)):  # request ids follow submission order
            classes.setdefault(names[picks[k]], []).append(by_req[rid])
        per_class = {name: {"n": len(rs),
                            "p50_ms": float(np.percentile([(r["done_s"] - r["submit_s"]) * 1e3 for r in rs], 50)),
                            "p99_ms": float(np.percentile([(r["done_s"] - r["submit_s"]) * 1e3 for r in rs], 99)),
                            "wait_p99_ms": float(np.percentile([(r["start_s"] - r["submit_s"]) * 1e3 for r in rs], 99)),
                            "service_p50_ms": float(np.percentile([(r["done_s"] - r["start_s"]) * 1e3 for r in rs], 50))}
                     for name, rs in classes.items()}
        span = max(r["done_s"] for r in out) - min(r["submit_s"] for r in out)
        tot = sum(r["count"] for r in out)
        ok = all(r["status"] == 0 for r in out)
        res = {(r["request"]): (r["count"], r["hash"]) for r in out}
        return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "max_ms": float(lat.max()), "requests_per_s": n_requests / span, "bicliques_per_s": tot / span,
                "all_ok": ok, "mean_batch": float(np.mean([r["batch_size"] for r in out])),
                "search_bytes": mem["search_bytes"], "graph_bytes": mem["graph_bytes"], "per_class": per_class}, res

    cont, r1 = run(2, 256, 3)
    plain, r2 = run(1, 1, 0)
    same = [r1[k] for k in sorted(r1)] == [r2[k] for k in sorted(r2)]
    return {"rate_req_per_s": rate, "requests": n_requests, "pool_graphs": len(pool), "request_mix": mix,
            "continuous_batching": cont, "one_request_per_launch": plain,
            "results_identical": same, "mem_budget_bytes": 120 << 30,
            "pool": "workloads.served_pool(): the 2,000 x 1,000 and 94,000 x 30,000 graphs, the stress shape at "
                    "1/250 and 1/100, and the batch graphs with |U| <= 1000"}


# Root sample of the full-size stress graph the bench times: every 10th
# root among the first 411,000 positions of the processing order (degree
# ascending; 457,386 roots have edges, and these reach degree 18).  The hub
# roots beyond carry the graph's explosive part (more than 10^12 maximal
# bicliques in all), which no engine enumerates.
STRESS_SAMPLE = dict(root_begin=0, root_end=411000, root_stride=10)


def stress_leg(eng):
    """The load-imbalance stress graph at its stated size (1.4M x 500k, 8M
    Chung-Lu edges, gamma 1.9 uncapped, 200 planted K_{20,30} blocks at
    density 0.9 over hubs) on a fixed root sample (STRESS_SAMPLE), and its
    shape at 1/50 of the size enumerated in full."""
    import cumbe_gb300 as cm
    from cumbe_gb300 import workloads
    p_full = workloads.SINGLE["power_law_1400k_500k"]
    t0 = time.perf_counter()
    g = cm.Graph.generate(**p_full)
    gen_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    eng.upload(g)  # H2D, transpose, root order on the device
    upload_s = time.perf_counter() - t0
    eng.enumerate(g, root_begin=0, root_end=1000, root_stride=10)  # warm-up
    r = eng.enumerate(g, **STRESS_SAMPLE)
    eng.release(g)
    full = {"workload": "power_law_1400k_500k (stated size)", **p_full, "n_edges_distinct": g.info()["n_edges"],
            "root_sample": STRESS_SAMPLE, "roots_sampled": len(range(0, 411000, 10)),
            "bicliques": r.count, "hash": f"{r.hash:#018x}", "tree_nodes": r.nodes, "ms": r.ms,
            "bicliques_per_s": r.count / (r.ms / 1e3) if r.ms > 0 else None,
            "tree_nodes_per_s": r.nodes / (r.ms / 1e3) if r.ms > 0 else None,
            "generate_s": gen_s, "upload_transpose_s": upload_s}
    p = workloads.stress_params(50)
    gs = cm.Graph.generate(**p)
    eng.enumerate(cm.Graph.generate(**workloads.stress_params(100)))  # warm-up
    rs = eng.enumerate(gs)
    eng.release(gs)
    scaled = {"workload": "stress shape at 1/50 scale, full enumeration", **p, "bicliques": rs.count,
              "hash": f"{rs.hash:#018x}", "ms": rs.ms, "bicliques_per_s": rs.count / (rs.ms / 1e3)}
    return {"full_size_sample": full, "scaled_full": scaled}


def run_reference(args, wl, rank, world):
    """--impl reference: the CPU restatement of the reference's search, on
    a graph built by the oracle's own copy of the generator (this arm never
    loads the product library)."""
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    params = {k: v for k, v in wl.items() if k != "cpu_stride"}
    csr = oracle.generate(**params)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_baseline(csr, wl, threads, stride_mult=10)  # warm caches on a 10x thinner sample
    tot_c, tot_t = 0, 0.0
    for _ in range(args.steps):
        r, dt, stride = cpu_baseline(csr, wl, threads)
        tot_c += r.count
        tot_t += dt
    v = tot_c / tot_t if tot_t > 0 else 0.0
    sample = (f"every {stride}-th root in processing order (stride sample) of the {args.workload} graph, "
              f"{threads} threads")
    line = {"impl": "reference", "metric": "maximal bicliques/sec", "value": v, "unit": "bicliques/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": tot_t * 1000 / max(1, args.steps), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": args.workload, **params, "variant": "cuMBE"},
            "cpu_baseline": {"value": v, "unit": "bicliques/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": "bicliques/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def reference_gpu_leg(eng, workload="power_law_94k_30k_e100k"):
    """The reference's own cuMBE kernel (compiled from its unmodified
    sources into oracle/_ref by oracle/build_ref.py, driven by
    oracle/ref_runner) on one graph, timed as the reference times it: CUDA
    events around its cooperative launch.  This engine runs the same graph
    for the same-config ratio.  None when the reference build is absent."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import re
    import tempfile
    import build_ref
    import cumbe_gb300 as cm
    try:
        built = build_ref.build()
    except Exception as e:  # no CUDA headers / compiler on this host
        return {"unavailable": f"reference runner build failed: {e}"}
    if not built.get("cubin") or not built.get("runner"):
        return {"unavailable": "the reference's kernels were not built here (oracle/_ref/cumbe_ref.cubin missing)"}
    params = {k: v for k, v in WORKLOADS[workload].items() if k != "cpu_stride"}
    g = cm.Graph.generate(**params)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "g.bi")
        g.write_bi(path)
        r = subprocess.run([built["runner"], built["cubin"], path, "cuMBE"], capture_output=True, text=True,
                           timeout=300)
    m = re.search(r"maximal bicliques: (-?\d+)", r.stdout)
    t = re.search(r"runtime \(s\): ([0-9.eE+-]+)", r.stdout)
    if r.returncode != 0 or not m or not t:
        return {"unavailable": f"reference runner failed (rc {r.returncode}): {r.stderr[-300:]}"}
    ref_count, ref_s = int(m.group(1)), float(t.group(1))
    eng.enumerate(g)  # warm-up (upload, transpose)
    mine = eng.enumerate(g)
    eng.release(g)
    return {"workload": workload, **params, "variant": "cuMBE",
            "reference_count": ref_count, "reference_kernel_s": ref_s,
            "reference_bicliques_per_s": ref_count / ref_s if ref_s > 0 else None,
            "engine_count": mine.count, "engine_ms": mine.ms,
            "engine_bicliques_per_s": mine.count / (mine.ms / 1e3) if mine.ms > 0 else None,
            "counts_equal": ref_count == mine.count % (1 << 32) if ref_count >= 0 else None,
            "speedup_kernel_time": ref_s * 1e3 / mine.ms if mine.ms > 0 else None,
            "how": "reference: its kernels compiled from its own sources for sm_103a, launched cooperatively by "
                   "oracle/ref_runner (a restatement of src/main.cu's host steps), event time of the launch; "
                   "engine: root expansion + DFS event time, graph resident"}


# Frozen numerator of the dfs_kernel roofline, per workload: 4 B x the
# 32-bit words of set data that the kernel's node evaluations must read
# (row words of each candidate scanned, L_i words, written child records),
# as the kernel's word counter defined them when these figures were fixed
# (1.2040e10 words per launch on the 293,000-edge graph).  The
# figure is held fixed so that a kernel that skips work shows as a higher
# achieved rate on the same work, never as a smaller numerator.  The
# counter itself is a diagnostic compiled into MBE_COUNT_WORDS=1 builds
# only; when the running build has it, its live figure is reported beside
# the frozen one (null otherwise).
FROZEN_ALGORITHMIC_BYTES = {
    "power_law_94k_30k": 48_160_205_850,
    "power_law_94k_30k_e100k": 711_051_424,
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--variant", default="cuMBE", choices=["cuMBE", "noRS", "noES", "noWS"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--no-stress", action="store_true")
    ap.add_argument("--no-reference-gpu", action="store_true")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    rank, world, local = dist_env()
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        run_reference(args, wl, rank, world)
        return

    import torch
    import cumbe_gb300 as cm
    from cumbe_gb300 import build as b
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    b.build()
    torch.cuda.set_device(local)
    dev = f"cuda:{local}"
    params = {k: v for k, v in wl.items() if k != "cpu_stride"}
    g = cm.Graph.generate(**params)
    info = g.info()
    shard = shard_of(rank, world)
    eng = cm.Engine(local)
    eng.upload(g)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        r0 = eng.enumerate(g, args.variant, **shard)
    # ---- device-resident throughput (value) ----
    c0 = eng.counters()
    sampler = ClockSampler(local)
    sampler.start()
    barrier()
    tot_count, tot_ms, tot_dfs_ms, tot_words = 0, 0.0, 0.0, 0
    results = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        r = eng.enumerate(g, args.variant, **shard)
        results.append(r)
        tot_count += r.count
        tot_ms += r.ms
        tot_dfs_ms += r.ms - r.ms_prep
        tot_words += r.words
    barrier()
    clocks = sampler.stop()
    c1 = eng.counters()
    if any((x.count, x.hash) != (r0.count, r0.hash) for x in results):
        raise SystemExit("enumeration results differ between steps")
    ms_step = max_over_ranks(tot_ms / args.steps, world, dev)
    job_count = sum_over_ranks(r0.count, world, dev)  # every rank's share of one step
    job_hash = sum_over_ranks(r0.hash - (1 << 64) if r0.hash >= (1 << 63) else r0.hash, world, dev) % (1 << 64)
    value = sharded_value(job_count, ms_step)

    # ---- end to end through the C ABI from host buffers (e2e) ----
    e_c0 = eng.counters()
    barrier()
    e2e_wall, e2e_count = 0.0, 0
    for _ in range(args.steps):
        eng.release(g)
        t0 = time.perf_counter()
        r = eng.enumerate(g, args.variant, **shard)  # upload (H2D + transpose) + enumerate + D2H
        e2e_wall += time.perf_counter() - t0
        e2e_count += r.count
    barrier()
    e_c1 = eng.counters()
    e2e_s = max_over_ranks(e2e_wall, world, dev)
    e2e = {"value": sum_over_ranks(e2e_count, world, dev) / e2e_s, "unit": "bicliques/s",
           "h2d_bytes_per_step": (e_c1["h2d"] - e_c0["h2d"]) // args.steps,
           "d2h_bytes_per_step": (e_c1["d2h"] - e_c0["d2h"]) // args.steps}

    # ---- roofline of the dominant kernel (dfs_kernel) ----
    peak, peak_kind = peak_hbm()
    launch_ms = tot_dfs_ms / args.steps
    live_bytes = tot_words * 4 // args.steps if tot_words else None  # None: counter compiled out
    frozen = FROZEN_ALGORITHMIC_BYTES.get(args.workload) if world == 1 else None
    alg_bytes = frozen if frozen is not None else live_bytes
    achieved = alg_bytes / (launch_ms / 1000.0) / 1e9 if alg_bytes is not None and launch_ms > 0 else None
    traffic = profile_traffic(args.workload)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak if achieved is not None else None,
                "traffic": traffic, "peak_source": peak_kind, "kernel": "dfs_kernel",
                "algorithmic_bytes_per_launch": alg_bytes,
                "numerator": "frozen per workload" if frozen is not None else (
                    "live kernel word counter" if live_bytes is not None else "none (counter compiled out)"),
                "live_counter_bytes_per_launch": live_bytes,
                "launch_ms": launch_ms,
                "dram_bytes_per_launch_ncu": traffic,
                # from the committed ncu summaries: the kernel is L1/L2- and latency-bound
                "l2_hit_rate": profile_value(args.workload, "l2_hit_rate"),
                "int_pipe_active": profile_value(args.workload, "int_pipe_active")}

    line = {"metric": "maximal bicliques/sec", "value": value, "unit": "bicliques/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "strong" if world > 1 else "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic",
            "config": {"workload": args.workload, **params, "variant": args.variant,
                       "l2": "flushed before every timed step (512 MiB write)",
                       "parallelism": (f"roots sharded round-robin over {world} ranks (positions r, r+{world}, ...)"
                                       if world > 1 else "single GPU"),
                       "bicliques_per_step": job_count, "hash": f"{job_hash:#018x}",
                       "tree_nodes_per_step": r0.nodes, "n_edges": info["n_edges"]},
            "e2e": e2e, "roofline": roofline,
            "gpu_launches": c1["launches"] - c0["launches"],
            "clocks": clocks}
    if rank == 0 and world == 1 and not args.no_reference_gpu:
        line["reference_gpu"] = reference_gpu_leg(eng)
    if rank == 0 and not args.no_batched:
        line["batched"] = batched_leg(eng)
    if rank == 0 and not args.no_served:
        line["served"] = served_leg()
        # saturating load: arrivals faster than one request per launch can serve
        line["served_saturated"] = served_leg(rate=20000.0, n_requests=20000, seed=12)
    if rank == 0 and not args.no_stress:
        line["stress"] = stress_leg(eng)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rc, dt, stride = cpu_baseline(g.csr(), wl, threads)
        line["cpu_baseline"] = {"value": rc.count / dt if dt > 0 else 0.0, "unit": "bicliques/s", "cores": threads,
                                "kind": "port",
                                "sample": f"every {stride}-th root (stride sample) of the same graph: "
                                          f"{rc.count} bicliques in {dt:.2f} s"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    eng.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
