"""Serving (mbe_server_*): continuous batching over device-resident graphs.
Each request's count and hash are the same alone and in the mix."""
import time

import numpy as np
import pytest

import cumbe_gb300 as cm
from cumbe_gb300 import workloads

pytestmark = pytest.mark.gpu


def _drain(srv, n, timeout=120.0):
    out = []
    t0 = time.time()
    while len(out) < n:
        out += srv.poll()
        if time.time() - t0 > timeout:
            raise TimeoutError(f"{len(out)}/{n} requests finished")
        time.sleep(0.002)
    return out


@pytest.mark.parametrize("slots,max_batch", [(2, 256), (1, 1), (3, 8)])
def test_results_same_alone_and_in_the_mix(engine, slots, max_batch):
    rng = np.random.default_rng(17)
    graphs = [cm.Graph.generate(**workloads.batch_params(s)) for s in range(24)
              if workloads.batch_params(s)["n_rows"] <= 1500]
    graphs.append(cm.Graph.generate(**workloads.SINGLE["power_law_2k_1k"]))
    srv = cm.Server(0, slots=slots, max_batch=max_batch)
    try:
        gids = [srv.add_graph(g) for g in graphs]
        reqs = []
        for _ in range(150):
            k = int(rng.integers(len(gids)))
            a, b = (0, 0) if rng.random() < 0.5 else (int(rng.integers(1, 6)), int(rng.integers(1, 6)))
            reqs.append((srv.submit(gids[k], a, b), k, a, b))
            if rng.random() < 0.3:
                time.sleep(0.0005)
        res = {r["request"]: r for r in _drain(srv, len(reqs))}
    finally:
        srv.stop()
    alone = {}
    for rid, k, a, b in reqs:
        if (k, a, b) not in alone:
            r = engine.enumerate(graphs[k], min_rows=a, min_cols=b)
            alone[(k, a, b)] = (r.count, r.hash)
        got = res[rid]
        assert got["status"] == 0
        assert (got["count"], got["hash"]) == alone[(k, a, b)], (k, a, b)
        assert got["done_s"] >= got["start_s"] >= got["submit_s"]
    if max_batch > 1:
        assert max(r["batch_size"] for r in res.values()) > 1  # requests were batched


def test_memory_budget_bounds_what_the_server_holds(engine):
    """mem_budget is divided among the slots up front; after warm-up and a
    stream of requests (the 2,000 x 1,000 graph and batch graphs) the slots'
    device buffers stay within it, and every result is still exact."""
    rng = np.random.default_rng(5)
    graphs = [cm.Graph.generate(**workloads.batch_params(s)) for s in range(40)
              if workloads.batch_params(s)["n_rows"] <= 2000]
    graphs.append(cm.Graph.generate(**workloads.SINGLE["power_law_2k_1k"]))
    budget = 3 << 30
    srv = cm.Server(0, slots=2, max_batch=64, mem_budget=budget)
    try:
        gids = [srv.add_graph(g) for g in graphs]
        srv.warmup()
        warm = srv.memory()
        assert warm["slot_cap"] == budget // 2
        assert 0 < warm["search_bytes"] <= budget
        reqs = []
        for _ in range(80):
            k = int(rng.integers(len(gids)))
            reqs.append((srv.submit(gids[k]), k))
        res = {r["request"]: r for r in _drain(srv, len(reqs))}
        after = srv.memory()
    finally:
        srv.stop()
    assert after["search_bytes"] <= budget
    assert after["graph_bytes"] > 0
    for rid, k in reqs:
        want = engine.enumerate(graphs[k])
        assert res[rid]["status"] == 0
        assert (res[rid]["count"], res[rid]["hash"]) == (want.count, want.hash)


def test_heavy_requests_run_alone_on_slot_0(engine):
    """With heavy_bytes below the 2,000 x 1,000 graph's estimate (~5.9 MB)
    its requests count as heavy: they run on slot 0 only, one per launch,
    while the light batch graphs keep being served and batched."""
    rng = np.random.default_rng(9)
    light = [cm.Graph.generate(**workloads.batch_params(s)) for s in range(12)
             if workloads.batch_params(s)["n_rows"] <= 800]
    heavy = cm.Graph.generate(**workloads.SINGLE["power_law_2k_1k"])
    graphs = light + [heavy]
    srv = cm.Server(0, slots=3, max_batch=64, heavy_bytes=1 << 20)
    try:
        gids = [srv.add_graph(g) for g in graphs]
        assert srv.estimate(gids[-1]) > (1 << 20) >= max(srv.estimate(g) for g in gids[:-1])
        reqs = []
        for i in range(120):
            k = len(graphs) - 1 if i % 10 == 0 else int(rng.integers(len(light)))
            reqs.append((srv.submit(gids[k]), k))
        res = {r["request"]: r for r in _drain(srv, len(reqs))}
    finally:
        srv.stop()
    for rid, k in reqs:
        r = res[rid]
        want = engine.enumerate(graphs[k])
        assert r["status"] == 0 and (r["count"], r["hash"]) == (want.count, want.hash)
        if k == len(graphs) - 1:
            assert r["slot"] == 0 and r["batch_size"] == 1
