"""Synthetic workloads (seeded; the reference's KONECT datasets need network).

  power_law_2k_1k      2,000 x 1,000 rows x cols, 10,000 edges, Chung-Lu
                       gamma 2.1 on both sides, seed 1.
  power_law_94k_30k    94,000 x 30,000, 293,000 edges, gammas 2.0 / 2.3,
                       degree cap 7,500, seed 2 (the headline workload).
  power_law_1400k_500k 1.4M x 500k, 8M edges, gamma 1.9, plus 200 planted
                       K_{20,30} blocks at density 0.9 over hubs (stress).
  stress_params(k)     the stress shape at 1/k of its size.
  served_pool()        the served workload's pool (from the four above).
  batch_4096           4,096 independent uniform random bipartite graphs,
                       graph s: |U| log-uniform in [50, 5000], |V| = |U|/2,
                       density log-uniform in [0.002, 0.05], parameters
                       drawn with numpy's PCG64 seeded by s, edges by the
                       library generator seeded by s.
"""
from __future__ import annotations

import math

import numpy as np

SINGLE = {
    "power_law_2k_1k": dict(n_rows=2000, n_cols=1000, n_edges=10000, gamma_rows=2.1, gamma_cols=2.1, max_deg=0,
                            seed=1),
    "power_law_94k_30k": dict(n_rows=94000, n_cols=30000, n_edges=293000, gamma_rows=2.0, gamma_cols=2.3,
                              max_deg=7500, seed=2),
    "power_law_94k_30k_e100k": dict(n_rows=94000, n_cols=30000, n_edges=100000, gamma_rows=2.0, gamma_cols=2.3,
                                    max_deg=7500, seed=2),
    "power_law_1400k_500k": dict(n_rows=1400000, n_cols=500000, n_edges=8000000, gamma_rows=1.9, gamma_cols=1.9,
                                 max_deg=0, seed=3, planted=200, planted_rows=20, planted_cols=30,
                                 planted_density=0.9),
}


def stress_params(scale: int) -> dict:
    """The load-imbalance stress graph's shape (power_law_1400k_500k) at
    1/scale of its size: sides and edges divided by scale, 200/scale
    planted K_{20,30} blocks (at least one)."""
    full = SINGLE["power_law_1400k_500k"]
    return dict(full, n_rows=full["n_rows"] // scale, n_cols=full["n_cols"] // scale,
                n_edges=full["n_edges"] // scale, planted=max(1, round(full["planted"] / scale)))


def served_pool() -> list[tuple[str, dict]]:
    """The served workload's graph pool, drawn from the four other
    workloads: the 2,000 x 1,000 graph, the 94,000 x 30,000 graph, the
    stress shape at 1/250 and 1/100 of its size, and the batch graphs with
    |U| <= 1000 (the larger batch graphs are left out so that 2,000
    requests/s stay within what one GPU serves)."""
    pool = [("power_law_2k_1k", SINGLE["power_law_2k_1k"]),
            ("power_law_94k_30k", SINGLE["power_law_94k_30k"]),
            ("stress_1_250", stress_params(250)),
            ("stress_1_100", stress_params(100))]
    pool += [("batch", p) for p in batch(4096) if p["n_rows"] <= 1000]
    return pool


def batch_params(seed: int) -> dict:
    """Generator parameters of graph `seed` of the batched workload."""
    rng = np.random.default_rng(seed)
    u = int(round(math.exp(rng.uniform(math.log(50), math.log(5000)))))
    v = max(1, u // 2)
    dens = math.exp(rng.uniform(math.log(0.002), math.log(0.05)))
    e = max(1, int(round(dens * u * v)))
    return dict(n_rows=u, n_cols=v, n_edges=e, gamma_rows=0.0, gamma_cols=0.0, max_deg=0, seed=seed)


def batch(n: int = 4096, first_seed: int = 0) -> list[dict]:
    return [batch_params(s) for s in range(first_seed, first_seed + n)]
