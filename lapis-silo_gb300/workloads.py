"""Named synthetic query workloads built on the seeded generator (Table.queries).

batching_workload: the batching shape — thousands of filter trees of 1 to 64 leaves with NOf of up
to 64 children, whose selectivities spread log-uniformly over [1e-5, 0.9]. The generator does not
aim at a selectivity, so a larger seeded candidate set is drawn, every candidate is counted on the
device, and the batch takes, for targets evenly spaced in log(selectivity), the unused candidate
nearest to each target.
"""
from __future__ import annotations

import numpy as np


def log_uniform_pick(counts, n_rows: int, n: int, lo: float = 1e-5, hi: float = 0.9) -> np.ndarray:
    """Indices of n candidates whose selectivities (counts / n_rows) spread log-uniformly over
    [lo, hi]: target k sits at lo * (hi / lo) ** ((k + 0.5) / n) and takes the nearest candidate not
    taken yet. Raises if fewer than n candidates lie in the range."""
    sel = np.asarray(counts, dtype=np.float64) / float(n_rows)
    cand = np.flatnonzero((sel >= lo) & (sel <= hi))
    if len(cand) < n:
        raise ValueError(f"{len(cand)} candidates in [{lo}, {hi}], {n} needed")
    order = cand[np.argsort(np.log(sel[cand]), kind="stable")]
    ls = np.log(sel[order])
    targets = np.log(lo) + (np.arange(n) + 0.5) / n * (np.log(hi) - np.log(lo))
    taken = np.zeros(len(order), bool)
    out = np.empty(n, np.int64)
    for k, x in enumerate(targets):
        j = int(np.searchsorted(ls, x))
        a, b = j - 1, j  # nearest untaken on either side
        while a >= 0 and taken[a]:
            a -= 1
        while b < len(order) and taken[b]:
            b += 1
        if b >= len(order) or (a >= 0 and x - ls[a] <= ls[b] - x):
            j = a
        else:
            j = b
        taken[j] = True
        out[k] = order[j]
    return out


def batching_workload(table, device, n: int = 4096, seed: int = 44, candidates: int = 40000,
                      use_aa: bool = True, use_metadata: bool = True) -> list[str]:
    """n expressions of 1..64 leaves (NOf up to 64 children) with log-uniform selectivities in
    [1e-5, 0.9], chosen from `candidates` seeded trees counted on `device`."""
    qs = table.queries(candidates, seed=seed, max_depth=4, max_nof_children=64, max_leaves=64, use_aa=use_aa,
                       use_metadata=use_metadata)
    counts, _ = device.batch(qs)
    return [qs[i] for i in log_uniform_pick(counts, table.n_rows, n)]
