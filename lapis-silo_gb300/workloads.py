"""Named synthetic query workloads built on the seeded generator (Table.queries).

batching_workload: the batching shape — thousands of filter trees of 1 to 64 leaves with NOf of up
to 64 children, whose selectivities spread log-uniformly over [1e-5, 0.9]. The generator does not
aim at a selectivity, so a larger seeded candidate set is drawn, every candidate is counted on the
device, and the batch takes, for targets evenly spaced in log(selectivity), the unused candidate
nearest to each target.

profile_query_sequence: a MutationProfile query sequence near the data, one row's own aligned
sequence with a few seeded substitutions (the shape of the reference's nof_sequence_filter
benchmark, whose profile is an evolved sequence).
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


def profile_query_sequence(table, row: int = 123457, substitutions: int = 20, seed: int = 17,
                           column: int = 0) -> str:
    """Row `row`'s aligned sequence in sequence column `column` (its runs over the reference),
    with `substitutions` seeded positions set to a random A/C/G/T."""
    raw = table.raw()
    s = raw.seq[column]
    row = row % table.n_rows
    seq = bytearray(s.reference[: s.L])
    for k in range(s.row_off[row], s.row_off[row + 1]):
        seq[s.run_pos[k]: s.run_pos[k] + s.run_len[k]] = s.run_char[k] * s.run_len[k]
    rng = np.random.default_rng(seed)
    for p in rng.choice(s.L, substitutions, replace=False):
        seq[p] = ord("ACGT"[rng.integers(4)])
    return seq.decode()
