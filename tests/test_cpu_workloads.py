"""The seeded workload helpers: leaf-limited trees, the log-uniform selectivity pick and the
MutationProfile query sequence."""
import re

import numpy as np
import pytest

import rhydb_gpu as R
import workloads


def test_leaf_limit_and_unlimited_stream():
    t = R.Table.generate(2000, seed=3, genome_len=800, pool_sites=100, n_aa_genes=2)
    qs = t.queries(2000, seed=44, max_depth=4, max_nof_children=64, max_leaves=64, use_aa=True, use_metadata=True)
    n = np.array([len(re.findall(r"SymEq|HasMut|StrEq|DateBetween", q)) for q in qs])
    assert n.min() >= 1 and n.max() == 64
    for q in qs[:200]:
        t.plan(q)  # every generated tree parses and compiles
    # without a limit the stream is the generator's usual one: a limit that never binds changes nothing
    a = t.queries(300, seed=5, max_depth=3, max_nof_children=4)
    b = t.queries(300, seed=5, max_depth=3, max_nof_children=4, max_leaves=10 ** 6)
    assert a == b


def test_log_uniform_pick():
    rng = np.random.default_rng(1)
    rows = 1_000_000
    counts = np.floor(10 ** rng.uniform(-7, 0, 50000) * rows).astype(np.int64)
    idx = workloads.log_uniform_pick(counts, rows, 2000)
    assert len(set(idx.tolist())) == 2000
    sel = counts[idx] / rows
    assert sel.min() >= 1e-5 and sel.max() <= 0.9
    per_decade = np.histogram(np.log10(sel), bins=[-5, -4, -3, -2, -1, np.log10(0.9)])[0]
    assert per_decade.min() > 300 and per_decade.max() < 500, per_decade
    with pytest.raises(ValueError):
        workloads.log_uniform_pick(counts[:10], rows, 2000)


def test_profile_query_sequence():
    """The benchmark's MutationProfile query sequence is the row's aligned sequence (its runs over the
    reference), with exactly the seeded substitutions changed."""
    import semantic

    t = R.Table.generate(3000, seed=4, genome_len=600, pool_sites=120, n_aa_genes=0, null_fraction=0.0)
    col = semantic.from_raw(t.raw()).cols["main"]
    for row in (0, 1234, 2999):
        own = "".join(col.alpha[x] for x in col.sym[row])
        assert workloads.profile_query_sequence(t, row=row, substitutions=0) == own
        changed = workloads.profile_query_sequence(t, row=row, substitutions=7, seed=3)
        assert len(changed) == len(own) and sum(a != b for a, b in zip(own, changed)) <= 7
