"""Oracle parity at the benchmarked scale.

* The benchmark's own batch: 2,000,000 sequences (seed 42, 12 amino-acid genes, metadata), 2,048
  queries (seed 43, nucleotide, amino-acid and metadata leaves), every fourth a Mutations query of
  the nucleotide column. It runs through rhy_batch_rows, the call the end-to-end number times, and
  every count is compared with the oracle's, as are the Mutations rows (minimum proportion 0.05)
  and the dense count tables of 64 Mutations queries.
* The at-scale plain configuration: 2,000 further seeded queries on the same table through the
  single-query path, every count against the oracle, plus Mutations tables of 48 of them over
  columns drawn from all 13 sequence columns.
* The small plain configuration: all 1,000 trees of depth <= 4 over 100,000 sequences, each with
  its Count and its Mutations table and rows, against the oracle.
The oracle evaluates many queries at once on all host cores (Oracle.check_batch)."""
import numpy as np
import pytest

import rhydb_gpu as R
from rawtable import oracle_for

pytestmark = pytest.mark.gpu

MIN_PROPORTION = 0.05


def _rows_tuple(rows):
    return [(int(r["position"]), r["from_"].decode(), r["to"].decode(), int(r["count"]), int(r["coverage"]),
             float(r["proportion"])) for r in rows]


@pytest.fixture(scope="module")
def bench_table():
    t = R.Table.generate(2_000_000, seed=42, n_aa_genes=12)
    orc = oracle_for(t)
    dev = R.Device(t, 0)
    yield t, orc, dev
    dev.close()


def test_benchmark_batch_against_the_oracle(bench_table):
    t, orc, dev = bench_table
    qs = t.queries(2048, seed=43, use_aa=True, use_metadata=True)
    acts = np.array([1 if i % 4 == 3 else 0 for i in range(len(qs))], np.int32)
    cols = np.zeros(len(qs), np.uint32)
    mut_idx = [int(i) for i in np.flatnonzero(acts)][:64]
    o_counts, o_tables = orc.check_batch(qs, cols, tables=mut_idx)
    counts, rows, begin, cnt = dev.batch_rows(qs, acts, cols, np.full(len(qs), MIN_PROPORTION))
    assert np.array_equal(np.asarray(counts, np.uint64), o_counts)
    # the rows the device built equal the oracle's addMutationsToOutput of the oracle's counts
    for i in mut_idx:
        got = _rows_tuple(rows[int(begin[i]):int(begin[i]) + int(cnt[i])])
        assert got == orc.mutation_rows(0, o_tables[i], MIN_PROPORTION), qs[i]
    # the dense count tables of the same batch
    d_counts, muts = dev.batch(qs, acts, cols)
    assert np.array_equal(np.asarray(d_counts, np.uint64), o_counts)
    for i in mut_idx:
        assert np.array_equal(muts[i], o_tables[i]), qs[i]
    # the spread of the checked filters: empty, sparse (row-index pass) and dense ones
    sel = o_counts[mut_idx].astype(np.float64) / t.n_rows
    assert (sel == 0).any() and ((sel > 0) & (sel <= 1 / 64)).any() and (sel > 1 / 64).any()


def test_at_scale_plain_queries_against_the_oracle(bench_table):
    t, orc, dev = bench_table
    qs = t.queries(2000, seed=44, use_aa=True, use_metadata=True)
    rng = np.random.default_rng(45)
    mut_idx = sorted(rng.choice(len(qs), 48, replace=False).tolist())
    cols = np.zeros(len(qs), np.uint32)
    cols[mut_idx] = rng.integers(0, t.n_seq, len(mut_idx))
    o_counts, o_tables = orc.check_batch(qs, cols, tables=mut_idx)
    got = np.array([dev.count(q) for q in qs], np.uint64)
    assert np.array_equal(got, o_counts)
    for i in mut_idx:
        m, n = dev.mutations(qs[i], int(cols[i]))
        assert n == o_counts[i] and np.array_equal(m, o_tables[i]), (qs[i], cols[i])


def test_config1_all_trees_count_and_mutations():
    t = R.Table.generate(100000, seed=42)
    orc = oracle_for(t)
    dev = R.Device(t, 0)
    qs = t.queries(1000, seed=43, max_depth=4, max_nof_children=8)
    for lo in range(0, len(qs), 250):  # 250 tables (1.9 MB each) at a time
        part = qs[lo:lo + 250]
        o_counts, o_tables = orc.check_batch(part, tables=range(len(part)))
        for i, q in enumerate(part):
            assert dev.count(q) == o_counts[i], q
            m, n = dev.mutations(q, 0)
            assert n == o_counts[i] and np.array_equal(m, o_tables[i]), q
            assert t.mutation_rows(0, m, MIN_PROPORTION) == orc.mutation_rows(0, o_tables[i], MIN_PROPORTION), q
    dev.close()
