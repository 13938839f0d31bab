"""Ingestion on the GPU (rhy_table_from_raw_gpu) builds the same table as host ingestion: every
sequence column's storage image is identical (checksum over all of its arrays), on generated
tables and on the storage scenarios of the reference's tests (missing reference symbols, flips
and ties of the local reference, coverage across chunks), and a GPU-built table answers queries
as the oracle does."""
import numpy as np
import pytest

import rhydb_gpu as R
from golden import storage_cases as G
from rawtable import RawBuilder, oracle_for

pytestmark = pytest.mark.gpu


def same_image(raw):
    host = R.Table.from_raw(raw)
    gpu = R.Table.from_raw_gpu(raw, 0)
    assert host.n_rows == gpu.n_rows and host.n_seq == gpu.n_seq
    for c in range(host.n_seq):
        assert host.local_reference(c) == gpu.local_reference(c), c
        assert host.checksum(c) == gpu.checksum(c), c
    return host, gpu


@pytest.mark.parametrize("rows,kw", [
    (70000, dict(seed=5, genome_len=4000, pool_sites=300, n_aa_genes=2, null_fraction=0.01)),
    (140000, dict(seed=11, genome_len=29903, n_aa_genes=12, null_fraction=0.003)),
    (1, dict(seed=3, genome_len=500, pool_sites=40)),
    (65537, dict(seed=4, genome_len=1000, pool_sites=100, null_fraction=0.2)),
])
def test_generated_tables(rows, kw):
    t = R.Table.generate(rows, **kw)
    same_image(t.raw())


def test_gpu_built_table_answers_like_the_oracle():
    t = R.Table.generate(100000, seed=8, genome_len=6000, pool_sites=500, n_aa_genes=2, null_fraction=0.01)
    raw = t.raw()
    _, gpu = same_image(raw)
    orc = oracle_for(gpu, raw)
    dev = R.Device(gpu, 0)
    # query texts come from the generated table: the GPU-built one holds the same rows
    for q in t.queries(60, seed=9, use_aa=True, use_metadata=True):
        bits, n = dev.compute_filter(q)
        obits, on = orc.compute_filter(q)
        assert n == on and np.array_equal(bits, obits), q
    for q in t.queries(8, seed=10):
        m, n = dev.mutations(q, 0)
        om, on = orc.mutations(q, 0)
        assert n == on and np.array_equal(m, om), q
    dev.close()


def _placed(fragment, offset, L, kind=0):
    m = "N" if kind == 0 else "X"
    return m * offset + fragment + m * (L - offset - len(fragment))


def test_storage_scenarios():
    # aligned sequences (missing reference symbols, gaps, lower case, amino acids) next to rows
    # holding the reference
    for case in G.ALIGNED:
        if len(case) != 9:
            continue
        _, kind, frag, offset, ref, *_ = case
        b = RawBuilder(3)
        b.add_sequences("main", kind, ref, [_placed(frag, offset, len(ref), kind), ref, ref])
        same_image(b.raw())
    # local-reference adaptation, ties included
    for _, rows, ref, _, _ in G.ADAPTATION:
        b = RawBuilder(len(rows))
        b.add_sequences("main", 0, ref, list(rows))
        same_image(b.raw())
    # coverage scenarios with null rows
    for _, rows, _ in G.COVERAGE:
        L = len(G.COVERAGE_REFERENCE)
        b = RawBuilder(len(rows))
        b.add_sequences("main", 0, G.COVERAGE_REFERENCE, [None if r is None else _placed(r[0], r[1], L) for r in rows])
        same_image(b.raw())
    # rows at the starts of three chunks, null rows between them
    _, placed_rows = G.COVERAGE_CHUNKS
    n = max(placed_rows) + 1
    L = len(G.COVERAGE_REFERENCE)
    b = RawBuilder(n)
    b.add_sequences("main", 0, G.COVERAGE_REFERENCE,
                    [_placed(*placed_rows[i], L) if i in placed_rows else None for i in range(n)])
    same_image(b.raw())
    # stored symbols of every nucleotide and amino-acid symbol, and 70,000 rows at two positions
    for _, kind, ref, rows in G.STORED_SYMBOLS:
        b = RawBuilder(len(rows))
        b.add_sequences("main", kind, ref, rows)
        same_image(b.raw())


def test_illegal_character_is_rejected():
    b = RawBuilder(2)
    b.add_sequences("main", 0, "ACGT", ["ACGT", "ACQT"])
    with pytest.raises(R.RhyError) as e:
        R.Table.from_raw_gpu(b.raw(), 0)
    assert e.value.code == 4 and "illegal character 'Q' at position 2" in str(e.value)
