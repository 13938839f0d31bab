"""Random filter expressions on small seeded tables: the CPU oracle against the independent
row-by-row semantics of tests/semantic.py."""
import numpy as np
import pytest

import rhydb_gpu as R
import semantic
import oracle as oracle_mod
from rawtable import oracle_for


@pytest.fixture(scope="module", params=[(1, 3000, 0.0), (2, 5000, 0.01), (3, 70000, 0.002)], ids=lambda p: f"seed{p[0]}")
def small(request):
    seed, rows, nulls = request.param
    t = R.Table.generate(rows, seed=seed, genome_len=600, pool_sites=120, n_aa_genes=2, null_fraction=nulls)
    raw = t.raw()
    return t, oracle_for(t, raw), semantic.from_raw(raw)


def _rows(bits, n):
    return R.bits_to_rows(bits)


def test_oracle_matches_semantics(small):
    t, orc, sem = small
    queries = t.queries(150, seed=5, use_aa=True, use_metadata=True)
    # chunk-aware row ids: global id = chunk << 16 | row, rows are consecutive per chunk
    n = t.n_rows
    gid = np.array([(i >> 16) << 16 | (i & 0xFFFF) for i in range(n)], np.uint32)
    for q in queries:
        expect = gid[sem.evaluate(q)]
        bits, cnt = orc.compute_filter(q)
        got = R.bits_to_rows(bits)
        assert cnt == len(expect), q
        assert np.array_equal(got, expect), q


def test_handwritten_edge_queries(small):
    t, orc, sem = small
    qs = [
        "SymEq(main,1,N)", "SymEq(main,600,N)", "SymEq(main,1,.)", "HasMut(main,300)", "Maybe(HasMut(main,300))",
        "Exact(SymEq(main,5,R))", "Maybe(SymEq(main,5,R))", "Not(SymEq(main,10,-))", "Maybe(Not(SymEq(main,10,A)))",
        "Maybe(NOf(1,exactly,SymEq(main,5,A),SymEq(main,6,C),SymEq(main,7,G)))",
        "Exact(NOf(2,exactly,Not(SymEq(main,5,A)),SymEq(main,6,N),HasMut(main,7)))",
        "NOf(-1,exactly,SymEq(main,5,A))", "NOf(-1,atleast,SymEq(main,5,A))", "NOf(3,atleast,SymEq(main,5,A))",
        "Or(SymEq(main,5,A),SymEq(main,5,C),SymEq(main,5,N))", "Or(SymEq(main,5,.),SymEq(main,5,N))",
        "And()", "Or()", "And(True,False)", "Or(False,Not(True))", "NOf(0,exactly)", "NOf(0,atleast)",
        "Or(SymEq(ORF1a,3,X),SymEq(ORF1a,3,.))", "HasMut(ORF1b,50)", "Maybe(SymEq(ORF1b,50,B))",
        "And(DateBetween(date,*,*),Not(StrEq(country,country_000)))",
        "NOf(2,atleast,DateBetween(date,18300,18700),StrEq(lineage,lineage_0001),SymEq(main,20,-),Not(HasMut(main,2)))",
    ]
    n = t.n_rows
    gid = np.array([(i >> 16) << 16 | (i & 0xFFFF) for i in range(n)], np.uint32)
    for q in qs:
        expect = gid[sem.evaluate(q)]
        bits, cnt = orc.compute_filter(q)
        assert np.array_equal(R.bits_to_rows(bits), expect), q


def test_mutation_profile(small):
    t, orc, sem = small
    n = t.n_rows
    gid = np.array([(i >> 16) << 16 | (i & 0xFFFF) for i in range(n)], np.uint32)
    for q in semantic.profile_queries(sem, np.random.default_rng(3)):
        expect = gid[sem.evaluate(q)]
        bits, cnt = orc.compute_filter(q)
        assert cnt == len(expect) and np.array_equal(R.bits_to_rows(bits), expect), q[:80]


def test_mutation_profile_sequence_id():
    """MutProfileSequenceId: the profile is the aligned sequence of the first row holding the
    primary key (all missing for a row without a sequence); the oracle against the row-level
    semantics, and the product's compile step (plan) for its error cases."""
    from rawtable import accession_table

    b, raw, acc = accession_table()
    t = R.Table.from_raw(raw)
    orc = oracle_mod.Oracle(raw, t.n_chunks, [(c.name, c.n_symbols, c.L) for c in t.columns])
    sem = semantic.from_raw(raw)
    col = sem.cols["main"]
    L = len(col.reference)
    with pytest.raises(R.RhyError):
        t.plan("MutProfileSequenceId(main,1,seq_0003)")  # no primary key yet
    t.set_primary_key("accession")
    orc.set_primary_key("accession")
    gid = np.arange(t.n_rows, dtype=np.uint32)
    for key in ("seq_0003", "shared_a", "shared_b", "null_row", "seq_0299"):
        row = acc.index(key)
        seq = "N" * L if col.null[row] else "".join(col.alpha[x] for x in col.sym[row])
        for d in (0, 1, 3, 10):
            q = f"MutProfileSequenceId(main,{d},{key})"
            expect = gid[sem.evaluate(f"MutProfile(main,{d},{seq})")]
            bits, cnt = orc.compute_filter(q)
            assert cnt == len(expect) and np.array_equal(R.bits_to_rows(bits), expect), q
            tree, _, _ = t.plan(q)
            assert "Profile" in tree
    for bad in ("MutProfileSequenceId(main,1,nosuch)", "MutProfileSequenceId(main,-1,seq_0003)",
                "MutProfileSequenceId(nosuch,1,seq_0003)"):
        with pytest.raises(R.RhyError):
            t.plan(bad)
    with pytest.raises(R.RhyError):
        t.set_primary_key("nosuch")
