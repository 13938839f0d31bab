"""Random filter expressions on small seeded tables: the CPU oracle against the independent
row-by-row semantics of tests/semantic.py."""
import numpy as np
import pytest

import rhydb_gpu as R
import semantic
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
