"""The plan of the Mutations container pass on the CPU (rhy_container_pass_plan): the array units
tile every chunk's array payloads exactly once on 16-byte boundaries, each with the descriptors of
the arrays it overlaps; every bitset and run container has its own unit; and the CTA ranges cut the
units in order into pieces of at most two chunks, one wave of CTAs where the table allows it."""
import numpy as np
import pytest

import rhydb_gpu as R


def _chunk_arrays(table, column):
    """Per chunk: the storage indexes, cardinalities and types of its containers."""
    pos, chunk, sym, card, typ = table.containers(column)
    out = {}
    for v in np.unique(chunk):
        idx = np.flatnonzero(chunk == v)
        out[int(v)] = (idx, card[idx].astype(np.int64), typ[idx])
    return out


def _check_plan(table, column, ctas):
    au, ou, rg = table.container_pass_plan(column, ctas)
    chunks = _chunk_arrays(table, column)
    n_chunks = table.n_chunks
    # ---- array units: per chunk, consecutive pieces covering [base, A1) once
    for v, (idx, card, typ) in chunks.items():
        arr = idx[typ == 0]
        units = au[au[:, 4] == v]
        if len(arr) == 0:
            assert len(units) == 0
            continue
        acard = card[typ == 0]
        base = int(units[0, 0])
        assert base % 8 == 0
        start = base + np.concatenate([[0], np.cumsum(acard)[:-1]])
        end = start + acard
        e = base
        for e0, n, c0, nd, _ in units.astype(np.int64):
            assert e0 == e and e0 % 8 == 0 and 1 <= n <= 1024, (v, e0, e)
            overlap = arr[(start < e0 + n) & (end > e0)]
            assert len(overlap) > 0
            assert c0 <= overlap.min() and overlap.max() < c0 + nd, (v, e0)
            assert c0 == overlap.min() and c0 + nd - 1 == overlap.max()  # no descriptor beyond them
            assert nd <= 64 or n == 8
            e = e0 + n
        assert e == end[-1]
        # ---- bitset and run units: one per container, after the arrays, 16-byte aligned
        others = ou[ou[:, 1] == v]
        want = idx[typ != 0]
        assert np.array_equal(others[:, 3], want)
        assert np.array_equal(others[:, 0], typ[typ != 0])
        bits = others[others[:, 0] == 1]
        assert np.all(bits[:, 2] % 8 == 0) and np.all(bits[:, 2] >= end[-1])
    assert sorted(set(au[:, 4].tolist()) | set(ou[:, 1].tolist())) == sorted(chunks)
    # ---- ranges: an ordered partition of both unit lists, each within two chunks
    assert len(rg) > 0
    assert rg[0, 0] == 0 and rg[0, 2] == 0
    assert rg[-1, 1] == len(au) and rg[-1, 3] == len(ou)
    for r, s in zip(rg[:-1], rg[1:]):
        assert r[1] == s[0] and r[3] == s[2]
    for a0, a1, o0, o1, v0, v1 in rg.astype(np.int64):
        assert a1 > a0 or o1 > o0
        assert v0 <= v1
        assert set(au[a0:a1, 4].tolist()) | set(ou[o0:o1, 1].tolist()) <= {v0, v1}
    if n_chunks <= 2 * ctas:
        assert len(rg) <= ctas  # one wave
    else:
        assert len(rg) >= (n_chunks + 1) // 2  # two chunks a range at most
    return au, ou, rg


def test_plan_of_a_small_table():
    table = R.Table.generate(70000, seed=5, genome_len=4000, pool_sites=300, n_aa_genes=2, null_fraction=0.01)
    for column in range(table.n_seq):
        for ctas in (1, 3, 456):
            _check_plan(table, column, ctas)


def test_plan_with_bitsets_and_more_chunks_than_two_per_cta():
    """Few sites mutated in most rows give bitset containers; ten chunks over three CTAs need more
    ranges than CTAs, and the range builder must still end."""
    table = R.Table.generate(600000, seed=3, genome_len=500, pool_sites=20)
    au, ou, rg = _check_plan(table, 0, 3)
    assert (ou[:, 0] == 1).any()
    assert len(rg) > 3
    _check_plan(table, 0, 456)
