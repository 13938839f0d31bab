"""The reference's storage known answers (tests/golden/storage_cases.py): the aligned-sequence diff,
the horizontal coverage index, the vertical index with its local-reference adaptation, and the
Mutations output of union_all_node.test.cpp. Each runs through the CPU oracle and the product's
ingestion (its storage compared with the oracle's), and with -m gpu through the CUDA path."""
import numpy as np
import pytest

import oracle as oracle_mod
import rhydb_gpu as R
from golden import storage_cases as G
from rawtable import RawBuilder, oracle_for

ALPHABET = {0: R.NUC_SYMBOLS, 1: R.AA_SYMBOLS}
MISSING = {0: "N", 1: "X"}


def placed(fragment, offset, L, kind=0):
    """A fragment at an offset as a full aligned sequence (missing symbol around it)."""
    m = MISSING[kind]
    return m * offset + fragment + m * (L - offset - len(fragment))


def table_of(kind, reference, rows, dicts=()):
    b = RawBuilder(len(rows))
    b.add_sequences("main", kind, reference, rows)
    for name, values in dicts:
        b.add_dict(name, values)
    raw = b.raw()
    t = R.Table.from_raw(raw)
    return b, t, oracle_for(t, raw)


def covered_rows(orc, n_rows, pos):
    """Rows the oracle's coverage index covers at a position (null rows cover nothing)."""
    out = []
    for r in range(n_rows):
        s, e, missing = orc.row_coverage(0, r)
        if s <= pos < e and not any(a <= pos < b for a, b in missing):
            out.append(r)
    return out


def covered_nodes(pos):
    return [R.op_node(R.NODE_PRED_COVERED, column=0, position=pos), R.op_node(R.NODE_SELECTION, n_children=1)]


def storage_equal(t, orc):
    assert t.local_reference(0) == orc.local_reference(0)
    pos, ch, sym, card, _ = t.containers(0)
    p2, v2, s2, c2 = orc.vertical(0)
    assert sorted(zip(pos.tolist(), ch.tolist(), sym.tolist(), card.tolist())) == sorted(
        zip(p2.tolist(), v2.tolist(), s2.tolist(), c2.tolist()))


# ---------------------------------------------------------------------------------------------
# aligned sequences

VALID_ALIGNED = [c for c in G.ALIGNED if len(c) == 9]
ERROR_ALIGNED = [c for c in G.ALIGNED if len(c) == 6]


@pytest.mark.parametrize("case", VALID_ALIGNED, ids=lambda c: c[0])
def test_oracle_diff_known_answer(case):
    name, kind, frag, offset, ref, start, end, missing, muts = case
    seq = placed(frag, offset, len(ref), kind)
    s, e, miss, mm = oracle_mod.diff_string(kind, seq, ref)
    assert (s, e, miss) == (start, end, missing)
    assert [(p, ALPHABET[kind][x]) for p, x in mm] == muts


@pytest.mark.parametrize("case", ERROR_ALIGNED, ids=lambda c: c[0])
def test_illegal_character_is_rejected(case):
    name, kind, frag, offset, ref, message = case
    with pytest.raises(oracle_mod.OracleError) as e:
        oracle_mod.diff_string(kind, placed(frag, offset, len(ref), kind), ref)
    assert message in str(e.value)
    # the product's ingestion rejects the row as invalid input
    b = RawBuilder(1)
    b.add_sequences("main", kind, ref, [placed(frag, offset, len(ref), kind)])
    with pytest.raises(R.RhyError) as e:
        R.Table.from_raw(b.raw())
    assert e.value.code == 4 and "illegal character" in str(e.value)


@pytest.mark.parametrize("case", VALID_ALIGNED, ids=lambda c: c[0])
def test_product_ingestion_of_aligned_sequences(case):
    """The row next to two rows holding the reference (so no local reference flips): the product's
    storage equals the oracle's."""
    name, kind, frag, offset, ref, *_ = case
    _, t, orc = table_of(kind, ref, [placed(frag, offset, len(ref), kind), ref, ref])
    storage_equal(t, orc)


@pytest.mark.gpu
@pytest.mark.parametrize("case", VALID_ALIGNED, ids=lambda c: c[0])
def test_gpu_aligned_sequence_coverage_and_mutations(case):
    name, kind, frag, offset, ref, start, end, missing, muts = case
    L = len(ref)
    _, t, orc = table_of(kind, ref, [placed(frag, offset, L, kind), ref, ref])
    dev = R.Device(t, 0)
    for p in range(L):
        bits, _ = dev.program_eval(covered_nodes(p))
        row0 = 0 in R.bits_to_rows(bits).tolist()
        assert row0 == (start <= p < end and p not in missing), p
    for p, c in muts:
        bits, _ = dev.compute_filter(f"SymEq(main,{p + 1},{c})")
        assert 0 in R.bits_to_rows(bits).tolist(), (p, c)
    dev.close()


# ---------------------------------------------------------------------------------------------
# horizontal coverage index

def coverage_table(rows):
    L = len(G.COVERAGE_REFERENCE)
    seqs = [None if r is None else placed(r[0], r[1], L) for r in rows]
    return table_of(0, G.COVERAGE_REFERENCE, seqs)


@pytest.mark.parametrize("case", G.COVERAGE, ids=lambda c: c[0])
def test_oracle_coverage_known_answer(case):
    name, rows, checks = case
    _, t, orc = coverage_table(rows)
    for pos, expected in checks:
        assert covered_rows(orc, len(rows), pos) == expected, pos
    storage_equal(t, orc)


@pytest.mark.gpu
@pytest.mark.parametrize("case", G.COVERAGE, ids=lambda c: c[0])
def test_gpu_coverage_known_answer(case):
    name, rows, checks = case
    _, t, orc = coverage_table(rows)
    dev = R.Device(t, 0)
    for pos, expected in checks:
        bits, n = dev.program_eval(covered_nodes(pos))
        assert R.bits_to_rows(bits).tolist() == expected and n == len(expected), pos
    dev.close()


@pytest.mark.gpu
def test_gpu_coverage_cardinalities():
    for name, rows in G.COVERAGE_CARDINALITIES:
        _, t, orc = coverage_table(rows)
        dev = R.Device(t, 0)
        for pos in range(G.GENOME_LENGTH):
            assert dev.program_count(covered_nodes(pos)) == len(covered_rows(orc, len(rows), pos)), (name, pos)
        dev.close()
    name, placed_rows = G.COVERAGE_CHUNKS
    n = max(placed_rows) + 1
    rows = [placed_rows.get(i) for i in range(n)]
    _, t, orc = coverage_table(rows)
    dev = R.Device(t, 0)
    for pos in range(G.GENOME_LENGTH):
        want = [r for r in placed_rows if r in covered_rows_sparse(orc, placed_rows, pos)]
        assert dev.program_count(covered_nodes(pos)) == len(want), (name, pos)
    dev.close()


def covered_rows_sparse(orc, rows, pos):
    out = []
    for r in rows:
        s, e, missing = orc.row_coverage(0, r)
        if s <= pos < e and not any(a <= pos < b for a, b in missing):
            out.append(r)
    return out


# ---------------------------------------------------------------------------------------------
# vertical index: local-reference adaptation and stored symbols

@pytest.mark.parametrize("case", G.ADAPTATION, ids=lambda c: c[0])
def test_adaptation_known_answer(case):
    name, rows, ref, adapted, stored = case
    _, t, orc = table_of(0, ref, list(rows))
    assert t.local_reference(0) == adapted
    assert orc.local_reference(0) == adapted
    pos, ch, sym, card, _ = t.containers(0)
    got = {R.NUC_SYMBOLS[s]: int(c) for s, c in zip(sym.tolist(), card.tolist())}
    assert got == {s: len(r) for s, r in stored.items() if r}
    storage_equal(t, orc)


@pytest.mark.gpu
@pytest.mark.parametrize("case", G.ADAPTATION, ids=lambda c: c[0])
def test_gpu_stored_containers_after_adaptation(case):
    """IndexScan over the stored containers (getMatchingContainersAsBitmap) after adaptation."""
    name, rows, ref, adapted, stored = case
    _, t, orc = table_of(0, ref, list(rows))
    dev = R.Device(t, 0)
    for s, expected in stored.items():
        nodes = [R.op_node(R.NODE_SCAN_SEQ, column=0, position=0, symbols=1 << R.NUC_SYMBOLS.index(s))]
        bits, _ = dev.program_eval(nodes)
        assert R.bits_to_rows(bits).tolist() == expected, s
    dev.close()


def _holding(rows, p, c):
    return [i for i, r in enumerate(rows) if r[p].upper() == c]


@pytest.mark.parametrize("case", G.STORED_SYMBOLS, ids=lambda c: c[0])
def test_stored_symbols_known_answer(case):
    name, kind, ref, rows = case
    _, t, orc = table_of(kind, ref, rows)
    storage_equal(t, orc)
    for p in range(len(ref)):
        for c in sorted({r[p] for r in rows} - {MISSING[kind]}):
            bits, _ = orc.compute_filter(f"SymEq(main,{p + 1},{c})")
            assert R.bits_to_rows(bits).tolist() == _holding(rows, p, c), (p, c)


@pytest.mark.gpu
@pytest.mark.parametrize("case", G.STORED_SYMBOLS, ids=lambda c: c[0])
def test_gpu_stored_symbols_known_answer(case):
    name, kind, ref, rows = case
    _, t, orc = table_of(kind, ref, rows)
    dev = R.Device(t, 0)
    for p in range(len(ref)):
        for c in sorted({r[p] for r in rows} - {MISSING[kind]}):
            bits, _ = dev.compute_filter(f"SymEq(main,{p + 1},{c})")
            assert R.bits_to_rows(bits).tolist() == _holding(rows, p, c), (p, c)
    dev.close()


# ---------------------------------------------------------------------------------------------
# Mutations output

def union_all_table():
    U = G.UNION_ALL
    return table_of(0, U["reference"], U["rows"], dicts=[("country", U["country"])])


def test_oracle_mutations_known_answer():
    _, t, orc = union_all_table()
    for expr, min_prop, expected in G.UNION_ALL["cases"]:
        counts, _ = orc.mutations(expr, 0)
        assert orc.mutation_rows(0, counts, min_prop) == expected, expr


@pytest.mark.gpu
def test_gpu_mutations_known_answer():
    _, t, orc = union_all_table()
    dev = R.Device(t, 0)
    cases = G.UNION_ALL["cases"]
    for expr, min_prop, expected in cases:
        counts, _ = dev.mutations(expr, 0)
        assert t.mutation_rows(0, counts, min_prop) == expected, expr
    # the same through the batched call whose rows are built on the device
    exprs = [c[0] for c in cases]
    _, rows, begin, cnt = dev.batch_rows(exprs, [1] * len(cases), [0] * len(cases), [c[1] for c in cases])
    for i, (expr, _, expected) in enumerate(cases):
        got = [(int(r["position"]), r["from_"].decode(), r["to"].decode(), int(r["count"]), int(r["coverage"]),
                float(r["proportion"])) for r in rows[int(begin[i]):int(begin[i]) + int(cnt[i])]]
        assert got == expected, expr
    dev.close()
