"""Ingestion: the product's storage image against the oracle's own ingestion, and the run-based
diff against the reference's string diff (src/rhydb/common/aligned_sequence.cpp:19-122)."""
import numpy as np
import pytest

import oracle as oracle_mod
import rhydb_gpu as R
from rawtable import RawBuilder, oracle_for


def same_storage(t, orc):
    for ci in range(t.n_seq):
        assert t.local_reference(ci) == orc.local_reference(ci), ci
        pos, ch, sym, card, _ = t.containers(ci)
        p2, v2, s2, c2 = orc.vertical(ci)
        a = sorted(zip(pos.tolist(), ch.tolist(), sym.tolist(), card.tolist()))
        b = sorted(zip(p2.tolist(), v2.tolist(), s2.tolist(), c2.tolist()))
        assert a == b, ci


@pytest.mark.parametrize("rows,seed,genes,nulls", [(1, 1, 0, 0.0), (65536, 2, 0, 0.0), (65537, 3, 2, 0.01),
                                                    (100000, 42, 12, 0.002)])
def test_generated_storage_matches_oracle(rows, seed, genes, nulls):
    genome = 29903 if genes == 12 else 3000
    t = R.Table.generate(rows, seed=seed, genome_len=genome, pool_sites=400, n_aa_genes=genes, null_fraction=nulls)
    assert t.n_chunks == (rows + 65535) // 65536
    same_storage(t, oracle_for(t))


def test_local_reference_flips_on_majority():
    # sequence_column.test.cpp:159-189 / vertical_sequence_index.test.cpp:311: a position whose
    # majority symbol differs from the reference is flipped; ties keep the reference.
    ref = "ACGTACGT"
    rows = ["TCGTACGT", "TCGTACGT", "TCGTACGT", "ACGTACGT", "ACCTACGN", "NNNNNNNN", None]
    b = RawBuilder(len(rows)).add_sequences("main", 0, ref, rows)
    raw = b.raw()
    t = R.Table.from_raw(raw)
    orc = oracle_for(t, raw)
    assert t.local_reference(0) == orc.local_reference(0)
    # position 1: T in 3 rows, A in 2 rows (the all-N and the null row do not count)
    assert t.local_reference(0)[0] == "T"
    assert t.local_reference(0)[2] == "G"  # C in one row only
    same_storage(t, orc)
    # after the flip the old reference symbol is stored as a container
    pos, ch, sym, card, _ = t.containers(0)
    entries = {(int(p), "-ACGTRYSWKMBDHVN"[s]): int(c) for p, s, c in zip(pos, sym, card)}
    assert entries[(0, "A")] == 2  # rows 3 and 4 hold A at position 1
    assert (0, "T") not in entries


@pytest.mark.parametrize("ref,seqs", [
    ("ATGCN", ["ATGCN", "NNNNN", "CATTT", "atgcn", "AUGCN", "NTGCN", "ATGNN"]),
    ("ACGTACGTAC", ["NNACGTACNN", "ACGT-CGTAC", "RCGTACGTAY", "ACGTNNNTAC", "NNNNNNNNNA", "ANNNNNNNNN"]),
])
def test_run_ingestion_matches_string_diff(ref, seqs):
    """Coverage and mutations from the run form equal the reference's string diff."""
    b = RawBuilder(len(seqs)).add_sequences("main", 0, ref, seqs)
    raw = b.raw()
    t = R.Table.from_raw(raw)
    orc = oracle_for(t, raw)
    pos, ch, sym, card, _ = t.containers(0)
    for r, s in enumerate(seqs):
        start, end, missing, muts = oracle_mod.diff_string(0, s, ref)
        ostart, oend, ivs = orc.row_coverage(0, r)
        assert (ostart, oend) == (start, end), (s, start, end, ostart, oend)
        got_missing = [p for a, z in ivs for p in range(a, z)]
        assert got_missing == missing, s
    same_storage(t, orc)


def test_illegal_characters_are_rejected():
    b = RawBuilder(1).add_sequences("main", 0, "ACGT", ["AC!T"])
    with pytest.raises(R.RhyError):
        R.Table.from_raw(b.raw())


def test_dictionary_and_dates_round_trip():
    b = RawBuilder(3).add_sequences("main", 0, "ACGT", ["ACGT", None, "ACGA"])
    b.add_dict("country", ["CH", None, "DE"]).add_dates("date", [18262, None, 18300])
    raw = b.raw()
    t = R.Table.from_raw(raw)
    orc = oracle_for(t, raw)
    assert orc.count("StrEq(country,CH)") == 1
    assert orc.count("StrEq(country,FR)") == 0
    assert orc.count("DateBetween(date,*,*)") == 2
    assert orc.count("Not(DateBetween(date,18262,18262))") == 2
    assert "Empty" == t.plan("StrEq(country,FR)")[0]
