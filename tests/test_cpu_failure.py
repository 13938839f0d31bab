"""Host-side failure paths: a corrupted raw partition is rejected by rhy_table_from_raw with
RHY_INVALID_ARGUMENT and a message (never a crash or a silently wrong table), and user errors in
queries and operator trees come back as codes."""
import ctypes as C

import numpy as np
import pytest

import rhydb_gpu as R
from rawtable import RawBuilder


def good_builder():
    b = RawBuilder(4)
    b.add_sequences("main", 0, "ACGTACGTAC", ["ACGTACGTAC", "ACGAACGTAC", "NNGTACGTAC", None])
    b.add_dict("country", ["CH", "DE", None, "CH"])
    b.add_dates("date", [18000, None, 18100, 18200])
    return b


def rejected(raw, fragment):
    with pytest.raises(R.RhyError) as e:
        R.Table.from_raw(raw)
    assert e.value.code == 4, str(e.value)
    assert fragment in str(e.value), str(e.value)


def test_good_partition_builds():
    t = R.Table.from_raw(good_builder().raw())
    assert t.n_rows == 4


def test_runs_out_of_order_are_rejected():
    b = good_builder()
    col = b.seq[0]
    # row 1 holds one run; make a second row claim runs in the wrong order
    pos = np.array([5, 3], np.uint32)
    lens = np.array([1, 1], np.uint32)
    ch = np.frombuffer(b"TT", np.uint8).copy()
    off = np.array([0, 0, 2, 2, 2], np.uint64)
    b._keep += [pos, lens, ch, off]
    col.run_pos = pos.ctypes.data_as(C.POINTER(C.c_uint32))
    col.run_len = lens.ctypes.data_as(C.POINTER(C.c_uint32))
    col.run_char = ch.ctypes.data_as(C.POINTER(C.c_char))
    col.row_off = off.ctypes.data_as(C.POINTER(C.c_uint64))
    b.seq[0] = col
    rejected(b.raw(), "sorted")


def test_run_past_the_genome_is_rejected():
    b = good_builder()
    col = b.seq[0]
    pos = np.array([8], np.uint32)
    lens = np.array([5], np.uint32)
    ch = np.frombuffer(b"T", np.uint8).copy()
    off = np.array([0, 1, 1, 1, 1], np.uint64)
    b._keep += [pos, lens, ch, off]
    col.run_pos = pos.ctypes.data_as(C.POINTER(C.c_uint32))
    col.run_len = lens.ctypes.data_as(C.POINTER(C.c_uint32))
    col.run_char = ch.ctypes.data_as(C.POINTER(C.c_char))
    col.row_off = off.ctypes.data_as(C.POINTER(C.c_uint64))
    b.seq[0] = col
    rejected(b.raw(), "inside the genome")


def test_decreasing_row_offsets_are_rejected():
    b = good_builder()
    col = b.seq[0]
    off = np.array([0, 2, 1, 1, 1], np.uint64)
    b._keep.append(off)
    col.row_off = off.ctypes.data_as(C.POINTER(C.c_uint64))
    b.seq[0] = col
    rejected(b.raw(), "row_off")


def test_illegal_symbol_is_rejected():
    b = RawBuilder(2)
    b.add_sequences("main", 0, "ACGT", ["ACGT", "ACQT"])
    rejected(b.raw(), "illegal character 'Q'")


def test_dictionary_id_out_of_range_is_rejected():
    b = good_builder()
    d = b.dict[0]
    ids = np.array([0, 1, 7, 0], np.uint32)
    b._keep.append(ids)
    d.ids = ids.ctypes.data_as(C.POINTER(C.c_uint32))
    b.dict[0] = d
    rejected(b.raw(), "value id")


def test_reference_with_an_illegal_character_is_rejected():
    b = RawBuilder(1)
    b.add_sequences("main", 0, "ACGJ", ["ACGJ"])
    rejected(b.raw(), "reference")


def test_unknown_sequence_kind_is_rejected():
    b = good_builder()
    col = b.seq[0]
    col.kind = 5
    b.seq[0] = col
    rejected(b.raw(), "kind")


def test_query_errors_are_codes():
    t = R.Table.from_raw(good_builder().raw())
    with pytest.raises(R.IllegalQuery):
        t.plan("SymEq(main,11,A)")
    with pytest.raises(R.IllegalQuery):
        t.plan("SymEq(nosuch,1,A)")
    with pytest.raises(R.RhyError):
        t.plan("And(SymEq(main,1,A)")
    # an NOf asking for more matches than it has children is not an error: it compiles to Empty
    # (the reference's NOf::handleTrivialCases, nof.cpp:33-80)
    assert t.plan("NOf(3,atleast,SymEq(main,1,A))")[0] == "Empty"
