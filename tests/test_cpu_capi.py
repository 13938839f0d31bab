"""The C-ABI library: every declared entry point is exported, errors cross the boundary as status
codes, and the host planner reproduces the reference's operator-tree shapes."""
import ctypes as C
import re
from pathlib import Path

import pytest

import rhydb_gpu as R
from rawtable import RawBuilder

HEADER = Path(__file__).resolve().parents[1] / "include" / "rhydb_gpu.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\*)\s+(rhy_\w+)\s*\(", text, re.M)))


def test_every_declared_symbol_is_exported():
    lib = C.CDLL(str(R.LIB_PATH))
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_null_arguments_are_rejected_without_crashing():
    lib = R.lib()
    assert lib.rhy_table_info(None, None) == 4
    assert b"must not be NULL" in lib.rhy_last_error()
    assert lib.rhy_count(None, b"True", None, None) == 4


def test_open_without_gpu_fails_cleanly(gpu_available):
    if gpu_available:
        pytest.skip("a GPU is present")
    t = R.Table.generate(100, seed=1, genome_len=100, pool_sites=10)
    with pytest.raises(R.RhyError) as e:
        R.Device(t, 0)
    assert e.value.code == 3  # RHY_CUDA


@pytest.fixture(scope="module")
def small_table():
    rows = ["ATGCN", "ATGCN", "NNNNN", "CATTT", None]
    b = RawBuilder(5).add_sequences("segment1", 0, "ATGCN", rows)
    b.add_dict("country", ["CH", "CH", "DE", None, "FR"])
    b.add_dates("date", [18262, 18263, None, 18300, 18262])
    raw = b.raw()
    return b, R.Table.from_raw(raw)


@pytest.mark.parametrize("expr,shape", [
    # compileSymbolInSet shapes (symbol_in_set.cpp:230-264); the table has a null row
    ("SymEq(segment1,1,C)", r"^Scan\(0,1,0x4\)$"),                                    # only mutations
    ("SymEq(segment1,1,.)", r"^Intersection\(Select\[Covered\(1\)\]\(\);not:Scan\(0,1,"),  # with reference
    ("SymEq(segment1,1,N)", r"^Intersection\(Union\(Select\[!Covered\(1\)\]\(\),Scan\(0,1,0x8000\)\);not:Nulls\(0\)\)$"),
    ("Or(SymEq(segment1,1,.),SymEq(segment1,1,N))", r"^Intersection\(!Scan\(0,1,0x7ffd\);not:Nulls\(0\)\)$"),
    # NOf folding (nof.cpp:33-150)
    ("NOf(0,atleast,SymEq(segment1,1,C))", r"^Full$"),
    ("NOf(2,atleast,SymEq(segment1,1,C))", r"^Empty$"),
    ("NOf(1,atleast,SymEq(segment1,1,C),SymEq(segment1,2,A))", r"^Union\("),
    ("NOf(2,atleast,SymEq(segment1,1,C),SymEq(segment1,2,A))", r"^Intersection\("),
    ("NOf(2,atleast,SymEq(segment1,1,C),SymEq(segment1,2,A),SymEq(segment1,3,T))", r"^Threshold\(>=2;"),
    ("NOf(1,exactly,SymEq(segment1,1,C),SymEq(segment1,2,A))", r"^Threshold\(=1;"),
    ("Maybe(NOf(1,exactly,SymEq(segment1,1,C),SymEq(segment1,2,A)))", r"^Intersection\("),
    # And/Or/Not (and.cpp:91-219, or.cpp:194-241, operator.cpp:23-66)
    ("Not(SymEq(segment1,1,C))", r"^!Scan"),
    ("Not(Not(SymEq(segment1,1,C)))", r"^Scan"),
    ("Or(SymEq(segment1,1,C),Not(SymEq(segment1,2,A)))", r"^!Intersection\("),
    ("And(Not(SymEq(segment1,1,C)),Not(SymEq(segment1,2,A)))", r"^!Union\("),
    ("And(DateBetween(date,18262,18262),StrEq(country,CH))", r"^Select\[Date.*\]\(Dict\(0,0\)\)$"),
    ("Not(DateBetween(date,*,18262))", r"^!Select\["),
    ("StrEq(country,XX)", r"^Empty$"),
    ("And(True,StrEq(country,CH))", r"^Dict\(0,0\)$"),
    ("Or(True,StrEq(country,CH))", r"^Full$"),
])
def test_operator_tree_shapes(small_table, expr, shape):
    _, t = small_table
    tree, n_instr, depth = t.plan(expr)
    assert re.search(shape, tree), tree
    assert n_instr >= 1 and depth >= 1


@pytest.mark.parametrize("expr", ["SymEq(segment1,6,A)", "SymEq(segment1,0,A)", "HasMut(nope,1)", "SymEq(segment1,1,!)",
                                  "StrEq(nope,x)", "DateBetween(nope,*,*)", "Foo(1)", "And(", "SymEq(segment1,1)"])
def test_user_errors(small_table, expr):
    _, t = small_table
    with pytest.raises(R.IllegalQuery):
        t.plan(expr)


def test_mutation_rows_threshold_arithmetic(small_table):
    """addMutationsToOutput (mutations_node.cpp:292-366): total over valid symbols, threshold
    ceil(total * p) - 1 in double, rows only for symbols other than the global reference."""
    _, t = small_table
    import numpy as np
    counts = np.zeros((16, 5), np.uint32)
    counts[1, 0] = 95   # A (reference at position 1)
    counts[2, 0] = 5    # C: 5/100 = 0.05 -> threshold ceil(5) - 1 = 4 -> reported
    counts[15, 0] = 50  # N is not a valid mutation symbol: not in the total
    counts[9, 1] = 7    # K at position 2: ambiguity code, not counted
    rows = t.mutation_rows(0, counts, 0.05)
    assert rows == [(1, "A", "C", 5, 100, 0.05)]
    assert t.mutation_rows(0, counts, 0.051) == []
    assert t.mutation_rows(0, counts, 0.0) == [(1, "A", "C", 5, 100, 0.05)]
