"""Known answers of the reference's operator and row-set tests, restated as operator trees over
explicit row sets (the reference builds its test operators as IndexScan over given bitmaps, e.g.
intersection.test.cpp:16-27). tests/test_golden_operators.py runs them through the CPU oracle, the
host check of rhy_program_plan and, with -m gpu, rhy_program_eval on the GPU.

A case: name, n_rows (the RowLayout the reference test uses), sets (row id lists), tree, and the
expected row ids, or "compile_error" where the reference throws at construction.
Trees: ("rows", i) | ("and", [children], [negated]) | ("or", [children]) | ("not", child)
       | ("threshold", n, exact, [children], [negated]).
Expected values of the CopyOnWriteBitmap tests, which the reference computes with Roaring's own
set operators (left & right, left - right, a | b | c), are written out here as explicit sets."""


def _rows(*xs):
    return sorted(set(xs))


K = 1 << 16  # rows per chunk (one roaring key)

# src/rhydb/query_engine/filter/operators/intersection.test.cpp
INTERSECTION = [
    # :30-39 no children at all
    {"name": "intersection.test.cpp:30 shouldFailOnEmptyInput", "n_rows": 5, "sets": [],
     "tree": ("and", [], []), "expected": "compile_error"},
    # :41-53 only negated children
    {"name": "intersection.test.cpp:41 shouldFailOnOnlyNegated", "n_rows": 5, "sets": [[1, 2, 3], [1, 2, 3]],
     "tree": ("and", [], [("rows", 0), ("rows", 1)]), "expected": "compile_error"},
    # :55-65 one non-negated child
    {"name": "intersection.test.cpp:55 shouldFailOnOneNonNegated", "n_rows": 5, "sets": [[1, 2, 3]],
     "tree": ("and", [("rows", 0)], []), "expected": "compile_error"},
    # :67-77
    {"name": "intersection.test.cpp:67 evaluateShouldReturnCorrectValuesNoNegated", "n_rows": 5,
     "sets": [[1, 2, 3], [1, 3], [1, 2, 3]], "tree": ("and", [("rows", 0), ("rows", 1), ("rows", 2)], []),
     "expected": [1, 3]},
    # :79-92
    {"name": "intersection.test.cpp:79 evaluateShouldReturnCorrectValues", "n_rows": 5,
     "sets": [[1, 2, 3], [1, 3], [1, 2, 3], [], [3]],
     "tree": ("and", [("rows", 0), ("rows", 1), ("rows", 2)], [("rows", 3), ("rows", 4)]), "expected": [1]},
    # :94-108
    {"name": "intersection.test.cpp:94 evaluateShouldReturnCorrectValuesManyNegated", "n_rows": 5,
     "sets": [[1, 2, 3], [], [3], [4], [2, 4]],
     "tree": ("and", [("rows", 0)], [("rows", 1), ("rows", 2), ("rows", 3), ("rows", 4)]), "expected": [1]},
    # :110-123
    {"name": "intersection.test.cpp:110 evaluateShouldReturnCorrectValuesEmptyInput", "n_rows": 5,
     "sets": [[], [3], [4], [2, 4]],
     "tree": ("and", [("rows", 0)], [("rows", 1), ("rows", 2), ("rows", 3)]), "expected": []},
]

# src/rhydb/query_engine/filter/operators/union.test.cpp
UNION = [
    {"name": "union.test.cpp:27 evaluatesCorrectOnEmptyInput", "n_rows": 5, "sets": [], "tree": ("or", []),
     "expected": []},
    {"name": "union.test.cpp:35 evaluatesCorrectOnOneInput", "n_rows": 7, "sets": [[1, 3, 5]],
     "tree": ("or", [("rows", 0)]), "expected": [1, 3, 5]},
    {"name": "union.test.cpp:44 evaluateShouldReturnCorrectValues1", "n_rows": 7, "sets": [[1, 2, 3], [1, 3], [1, 2, 3]],
     "tree": ("or", [("rows", 0), ("rows", 1), ("rows", 2)]), "expected": [1, 2, 3]},
    {"name": "union.test.cpp:55 evaluateShouldReturnCorrectValues2", "n_rows": 8, "sets": [[1, 7], [1, 3], [3]],
     "tree": ("or", [("rows", 0), ("rows", 1), ("rows", 2)]), "expected": [1, 3, 7]},
    {"name": "union.test.cpp:66 evaluateShouldReturnCorrectValuesMany", "n_rows": 13,
     "sets": [[], [3], [4]] + [[2, 4]] * 11, "tree": ("or", [("rows", i) for i in range(14)]), "expected": [2, 3, 4]},
    {"name": "union.test.cpp:90 evaluateShouldReturnCorrectValuesEmptyInput", "n_rows": 80, "sets": [[]],
     "tree": ("or", [("rows", 0)]), "expected": []},
]

# src/rhydb/query_engine/filter/operators/complement.test.cpp
COMPLEMENT = [
    {"name": "complement.test.cpp:13 evaluateShouldReturnCorrectValues", "n_rows": 5, "sets": [[1, 2, 3]],
     "tree": ("not", ("rows", 0)), "expected": [0, 4]},
    {"name": "complement.test.cpp:23 evaluateShouldReturnCorrectValuesWhenEmptyInput", "n_rows": 3, "sets": [[]],
     "tree": ("not", ("rows", 0)), "expected": [0, 1, 2]},
    # :33-41 RowLayout::of() holds no rows; tables here hold at least one row, so only the oracle
    # runs this case
    {"name": "complement.test.cpp:33 evaluateShouldReturnCorrectValuesWhenEmptyDatabase", "n_rows": 0, "sets": [[]],
     "tree": ("not", ("rows", 0)), "expected": []},
    {"name": "complement.test.cpp:43 evaluateShouldReturnCorrectValuesWhenFullInput", "n_rows": 4, "sets": [[0, 1, 2, 3]],
     "tree": ("not", ("rows", 0)), "expected": []},
    {"name": "complement.test.cpp:53 evaluateShouldReturnCorrectValuesWhenSingleInput", "n_rows": 5, "sets": [[1]],
     "tree": ("not", ("rows", 0)), "expected": [0, 2, 3, 4]},
]

# src/rhydb/query_engine/copy_on_write_bitmap.test.cpp: the row-set algebra, over row sets that span
# several 2^16-row chunks (roaring keys). MULTI is multiContainer() (:21-27).
MULTI = [1, 5, 100, K + 3, 3 * K + 7]
_COW_ROWS = 10 * K  # keys 0 .. 9 exist


def _staggered():
    """fastUnionMergesManyInputsWithStaggeredKeyRanges (:130-157): 8 inputs over staggered key ranges."""
    out = []
    for b in range(8):
        s = set()
        for key in range(b, b + 5):
            s.update(range((key << 16) + b, (key << 16) + b + 5000 + key * 100))
            s.add((key << 16) + 60000)
        out.append(sorted(s))
    return out


_STAG = _staggered()
COPY_ON_WRITE = [
    # :31-40 cardinality of a multi-chunk row set (and of the empty one)
    {"name": "copy_on_write_bitmap.test.cpp:31 cardinalityAndEmptiness", "n_rows": _COW_ROWS, "sets": [MULTI],
     "tree": ("rows", 0), "expected": MULTI},
    # :48-62 left & right
    {"name": "copy_on_write_bitmap.test.cpp:48 intersection", "n_rows": _COW_ROWS,
     "sets": [MULTI, [5, 100, K + 3, 999]], "tree": ("and", [("rows", 0), ("rows", 1)], []),
     "expected": _rows(5, 100, K + 3)},
    # :64-74 left - right
    {"name": "copy_on_write_bitmap.test.cpp:64 difference", "n_rows": _COW_ROWS, "sets": [MULTI, [5, K + 3]],
     "tree": ("and", [("rows", 0)], [("rows", 1)]), "expected": _rows(1, 100, 3 * K + 7)},
    # :76-90 first | second, then first | second | third
    {"name": "copy_on_write_bitmap.test.cpp:76 unionInPlace", "n_rows": _COW_ROWS, "sets": [[1, 5], MULTI],
     "tree": ("or", [("rows", 0), ("rows", 1)]), "expected": MULTI},
    {"name": "copy_on_write_bitmap.test.cpp:76 fastUnion", "n_rows": _COW_ROWS,
     "sets": [[1, 5], MULTI, [5, 3 * K + 7, 4 * K + 1]], "tree": ("or", [("rows", 0), ("rows", 1), ("rows", 2)]),
     "expected": _rows(*MULTI, 4 * K + 1)},
    # :92-111 fastUnion of nothing, of empties around one input, of only empties, of one input
    {"name": "copy_on_write_bitmap.test.cpp:92 fastUnionEdgeCases (none)", "n_rows": _COW_ROWS, "sets": [],
     "tree": ("or", []), "expected": []},
    {"name": "copy_on_write_bitmap.test.cpp:92 fastUnionEdgeCases (empties around one)", "n_rows": _COW_ROWS,
     "sets": [[], MULTI, []], "tree": ("or", [("rows", 0), ("rows", 1), ("rows", 2)]), "expected": MULTI},
    {"name": "copy_on_write_bitmap.test.cpp:92 fastUnionEdgeCases (only empties)", "n_rows": _COW_ROWS,
     "sets": [[], []], "tree": ("or", [("rows", 0), ("rows", 1)]), "expected": []},
    {"name": "copy_on_write_bitmap.test.cpp:92 fastUnionEdgeCases (single)", "n_rows": _COW_ROWS, "sets": [MULTI],
     "tree": ("or", [("rows", 0)]), "expected": MULTI},
    # :130-157 staggered key ranges with array, bitset and run sized containers
    {"name": "copy_on_write_bitmap.test.cpp:130 fastUnionMergesManyInputsWithStaggeredKeyRanges", "n_rows": 13 * K,
     "sets": _STAG, "tree": ("or", [("rows", i) for i in range(8)]),
     "expected": sorted(set().union(*map(set, _STAG)))},
    # :159-185 the union of four inputs in every order
    {"name": "copy_on_write_bitmap.test.cpp:159 fastUnionIsOrderIndependent", "n_rows": _COW_ROWS,
     "sets": [[1, 5, 100], MULTI, [5, 3 * K + 7, 4 * K + 1], [4 * K + 1, 9 * K]],
     "tree": "permutations-of-or-4", "expected": _rows(*MULTI, 4 * K + 1, 9 * K)},
    # :204-230 fromContainerViews: views of keys 3, 1, 0, 1 assembled, the two of key 1 ORed
    {"name": "copy_on_write_bitmap.test.cpp:204 fromContainerViewsAssemblesAndOrsSharedKeys", "n_rows": _COW_ROWS,
     "sets": [[3 * K + 7], [K + 3], [1, 5], [K + 9]], "tree": ("or", [("rows", i) for i in range(4)]),
     "expected": _rows(1, 5, K + 3, K + 9, 3 * K + 7)},
]

CASES = INTERSECTION + UNION + COMPLEMENT + COPY_ON_WRITE
