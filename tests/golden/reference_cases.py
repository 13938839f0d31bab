"""Known-answer scenarios of the reference's own test suite, restated in this project's expression
syntax. Each dataset and expected result is taken from the cited reference test file; the test
that consumes them (tests/test_golden_reference.py) runs them through the CPU oracle, the host
planner and the GPU path.

Reference test data: sequences as NDJSON rows, reference genomes per sequence column, metadata.
Here a dataset is a dict with per-column literal aligned sequences (None = the row has no sequence)
and metadata lists.
"""

# src/rhydb/query_engine/scalar_expressions/symbol_equals.test.cpp:42-66 (nucleotide TEST_DATA)
SYMBOL_EQUALS_NUC = {
    "name": "symbol_equals.test.cpp:42-66",
    "n_rows": 5,
    "seq": [
        ("segment1", 0, "ATGCN", ["ATGCN", "ATGCN", "NNNNN", "CATTT", None]),
        ("gene1", 1, "M*", [None, None, None, None, None]),
    ],
    "cases": [
        # symbol_equals.test.cpp:86-226: nucleotideEquals(position, symbol) -> count
        ("SymEq(segment1,1,C)", 1), ("SymEq(segment1,1,.)", 2),
        ("SymEq(segment1,2,C)", 0), ("SymEq(segment1,3,C)", 0), ("SymEq(segment1,4,C)", 2), ("SymEq(segment1,5,C)", 0),
        ("SymEq(segment1,1,A)", 2), ("SymEq(segment1,2,A)", 1), ("SymEq(segment1,3,A)", 0), ("SymEq(segment1,4,A)", 0),
        ("SymEq(segment1,5,A)", 0),
        ("SymEq(segment1,1,G)", 0), ("SymEq(segment1,2,G)", 0), ("SymEq(segment1,3,G)", 2), ("SymEq(segment1,4,G)", 0),
        ("SymEq(segment1,5,G)", 0),
        ("SymEq(segment1,1,T)", 0), ("SymEq(segment1,2,T)", 2), ("SymEq(segment1,3,T)", 1), ("SymEq(segment1,4,T)", 1),
        ("SymEq(segment1,5,T)", 1),
        ("SymEq(segment1,1,N)", 1), ("SymEq(segment1,5,N)", 3),
        # symbol_equals.test.cpp:228-236: every amino-acid sequence is null, nothing matches X
        ("SymEq(gene1,1,X)", 0),
    ],
    # symbol_equals.test.cpp:238-249: out of range -> user error
    "errors": ["SymEq(segment1,1000,C)", "SymEq(segment1,0,.)"],
}

# src/rhydb/query_engine/scalar_expressions/has_mutation.test.cpp:22-44
HAS_MUTATION = {
    "name": "has_mutation.test.cpp:22-44",
    "n_rows": 4,
    "seq": [
        ("segment1", 0, "ATGCN", ["ATGCN", "ATGCN", "NNNNN", "CATTT"]),
        ("gene1", 1, "M*", ["M*", "C*", "M*", "X*"]),
    ],
    "cases": [
        ("HasMut(segment1,1)", 1),   # has_mutation.test.cpp:46-52
        ("HasMut(gene1,1)", 1),      # :54-59
        ("HasMut(segment1,5)", 1),   # :85-91
    ],
    # :61-83, :93-99: positions out of bounds
    "errors": ["HasMut(segment1,2000)", "HasMut(segment1,6)", "HasMut(gene1,1000)", "HasMut(segment1,0)"],
}

# src/rhydb/query_engine/scalar_expressions/symbol_equals.test.cpp:262-316 (amino-acid TEST_DATA)
SYMBOL_EQUALS_AA = {
    "name": "symbol_equals.test.cpp:262-316",
    "n_rows": 4,
    "seq": [
        ("segment1", 0, "A", [None, None, None, None]),
        ("gene1", 1, "M*", ["D*", "M*", "M*", "B*"]),
    ],
    "cases": [
        ("SymEq(gene1,1,D)", 1),  # :301-307
        ("SymEq(gene1,1,.)", 2),  # :309-315
    ],
    "errors": [],
}

# src/rhydb/query_engine/scalar_expressions/nof.test.cpp:56-120: five rows with country, region, date
_NOF_ROWS = [("Switzerland", "Europe", "2020-01-01"), ("Germany", "Europe", "2021-06-15"),
             ("USA", "Americas", "2019-03-20"), ("Switzerland", "Europe", "2018-11-01"),
             ("France", "Europe", "2022-07-10")]
NOF = {
    "name": "nof.test.cpp:56-120",
    "n_rows": 5,
    "seq": [("segment1", 0, "ATGCN", ["ACGTN"] * 5)],
    "dict": [("country", [r[0] for r in _NOF_ROWS]), ("region", [r[1] for r in _NOF_ROWS])],
    "date": [("date", [r[2] for r in _NOF_ROWS])],
    # expected row ids (the reference's expected primary keys id_<row>)
    "row_cases": [
        ("NOf(2,atleast,StrEq(country,Switzerland),StrEq(country,Germany),StrEq(region,Europe))", [0, 1, 3]),
        ("NOf(3,atleast,StrEq(country,Switzerland),DateBetween(date,18262,18262),StrEq(region,Europe))", [0]),
        ("NOf(3,atleast,StrEq(country,Switzerland),StrEq(country,Germany),StrEq(region,Europe))", []),
        ("NOf(1,atleast,StrEq(country,Switzerland),StrEq(country,USA))", [0, 2, 3]),
        ("NOf(1,exactly,StrEq(country,Switzerland),StrEq(region,Europe))", [1, 4]),
        ("NOf(2,exactly,StrEq(country,Switzerland),StrEq(region,Europe))", [0, 3]),
        ("NOf(0,atleast,StrEq(country,Switzerland),StrEq(country,Germany))", [0, 1, 2, 3, 4]),
        ("NOf(0,exactly,StrEq(country,Switzerland),StrEq(region,Europe))", [2]),
        ("NOf(2,atleast,StrEq(country,Switzerland),Not(StrEq(country,USA)))", [0, 3]),
        ("NOf(1,atleast,StrEq(country,Switzerland),Not(StrEq(country,Germany)))", [0, 2, 3, 4]),
        ("NOf(0,exactly,StrEq(country,Switzerland))", [1, 2, 4]),
        ("NOf(0,exactly,Not(StrEq(country,Switzerland)))", [0, 3]),
        ("NOf(2,atleast,Not(StrEq(country,Switzerland)),Not(StrEq(country,USA)))", [1, 4]),
        ("NOf(0,exactly,StrEq(country,Switzerland),Not(StrEq(country,USA)))", [2]),
        ("NOf(5,exactly,StrEq(country,Switzerland),StrEq(country,USA))", []),
    ],
    "cases": [],
    "errors": [],
}

# src/rhydb/query_engine/scalar_expressions/mutation_profile.test.cpp:23-62: six rows, the primary
# key a metadata column; segment1 reference ATGCN, gene1 reference M* (gene2 has no sequences)
MUTATION_PROFILE = {
    "name": "mutation_profile.test.cpp:23-62",
    "n_rows": 6,
    "seq": [
        ("segment1", 0, "ATGCN", ["ATGCN", "CTGCN", "CTCCN", "CTCTN", "NNNNN", "RTGCN"]),
        ("gene1", 1, "M*", ["M*", "C*", "M*", "M*", "M*", "M*"]),
        ("gene2", 1, "M*", [None] * 6),
    ],
    "dict": [("primaryKey", ["seq_ref", "seq_1mut", "seq_2mut", "seq_3mut", "seq_all_n", "seq_mixed_amb"])],
    "primary_key": "primaryKey",
    # expected row ids (rows in input order: seq_ref, seq_1mut, seq_2mut, seq_3mut, seq_all_n, seq_mixed_amb)
    "row_cases": [
        ("MutProfileMutations(segment1,0)", [0, 4, 5]),                 # :68-77
        ("MutProfileMutations(segment1,1)", [0, 1, 4, 5]),              # :79-88
        ("MutProfileMutations(segment1,2)", [0, 1, 2, 4, 5]),           # :90-99
        ("MutProfileMutations(segment1,0,1:C)", [1, 4]),                # :103-111
        ("MutProfile(segment1,0,ATGCN)", [0, 4, 5]),                    # :116-125
        ("MutProfileSequenceId(segment1,0,seq_1mut)", [1, 4]),          # :141-149
        ("MutProfileMutations(gene1,0)", [0, 2, 3, 4, 5]),              # :187-197
        ("MutProfileMutations(gene1,1)", [0, 1, 2, 3, 4, 5]),           # :199-209
        ("MutProfileMutations(gene1,0,1:C)", [1]),                      # :211-217
        ("MutProfile(gene1,0,M*)", [0, 2, 3, 4, 5]),                    # :221-231
        ("MutProfileSequenceId(gene1,0,seq_1mut)", [1]),                # :233-240
    ],
    "cases": [],
    "errors": [
        "MutProfile(segment1,0,ATG)",                      # :127-137, querySequence of the wrong length
        "MutProfileSequenceId(segment1,0,nonexistent_id)", # :151-159
        "MutProfileMutations(nonexistent_gene,0)",         # :242-249
        "MutProfileMutations(gene1,0,123456:C)",           # :259-268, position out of bounds
    ],
}

# src/rhydb/query_engine/scalar_expressions/date_between.test.cpp:10-47: one row, a sorted and an
# unsorted date column (2020-12-24 = day 18620, 2023-01-20 = day 19377); the reference has no
# sequence columns, the five-position column of the other datasets stands in here
DATE_BETWEEN = {
    "name": "date_between.test.cpp:10-47",
    "n_rows": 1,
    "seq": [("segment1", 0, "ATGCN", ["ACGTN"])],
    "dict": [("primaryKey", ["id"])],
    "date": [("sorted_date", ["2020-12-24"]), ("unsorted_date", ["2023-01-20"])],
    "row_cases": [
        ("DateBetween(sorted_date,18620,18620)", [0]),    # :49-53
        ("DateBetween(sorted_date,*,18620)", [0]),        # :55-59
        ("DateBetween(sorted_date,18620,*)", [0]),        # :61-65
        ("DateBetween(unsorted_date,19377,19377)", [0]),  # :67-71
        ("DateBetween(unsorted_date,*,19377)", [0]),      # :73-77
        ("DateBetween(unsorted_date,19377,*)", [0]),      # :79-83
    ],
    "cases": [],
    "errors": [
        "DateBetween(something_not_in_database,10957,*)",  # :85-90
        "DateBetween(primaryKey,18262,*)",                 # :92-96, not a date column
    ],
}

# src/rhydb/query_engine/scalar_expressions/or.test.cpp:404-461: six rows with country and region
# (USA -> Americas, else Europe)
_OR_COUNTRIES = ["Switzerland", "Germany", "USA", "Switzerland", "France", "Germany"]
OR = {
    "name": "or.test.cpp:404-461",
    "n_rows": 6,
    "seq": [("segment1", 0, "ATGCN", ["ACGTN"] * 6)],
    "dict": [("country", _OR_COUNTRIES), ("region", ["Americas" if c == "USA" else "Europe" for c in _OR_COUNTRIES])],
    "row_cases": [
        ("Or(Or(StrEq(country,Switzerland),StrEq(country,Germany)),StrEq(country,France))", [0, 1, 3, 4, 5]),  # :463-477
        ("Or(StrEq(country,Switzerland),StrEq(country,Germany))", [0, 1, 3, 5]),                                # :479-492
        ("Or(StrEq(country,Switzerland))", [0, 3]),                                                              # :494-500
        ("Or(StrEq(country,Switzerland),StrEq(country,Germany),StrEq(country,France))", [0, 1, 3, 4, 5]),       # :502-516
        ("Or(StrEq(country,USA),StrEq(region,Europe))", [0, 1, 2, 3, 4, 5]),                                    # :518-533
        ("Or(And(StrEq(country,Switzerland),StrEq(region,Europe)),StrEq(country,USA))", [0, 2, 3]),            # :535-547
        ("False", []),                                                                                           # :549-552
        ("Or()", []),
    ],
    "cases": [],
    "errors": [],
}

# src/rhydb/query_engine/scalar_expressions/and.test.cpp:67-90: six rows with country and date
# (2009-01-01 = day 14245, 2000-01-01 = day 10957)
_AND_ROWS = [("Switzerland", "2020-01-01"), ("Germany", "2000-03-07"), ("Germany", "2009-06-07"),
             ("Switzerland", "2003-07-02"), ("Switzerland", "2002-01-04"), ("Switzerland", "2001-12-07")]
AND = {
    "name": "and.test.cpp:67-90",
    "n_rows": 6,
    "seq": [("segment1", 0, "ATGCN", ["ACGTN"] * 6)],
    "dict": [("country", [r[0] for r in _AND_ROWS])],
    "date": [("date", [r[1] for r in _AND_ROWS])],
    "row_cases": [
        ("And(DateBetween(date,14245,*),DateBetween(date,10957,*),StrEq(country,Germany))", [2]),  # :79-88
    ],
    "cases": [],
    "errors": [],
}

DATASETS = [SYMBOL_EQUALS_NUC, HAS_MUTATION, SYMBOL_EQUALS_AA, NOF, MUTATION_PROFILE, DATE_BETWEEN, OR, AND]

# Operator-level known answers: src/rhydb/query_engine/filter/operators/threshold.test.cpp:28-313.
# (kind 0 = Threshold; non-negated row sets, negated row sets, n, exactly, expected)
THRESHOLD_CASES = [
    # :39-55 evaluatesCorrectOnlyNegated (RowLayout::of(4))
    ([], [[1, 2, 3], [1, 3]], 1, True, [2]),
    ([], [[1, 2, 3], [1, 3]], 1, False, [0, 2]),
    # :57-83 evaluateShouldReturnCorrectValuesNoNegated
    ([[1, 2], [1, 3], [1, 2, 3]], [], 1, True, []),
    ([[1, 2], [1, 3], [1, 2, 3]], [], 2, True, [2, 3]),
    ([[1, 2], [1, 3], [1, 2, 3]], [], 1, False, [1, 2, 3]),
    ([[1, 2], [1, 3], [1, 2, 3]], [], 2, False, [1, 2, 3]),
    # :85-150 evaluateShouldReturnCorrectValues
    ([[1, 2, 3], [1, 3], [1, 2, 3]], [[], [3]], 1, True, []),
    ([[1, 2, 3], [1, 3], [1, 2, 3]], [[], [3]], 2, True, [0]),
    ([[1, 2, 3], [1, 3], [1, 2, 3]], [[], [3]], 3, True, []),
    ([[1, 2, 3], [1, 3], [1, 2, 3]], [[], [3]], 4, True, [2, 3]),
    ([[1, 2, 3], [1, 3], [1, 2, 3]], [[], [3]], 1, False, [0, 1, 2, 3]),
]
