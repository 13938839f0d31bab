"""Known answers of the reference's storage tests and of its one Mutations-output test, restated.

tests/test_golden_storage.py runs them through the CPU oracle, the product's ingestion (compared
with the oracle's storage) and, with -m gpu, the CUDA path (coverage predicates and index scans
through the operator-tree entry, Mutations rows through rhy_mutations).

A sequence placed "at an offset" in a reference test is stored here as the full aligned sequence:
the missing symbol before the offset and after the fragment, which the reference treats the same
way (positions below the offset and past the fragment are uncovered)."""

# ------------------------------------------------------------------------------------------------
# src/rhydb/common/aligned_sequence.test.cpp: extractCoverageAndMutationsFromSequence. Each case:
# kind (0 nucleotide, 1 amino acid), fragment, offset, reference, then the expected coverage start,
# end, missing positions and mutations [(position, character)], or an error message.
ALIGNED = [
    ("aligned_sequence.test.cpp:30 identicalSequenceHasNoMutationsAndFullCoverage", 0, "ACGT", 0, "ACGT", 0, 4, [], []),
    ("aligned_sequence.test.cpp:39 singleMutationIsRecordedWithGlobalPosition", 0, "AGGT", 0, "ACGT", 0, 4, [], [(1, "G")]),
    ("aligned_sequence.test.cpp:51 multipleMutationsAreRecordedInOrder", 0, "CCTT", 0, "ACGT", 0, 4, [],
     [(0, "C"), (2, "T")]),
    ("aligned_sequence.test.cpp:62 offsetShiftsPositionsAndIndexesIntoReference", 0, "AT", 2, "ACGT", 2, 4, [],
     [(2, "A")]),
    ("aligned_sequence.test.cpp:74 missingSymbolInsideCoveredRegionIsKept", 0, "ANGT", 0, "ACGT", 0, 4, [1], []),
    ("aligned_sequence.test.cpp:85 leadingAndTrailingMissingSymbolsAreTrimmed", 0, "NCGTAN", 0, "ACGTAC", 1, 5, [], []),
    ("aligned_sequence.test.cpp:95 onlyMissingOutsideCoverageIsTrimmedInnerKept", 0, "NCNTAN", 0, "ACGTAC", 1, 5, [2], []),
    ("aligned_sequence.test.cpp:106 fullyMissingSequenceHasEmptyCoverage", 0, "NNNN", 0, "ACGT", 0, 0, [], []),
    ("aligned_sequence.test.cpp:115 emptySequenceHasEmptyCoverage", 0, "", 0, "ACGT", 0, 0, [], []),
    ("aligned_sequence.test.cpp:124 deletionIsRecordedAsMutationToGapAndCountsAsCoverage", 0, "A-GT", 0, "ACGT", 0, 4, [],
     [(1, "-")]),
    ("aligned_sequence.test.cpp:136 leadingGapStartsCoverage", 0, "-CGT", 0, "ACGT", 0, 4, [], [(0, "-")]),
    ("aligned_sequence.test.cpp:147 charactersEncodingTheReferenceSymbolAreNoMutation", 0, "aCGU", 0, "ACGT", 0, 4, [],
     []),
    ("aligned_sequence.test.cpp:156 lowerCaseMissingSymbolIsMissing", 0, "AnGT", 0, "ACGT", 0, 4, [1], []),
    ("aligned_sequence.test.cpp:165 positionsWhereTheReferenceIsMissingAreMissing", 0, "ANGT", 0, "ANGT", 0, 4, [1], []),
    ("aligned_sequence.test.cpp:175 mutationAgainstAMissingReferenceSymbolIsRecorded", 0, "ACGT", 0, "ANGT", 0, 4, [],
     [(1, "C")]),
    ("aligned_sequence.test.cpp:186 sequencesLongerThanOneWordAreDiffed", 0,
     "N" + "A" * 2 + "C" + "A" * 11 + "G" + "A" * 12 + "NT", 0, "A" * 30, 1, 30, [28], [(3, "C"), (15, "G"), (29, "T")]),
    ("aligned_sequence.test.cpp:211 illegalCharacterHasError", 0, "ACXT", 0, "ACGT",
     "illegal character 'X' at position 2 in the input sequence"),
    ("aligned_sequence.test.cpp:217 offsetLeavesPositionsBelowOffsetWithoutCoverage", 0, "ACGT", 4, "AAAAACGT", 4, 8, [],
     []),
    ("aligned_sequence.test.cpp:227 offsetWithMutationUsesGlobalReferencePosition", 0, "AG", 4, "AAAAAC", 4, 6, [],
     [(5, "G")]),
    ("aligned_sequence.test.cpp:239 offsetKeepsInternalMissingAtGlobalPosition", 0, "ANT", 4, "AAAAACT", 4, 7, [5], []),
    ("aligned_sequence.test.cpp:250 offsetTrimsLeadingAndTrailingMissing", 0, "NCGN", 4, "AAAAACGA", 5, 7, [], []),
    ("aligned_sequence.test.cpp:261 offsetWithFullyMissingHasEmptyCoverage", 0, "NN", 4, "AAAAAA", 0, 0, [], []),
    ("aligned_sequence.test.cpp:270 offsetWithLeadingGapCoversFromOffset", 0, "-GT", 4, "AAAAAGT", 4, 7, [], [(4, "-")]),
    ("aligned_sequence.test.cpp:283 largeOffsetShiftsCoverageRange", 0, "ACGT", 50, "A" * 58, 50, 54, [],
     [(51, "C"), (52, "G"), (53, "T")]),
    ("aligned_sequence.test.cpp:297 sequencesLongerThanOneWordAreDiffedWithOffset", 0,
     "N" + "A" * 2 + "C" + "A" * 11 + "G" + "A" * 4 + "N" + "A" * 8 + "T", 51, "A" * 85, 52, 81, [71],
     [(54, "C"), (66, "G"), (80, "T")]),
    ("aligned_sequence.test.cpp:323 aminoAcidSequencesLongerThanOneWordAreDiffed", 1,
     "A" * 2 + "K" + "A" * 8 + "X" + "A" * 13 + "W" + "A" * 3 + "X", 0, "A" * 30, 0, 29, [11], [(2, "K"), (25, "W")]),
    ("aligned_sequence.test.cpp:348 worksForAminoAcidSymbolType", 1, "MXKL", 0, "MNKL", 0, 4, [1], []),
]


# ------------------------------------------------------------------------------------------------
# src/rhydb/storage/column/horizontal_coverage_index.test.cpp: the rows covered at a position
# (getCoverageBitmapForPositions<1>(position).at(0)). The fixture's reference is 256 x 'A' and its
# genome length 100 (:17-24). A row is (fragment, offset), or None for a null sequence.
COVERAGE_REFERENCE = "A" * 256
GENOME_LENGTH = 100
_G = GENOME_LENGTH
COVERAGE = [
    ("horizontal_coverage_index.test.cpp:57 NullSequenceIsUncoveredAtAllPositions", [None],
     [(0, []), (50, []), (98, [])]),
    ("horizontal_coverage_index.test.cpp:65 MultipleNullSequencesAllUncovered", [None, None, None],
     [(0, []), (50, [])]),
    ("horizontal_coverage_index.test.cpp:99 SequenceNotInBitmapForCoveredPositions", [("ACGT", 0)],
     [(0, [0]), (1, [0]), (2, [0]), (3, [0])]),
    ("horizontal_coverage_index.test.cpp:109 SequenceInBitmapForUncoveredPositions", [("ACGT", 0)],
     [(4, []), (10, []), (50, [])]),
    ("horizontal_coverage_index.test.cpp:118 MultipleSequencesWithOverlap", [("ACGTACGT", 0), ("TGCA", 5), ("AAAA", 10)],
     [(6, [0, 1]), (5, [0, 1]), (7, [0, 1]), (8, [1]), (11, [2])]),
    ("horizontal_coverage_index.test.cpp:139 NonOverlappingSequences", [("ACGT", 0), ("TGCA", 10)],
     [(2, [0]), (11, [1]), (5, [])]),
    ("horizontal_coverage_index.test.cpp:154 SequenceWithNIsUncoveredAtNPosition", [("ACNGT", 0)],
     [(0, [0]), (1, [0]), (3, [0]), (4, [0]), (2, [])]),
    ("horizontal_coverage_index.test.cpp:167 SequenceWithMultipleNs", [("ANNNGTA", 0)],
     [(0, [0]), (4, [0]), (5, [0]), (6, [0]), (1, []), (2, []), (3, [])]),
    ("horizontal_coverage_index.test.cpp:182 SequenceWithAllNs", [("NNNN", 5)],
     [(5, []), (6, []), (7, []), (8, []), (0, [])]),
    ("horizontal_coverage_index.test.cpp:195 MultipleSequencesWithNAtSamePosition",
     [("ACNGT", 0), ("AANAT", 0), ("ACGGT", 0)], [(2, [2]), (0, [0, 1, 2])]),
    ("horizontal_coverage_index.test.cpp:207 SequenceWithNAndOffset", [("ACNGT", 10)],
     [(12, []), (10, [0]), (11, [0]), (13, [0]), (14, [0])]),
    ("horizontal_coverage_index.test.cpp:225 SequenceWithLowercaseN", [("ACnGT", 0)], [(2, [])]),
    ("horizontal_coverage_index.test.cpp:238 GetBitmapAtGenomeBoundary", [("ACGT", 0)], [(_G - 1, [])]),
    ("horizontal_coverage_index.test.cpp:244 GetBitmapBeyondGenomeLength", [("ACGT", 0)], [(_G, []), (_G + 100, [])]),
    ("horizontal_coverage_index.test.cpp:253 InsertSequenceAtEndOfGenome", [("ACG", _G - 3)],
     [(_G - 3, [0]), (_G - 2, [0]), (_G - 1, [0]), (_G - 4, [])]),
    ("horizontal_coverage_index.test.cpp:265 InsertSequenceWithNAtEndOfGenome", [("ACN", _G - 3)],
     [(_G - 3, [0]), (_G - 2, [0]), (_G - 1, [])]),
    ("horizontal_coverage_index.test.cpp:276 InsertSequenceExtendingBeyondGenome", [("ACGTACGT", _G - 2)], []),
    ("horizontal_coverage_index.test.cpp:282 MixedNullAndCoveredSequences", [("ACGT", 0), None, ("TGCA", 0)],
     [(0, [0, 2]), (1, [0, 2]), (2, [0, 2]), (3, [0, 2]), (10, [])]),
    ("horizontal_coverage_index.test.cpp:297 MultipleNullsWithCoverage", [None, None, ("ACGT", 5), None],
     [(0, []), (5, [2]), (6, [2])]),
    ("horizontal_coverage_index.test.cpp:311 MixedNullCoverageAndNCharacters", [("ACNGT", 0), None, ("ACGGT", 0)],
     [(2, [2]), (0, [0, 2])]),
    ("horizontal_coverage_index.test.cpp:324 CompletelyOverlappingSequences", [("AAAA", 5), ("TTTT", 5), ("GGGG", 5)],
     [(5, [0, 1, 2]), (6, [0, 1, 2]), (7, [0, 1, 2]), (8, [0, 1, 2]), (4, [])]),
    ("horizontal_coverage_index.test.cpp:339 OverlappingSequencesWithN", [("ANNN", 5), ("NANN", 5), ("NNAN", 5)],
     [(5, [0]), (6, [1]), (7, [2]), (8, [])]),
    ("horizontal_coverage_index.test.cpp:357 PartiallyOverlappingSequences",
     [("AAAAAAAA", 0), ("TTTTTTTT", 4), ("GGGGGGGG", 8)], [(2, [0]), (5, [0, 1]), (9, [1, 2]), (14, [2])]),
    ("horizontal_coverage_index.test.cpp:375 AdjacentNonOverlappingSequences", [("AAAA", 0), ("TTTT", 4), ("GGGG", 8)],
     [(3, [0]), (4, [1]), (7, [1]), (8, [2])]),
    ("horizontal_coverage_index.test.cpp:387 ManySequences", [("ACGT", 0)] * 1000,
     [(0, list(range(1000))), (10, [])]),
    ("horizontal_coverage_index.test.cpp:403 ManySequencesAtDifferentPositions", [("A", i) for i in range(100)],
     [(p, [p]) for p in range(100)]),
    ("horizontal_coverage_index.test.cpp:416 LongSequence", [("A" * (_G // 2), 0)],
     [(0, [0]), (_G // 4, [0]), (_G // 2 - 1, [0]), (_G // 2, [])]),
    ("horizontal_coverage_index.test.cpp:432 InsertSequencesInOrder", [("A", 0), ("T", 0), ("G", 0)],
     [(0, [0, 1, 2]), (5, [])]),
    ("horizontal_coverage_index.test.cpp:444 InsertSequencesOutOfOrder", [("G", 0), ("A", 0), ("T", 0)],
     [(0, [0, 1, 2]), (5, [])]),
    ("horizontal_coverage_index.test.cpp:457 EmptySequenceIsAlwaysUncovered", [("", 5)], [(0, []), (5, []), (10, [])]),
]

# :469-490 computeCoverageCardinalities equals the covered-row count at every position < 100
COVERAGE_CARDINALITIES = [
    ("horizontal_coverage_index.test.cpp:469 CoverageCardinalitiesMatchBitmapCardinalities",
     [("A" * _G, 0), ("ACGTACGT", 10), ("ACGTNNNNNNACGT", 20), ("NNNACGTNNN", 40), ("N" * 15, 5), None, ("", 30)]),
]
# :492-514 one row at the start of each of three 2^16-row chunks (the rows between are absent from
# the reference's index; here they are null rows, which no position covers)
COVERAGE_CHUNKS = ("horizontal_coverage_index.test.cpp:492 CoverageCardinalitiesAcrossMultipleChunks",
                   {0: ("ACGTNNACGT", 0), 1 << 16: ("ACGTNNACGT", 5), 2 << 16: ("ACGTNNACGT", 10)})


# ------------------------------------------------------------------------------------------------
# src/rhydb/storage/column/vertical_sequence_index.test.cpp: the stored containers of one position
# (getMatchingContainersAsBitmap(position, {symbol})) after the local reference adapts at finalize,
# for columns whose rows hold the listed symbols ('N' = missing) under the given reference symbol.
# Each case: rows (one character per row at position 0), reference symbol, the adapted local
# reference symbol, and the stored rows per symbol.
ADAPTATION = [
    ("vertical_sequence_index.test.cpp:311 referenceAdaptsSingleSymbol", "A", "C", "A", {"A": [], "C": []}),
    ("vertical_sequence_index.test.cpp:337 referenceAdaptsSingleSymbolWhenSomeSymbolsAreMissing", "ANN", "C", "A",
     {"A": [], "C": []}),
    ("vertical_sequence_index.test.cpp:359 referenceDoesNotAdaptSingleSymbol", "AC", "C", "C", {"A": [0]}),
    ("vertical_sequence_index.test.cpp:373 referenceDoesNotAdaptSingleSymbolWhenSomeSymbolsAreMissing", "ANTNTTA", "T",
     "T", {"A": [0, 6]}),
    ("vertical_sequence_index.test.cpp:388 adaptsAndFlipsCorrectly", "ANTNATA", "T", "A", {"A": [], "T": [2, 5]}),
    ("vertical_sequence_index.test.cpp:412 adaptsAndFlipsCorrectlyWithManySymbols", "ANTNA---TA", "T", "-",
     {"A": [0, 4, 9], "T": [2, 8], "-": []}),
]

# Rows written to positions and read back (addSymbolsToPositions / overwriteSymbolsInSequences): the
# rows' symbols per position, as aligned sequences. The stored containers are checked through the
# SymbolEquals row sets: rows holding symbol c at position p.
STORED_SYMBOLS = [
    ("vertical_sequence_index.test.cpp:28 AddAndRetrieveSinglePosition", 0, "N", ["A", "C", "A", "C", "A"]),
    ("vertical_sequence_index.test.cpp:50 AddMultiplePositions", 0, "NNN", ["ACT", "AGT", "TGT"]),
    ("vertical_sequence_index.test.cpp:83 SelectiveRowRetrieval", 0, "GG", ["AC"] * 5),
    ("vertical_sequence_index.test.cpp:152 SingleSequence", 0, "TA", ["AT"]),
    ("vertical_sequence_index.test.cpp:170 LargeNumberOfSequences", 0, "NN", ["AG"] + ["AN"] * 69998 + ["AC"]),
    ("vertical_sequence_index.test.cpp:201 NonContiguousPositions", 0, "NNNNNNNNNNN", ["ANNNNCNNNNG"]),
    ("vertical_sequence_index.test.cpp:224 AllDifferentNucleotideSymbols", 0, "N", list("-ACGTRYSWKMBDHVN")),
    ("vertical_sequence_index.test.cpp:245 AllDifferentAminoAcidSymbols", 1, "X", list("-ACDEFGHIKLMNOPQRSTUVWYBJZ*X")),
    ("vertical_sequence_index.test.cpp:267 SparseRowSelection", 0, "N", ["B" if i % 2 == 0 else "Y" for i in range(100)]),
]


# ------------------------------------------------------------------------------------------------
# src/rhydb/query_engine/operators/union_all_node.test.cpp:10-47, 184-193 (UNION_ALL_OF_MUTATIONS):
# four rows with segment1 = "T" against the reference "A", countries CH, DE, CH, DE. The Mutations
# action with minProportion 0 of each country's rows gives one row, mutationTo T with proportion 1.
UNION_ALL = {
    "name": "union_all_node.test.cpp:184-193",
    "reference": "A",
    "rows": ["T", "T", "T", "T"],
    "country": ["CH", "DE", "CH", "DE"],
    # (filter, minProportion, [(position 1-based, from, to, count, coverage, proportion)])
    "cases": [
        ("StrEq(country,CH)", 0.0, [(1, "A", "T", 2, 2, 1.0)]),
        ("StrEq(country,DE)", 0.0, [(1, "A", "T", 2, 2, 1.0)]),
    ],
}
