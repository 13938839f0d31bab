"""The reference's operator and row-set known answers (tests/golden/operator_cases.py) through the
CPU oracle, the host check of an operator tree (rhy_program_plan) and, with -m gpu, the operator-tree
entry point on the GPU (rhy_program_eval / rhy_program_count) with the row sets passed as IndexScan
leaves.

Not restated: the CopyOnWriteBitmap tests of ownership and copying (copy_on_write_bitmap.test.cpp:
113-128, 232-256) concern the lifetime of host containers, which row sets on the device do not
share; the iteration test (:187-202) is the ascending row order every expected list here has."""
import itertools

import numpy as np
import pytest

import oracle as oracle_mod
import rhydb_gpu as R
from golden import operator_cases as G

CHUNK = 1 << 16


def chunk_sizes(n_rows):
    return [CHUNK] * (n_rows // CHUNK) + ([n_rows % CHUNK] if n_rows % CHUNK else [])


def to_nodes(tree):
    """Postorder OpNodes of a case's tree."""
    kind = tree[0]
    if kind == "rows":
        return [R.op_node(R.NODE_SCAN_ROWS, value=tree[1])]
    if kind == "and":
        pos, neg = tree[1], tree[2]
        out = [n for c in pos + neg for n in to_nodes(c)]
        return out + [R.op_node(R.NODE_INTERSECTION, n_children=len(pos) + len(neg), n_negated=len(neg))]
    if kind == "or":
        out = [n for c in tree[1] for n in to_nodes(c)]
        return out + [R.op_node(R.NODE_UNION, n_children=len(tree[1]))]
    if kind == "not":
        return to_nodes(tree[1]) + [R.op_node(R.NODE_COMPLEMENT, n_children=1)]
    if kind == "threshold":
        n, exact, pos, neg = tree[1:]
        out = [n for c in pos + neg for n in to_nodes(c)]
        return out + [R.op_node(R.NODE_THRESHOLD, n_children=len(pos) + len(neg), n_negated=len(neg), value=n,
                                flags=int(exact))]
    raise ValueError(kind)


def trees(case):
    if case["tree"] == "permutations-of-or-4":
        return [("or", [("rows", i) for i in p]) for p in itertools.permutations(range(4))]
    return [case["tree"]]


def oracle_eval(case, tree):
    """The oracle's operators over explicit row sets (one operator over row-set leaves)."""
    cs, sets = chunk_sizes(case["n_rows"]), case["sets"]
    kind = tree[0]
    if kind == "rows":
        return sorted(sets[tree[1]])
    if kind == "and":
        return oracle_mod.operator(1, cs, [sets[c[1]] for c in tree[1]], [sets[c[1]] for c in tree[2]])
    if kind == "or":
        return oracle_mod.operator(2, cs, [sets[c[1]] for c in tree[1]])
    if kind == "not":
        return oracle_mod.operator(3, cs, [sets[tree[1][1]]])
    raise ValueError(kind)


_tables = {}


def table_of(n_rows):
    if n_rows not in _tables:
        _tables[n_rows] = R.Table.generate(n_rows, seed=3, genome_len=16, pool_sites=4)
    return _tables[n_rows]


def row_sets(case, table):
    return [R.rows_to_bits(s, table.n_chunks) for s in case["sets"]]


@pytest.mark.parametrize("case", G.CASES, ids=lambda c: c["name"])
def test_oracle_known_answer(case):
    for tree in trees(case):
        if case["expected"] == "compile_error":
            with pytest.raises(oracle_mod.OracleError):
                oracle_eval(case, tree)
        else:
            assert oracle_eval(case, tree) == case["expected"]


@pytest.mark.parametrize("case", [c for c in G.CASES if c["n_rows"] > 0], ids=lambda c: c["name"])
def test_operator_tree_checked_on_host(case):
    t = table_of(case["n_rows"])
    for tree in trees(case):
        if case["expected"] == "compile_error":
            with pytest.raises(R.QueryCompilationError):
                t.program_plan(to_nodes(tree), row_sets(case, t))
        else:
            text, n_instr, depth = t.program_plan(to_nodes(tree), row_sets(case, t))
            assert n_instr >= 1 and depth >= 1


def test_malformed_operator_trees_are_rejected_on_host():
    t = table_of(5)
    sets = [R.rows_to_bits([1, 2], t.n_chunks)]
    bad = [
        [R.op_node(R.NODE_INTERSECTION, n_children=2)],                                    # no operands
        [R.op_node(R.NODE_SCAN_ROWS), R.op_node(R.NODE_SCAN_ROWS)],                         # two results
        [R.op_node(R.NODE_SCAN_ROWS), R.op_node(R.NODE_SCAN_ROWS),
         R.op_node(R.NODE_THRESHOLD, n_children=2, value=2)],                               # n >= children
        [R.op_node(R.NODE_SCAN_ROWS), R.op_node(R.NODE_SCAN_ROWS),
         R.op_node(R.NODE_THRESHOLD, n_children=2, value=0)],                               # n == 0
        [R.op_node(R.NODE_SCAN_ROWS), R.op_node(R.NODE_COMPLEMENT, n_children=2)],          # arity
        [R.op_node(R.NODE_PRED_COVERED, column=0, position=1)],                             # a bare predicate
        [R.op_node(R.NODE_SCAN_ROWS), R.op_node(R.NODE_SELECTION, n_children=1)],          # no predicate
        [R.op_node(99)],                                                                     # unknown kind
        [],                                                                                  # empty
    ]
    for nodes in bad:
        with pytest.raises(R.QueryCompilationError):
            t.program_plan(nodes, sets)
    # references to things the table does not hold are user errors
    for nd in (R.op_node(R.NODE_SCAN_SEQ, column=5, position=0, symbols=1),
               R.op_node(R.NODE_SCAN_SEQ, column=0, position=16, symbols=1),
               R.op_node(R.NODE_SCAN_SEQ, column=0, position=0, symbols=1 << 20),
               R.op_node(R.NODE_SCAN_DICT, column=0, value=1 << 30)):
        with pytest.raises(R.IllegalQuery):
            t.program_plan([nd], sets)
    # a row set that was not passed, and one holding rows beyond the table
    with pytest.raises(R.RhyError) as e:
        t.program_plan([R.op_node(R.NODE_SCAN_ROWS, value=1)], sets)
    assert e.value.code == 4
    with pytest.raises(R.RhyError) as e:
        t.program_plan([R.op_node(R.NODE_SCAN_ROWS)], [R.rows_to_bits([7], t.n_chunks)])
    assert e.value.code == 4


def test_expression_trees_round_trip_through_nodes():
    """rhy_program_from_expr gives the compiled tree of an expression; checked on the host it prints
    the same operator tree as rhy_plan."""
    t = R.Table.generate(3000, seed=5, genome_len=500, pool_sites=50, n_aa_genes=2, null_fraction=0.01)
    for q in t.queries(200, seed=6, use_aa=True, use_metadata=True):
        tree, _, _ = t.plan(q)
        text, _, _ = t.program_plan(t.program(q))
        assert text == tree, q


@pytest.mark.gpu
@pytest.mark.parametrize("case", [c for c in G.CASES if c["n_rows"] > 0 and c["expected"] != "compile_error"],
                         ids=lambda c: c["name"])
def test_gpu_known_answer(case):
    t = table_of(case["n_rows"])
    dev = R.Device(t, 0)
    sets = row_sets(case, t)
    for tree in trees(case):
        bits, n = dev.program_eval(to_nodes(tree), sets)
        assert R.bits_to_rows(bits).tolist() == case["expected"]
        assert n == len(case["expected"])
        assert dev.program_count(to_nodes(tree), sets) == len(case["expected"])
    dev.close()
