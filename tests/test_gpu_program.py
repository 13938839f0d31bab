"""The operator-tree entry points (rhy_program_*) on the GPU against the oracle: compiled trees of
seeded expressions over every column kind, the same trees combined with caller row sets, and the
Mutations action over an operator tree."""
import numpy as np
import pytest

import rhydb_gpu as R
from rawtable import oracle_for

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    t = R.Table.generate(150000, seed=17, n_aa_genes=12, null_fraction=0.003)
    orc = oracle_for(t)
    dev = R.Device(t, 0)
    yield t, orc, dev, t.queries(200, seed=18, use_aa=True, use_metadata=True)
    dev.close()


def test_compiled_trees_equal_the_expressions(setup):
    t, orc, dev, qs = setup
    for q in qs:
        nodes = t.program(q)
        bits, n = dev.program_eval(nodes)
        obits, on = orc.compute_filter(q)
        assert n == on and np.array_equal(bits, obits), q
        assert dev.program_count(nodes) == on, q


def test_trees_with_caller_row_sets(setup):
    """Intersection(tree, rows) and Union(tree; not rows) with a caller row set as an IndexScan leaf."""
    t, orc, dev, qs = setup
    rng = np.random.default_rng(19)
    for q in qs[:40]:
        lit = np.zeros(t.n_chunks * R.CHUNK_WORDS, np.uint32)
        rows = rng.choice(t.n_rows, 20000, replace=False)
        lit = R.rows_to_bits(rows, t.n_chunks)
        nodes = t.program(q)
        obits, _ = orc.compute_filter(q)
        both = nodes + [R.op_node(R.NODE_SCAN_ROWS, value=0),
                        R.op_node(R.NODE_INTERSECTION, n_children=2)]
        bits, n = dev.program_eval(both, [lit])
        want = obits & lit
        assert np.array_equal(bits, want) and n == int(R.bits_to_rows(want).size), q
        minus = nodes + [R.op_node(R.NODE_SCAN_ROWS, value=0),
                         R.op_node(R.NODE_INTERSECTION, n_children=2, n_negated=1)]
        bits, _ = dev.program_eval(minus, [lit])
        assert np.array_equal(bits, obits & ~lit), q


def test_mutations_over_operator_trees(setup):
    t, orc, dev, qs = setup
    rng = np.random.default_rng(20)
    for q in qs[:30]:
        col = int(rng.integers(0, t.n_seq))
        m, n = dev.program_mutations(t.program(q), col)
        om, on = orc.mutations(q, col)
        assert n == on and np.array_equal(m, om), (q, col)
