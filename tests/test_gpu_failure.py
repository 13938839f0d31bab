"""Failure paths on the GPU in the form this pool allows: a bounded device wait is made to run out
(the bulk copy it waits for is withheld, so nothing is left in flight), the call returns an error
status instead of hanging or trapping, and the handle's next calls succeed with correct results."""
import numpy as np
import pytest

import rhydb_gpu as R
from rawtable import oracle_for

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    table = R.Table.generate(140000, seed=21, genome_len=3000, pool_sites=300, null_fraction=0.01)
    dev = R.Device(table, 0)
    yield table, dev, oracle_for(table)
    dev.close()


def _dense_query(table, dev):
    """A filter of neither few rows nor every row: its Mutations action runs the container pass."""
    return next(q for q in table.queries(200, seed=31) if 0.2 * table.n_rows < dev.count(q) < 0.8 * table.n_rows)


def test_wait_that_gives_up_returns_an_error_and_the_handle_recovers(setup):
    table, dev, orc = setup
    q = _dense_query(table, dev)
    dev.test_withhold_copies(True)
    try:
        with pytest.raises(R.RhyError) as e:
            dev.mutations(q, 0)
    finally:
        dev.test_withhold_copies(False)
    assert e.value.code == 3 and "gave up" in str(e.value)
    # the next calls on the same handle succeed and agree with the oracle
    m, n = dev.mutations(q, 0)
    om, on = orc.mutations(q, 0)
    assert n == on and np.array_equal(m, om)
    assert dev.count(q) == orc.count(q)


def test_wait_failure_does_not_touch_filter_only_calls(setup):
    """Withholding affects only the container pass: counts and row sets are unaffected, and the
    error flag of a failed Mutations call is not reported again by a later call."""
    table, dev, orc = setup
    q = _dense_query(table, dev)
    dev.test_withhold_copies(True)
    try:
        assert dev.count(q) == orc.count(q)
        bits, n = dev.compute_filter(q)
        obits, on = orc.compute_filter(q)
        assert n == on and np.array_equal(bits, obits)
        with pytest.raises(R.RhyError):
            dev.mutations(q, 0)
    finally:
        dev.test_withhold_copies(False)
    assert dev.count(q) == orc.count(q)
