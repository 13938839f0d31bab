"""Failure paths on the GPU in the form this pool allows: a bounded device wait is made to run out
(the filter kernel's leaf payload copies are announced but withheld, so nothing is left in flight),
the call returns an error status instead of hanging or trapping, and the handle's next calls
succeed with correct results."""
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


def _queries(table):
    return table.queries(40, seed=31)


def test_wait_that_gives_up_returns_an_error_and_the_handle_recovers(setup):
    table, dev, orc = setup
    qs = _queries(table)
    failed = []
    dev.test_withhold_copies(True)
    try:
        for q in qs:
            try:
                dev.mutations(q, 0)
            except R.RhyError as e:
                assert e.code == 3 and "gave up" in str(e), str(e)
                failed.append(q)
    finally:
        dev.test_withhold_copies(False)
    assert failed  # programs whose leaves stage payload copies wait on them
    # the next calls on the same handle succeed and agree with the oracle
    for q in failed[:5] + qs[:5]:
        m, n = dev.mutations(q, 0)
        om, on = orc.mutations(q, 0)
        assert n == on and np.array_equal(m, om), q
        assert dev.count(q) == orc.count(q)


def test_wait_failure_is_reported_once(setup):
    """A failed count and a failed row set report the error on their own call; the error flag is
    cleared, so the next call does not report it again."""
    table, dev, orc = setup
    qs = _queries(table)
    dev.test_withhold_copies(True)
    try:
        errors = 0
        for q in qs:
            for call in (lambda: dev.count(q), lambda: dev.compute_filter(q)):
                try:
                    call()
                except R.RhyError as e:
                    assert e.code == 3
                    errors += 1
    finally:
        dev.test_withhold_copies(False)
    assert errors > 0
    for q in qs:
        assert dev.count(q) == orc.count(q), q
