"""Failure paths on the GPU without a fault: a bounded device wait is made to run out (the filter
kernel's leaf payload copies, or the Mutations container pass's ring copies, are announced but
withheld, so nothing is left in flight), the call returns an error status instead of hanging or
trapping, and the handle's next calls succeed with correct results."""
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


def _dense_mutation_queries(table, orc):
    """Queries whose filter takes the container pass: neither empty nor every row, and above the
    single-query row-index limit (rows / 32)."""
    picks = [q for q in table.queries(80, seed=37) if table.n_rows // 16 < orc.count(q) < table.n_rows]
    assert picks
    return picks[:6]


def test_container_pass_wait_that_gives_up_returns_an_error_and_the_handle_recovers(setup):
    """The container pass's ring copies are announced but withheld: its consumers' waits give up,
    the call reports the device error, and the next calls agree with the oracle."""
    table, dev, orc = setup
    picks = _dense_mutation_queries(table, orc)
    dev.test_withhold_copies(False, container_pass=True)
    try:
        for q in picks:
            with pytest.raises(R.RhyError) as e:
                dev.mutations(q, 0)
            assert e.value.code == 3 and "gave up" in str(e.value) and "error 7" in str(e.value), str(e.value)
            assert dev.count(q) == orc.count(q)  # the filter kernels are unaffected
    finally:
        dev.test_withhold_copies(False)
    for q in picks:
        m, n = dev.mutations(q, 0)
        om, on = orc.mutations(q, 0)
        assert n == on and np.array_equal(m, om), q


def test_container_pass_wait_failure_reaches_the_no_alloc_status_word(setup):
    """rhy_mutations_noalloc reports a give-up of the container pass in the caller's status word
    (device error 7) and leaves the handle's own error flag clear; the next call reports 0."""
    torch = pytest.importorskip("torch")
    table, dev, orc = setup
    q = _dense_mutation_queries(table, orc)[0]
    col = table.columns[0]
    bits, n = dev.compute_filter(q)
    d_filter = torch.from_numpy(bits.view(np.int32)).to("cuda:0")
    d_count = torch.full((1,), n, dtype=torch.int64, device="cuda:0")
    d_counts = torch.zeros(col.n_symbols * col.L, dtype=torch.int32, device="cuda:0")
    d_status = torch.full((1,), -1, dtype=torch.int32, device="cuda:0")
    args = (0, d_filter.data_ptr(), d_count.data_ptr(), d_counts.data_ptr(), d_status.data_ptr(),
            torch.cuda.current_stream().cuda_stream)
    dev.test_withhold_copies(False, container_pass=True)
    try:
        dev.mutations_noalloc(*args)
        torch.cuda.synchronize()
        assert int(d_status.item()) == 7
    finally:
        dev.test_withhold_copies(False)
    assert dev.count(q) == orc.count(q)  # the handle's flag was not set by the failed pass
    dev.mutations_noalloc(*args)
    torch.cuda.synchronize()
    assert int(d_status.item()) == 0
    om, _ = orc.mutations(q, 0)
    assert np.array_equal(d_counts.cpu().numpy().view(np.uint32).reshape(col.n_symbols, col.L), om)
