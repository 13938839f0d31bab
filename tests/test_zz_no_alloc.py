"""rhy_mutations_noalloc: the Mutations pass for callers that must not allocate device memory
during a query (their HBM belongs to their own pool, or the thread may not risk the
synchronisation of cudaMalloc / cudaFree). Its working memory is a fixed array in the device
image; its output must equal rhy_mutations' bit for bit, also when called twice in a row, since
every call reuses (and must re-clear) the same array. The status word the caller owns is cleared by
every call and reads 0 after a successful one.

Collected last so that a run stopping at the first failure has run every other test first."""
import numpy as np
import pytest

import rhydb_gpu as R

pytestmark = pytest.mark.gpu


def _device_buffers(torch, table, column):
    col = table.columns[column]
    d_filter = torch.zeros(table.n_chunks * R.CHUNK_WORDS, dtype=torch.int32, device="cuda:0")
    d_count = torch.zeros(1, dtype=torch.int64, device="cuda:0")
    d_counts = torch.full((col.n_symbols * col.L,), -1, dtype=torch.int32, device="cuda:0")
    d_status = torch.full((1,), -1, dtype=torch.int32, device="cuda:0")
    return d_filter, d_count, d_counts, d_status


def _load_filter(torch, dev, query, bufs):
    d_filter, d_count = bufs[0], bufs[1]
    bits, n = dev.compute_filter(query)
    d_filter.copy_(torch.from_numpy(bits.view(np.int32)))
    d_count.fill_(n)
    torch.cuda.synchronize()


def _enqueue(torch, dev, column, bufs):
    d_filter, d_count, d_counts, d_status = bufs
    stream = torch.cuda.current_stream()
    dev.mutations_noalloc(column, d_filter.data_ptr(), d_count.data_ptr(), d_counts.data_ptr(), d_status.data_ptr(),
                          stream.cuda_stream)


def _result(torch, table, column, bufs):
    torch.cuda.synchronize()
    col = table.columns[column]
    counts = bufs[2].cpu().numpy().view(np.uint32).reshape(col.n_symbols, col.L)
    return counts, int(bufs[3].item())


def _run(torch, dev, table, column, query, bufs):
    _load_filter(torch, dev, query, bufs)
    _enqueue(torch, dev, column, bufs)
    return _result(torch, table, column, bufs)


@pytest.fixture(scope="module")
def small():
    torch = pytest.importorskip("torch")
    table = R.Table.generate(70000, seed=5, genome_len=4000, pool_sites=300, n_aa_genes=2, null_fraction=0.01)
    dev = R.Device(table, 0)
    yield torch, table, dev
    dev.close()


def test_noalloc_matches_mutations_on_consecutive_calls(small):
    torch, table, dev = small
    # a sparse filter (row-index pass), dense filters, the full table and an empty filter
    queries = table.queries(4, seed=9, use_aa=True, use_metadata=True) + ["True", "False", "SymEq(main,1,A)"]
    for column in range(table.n_seq):
        bufs = _device_buffers(torch, table, column)
        for q in queries:
            expect, _ = dev.mutations(q, column)
            first, st1 = _run(torch, dev, table, column, q, bufs)
            second, st2 = _run(torch, dev, table, column, q, bufs)
            assert st1 == 0 and st2 == 0, (q, column)
            assert np.array_equal(first, expect), (q, column)
            assert np.array_equal(second, expect), (q, column)


def test_noalloc_allocates_no_device_memory(small):
    """After one warm-up call (which loads the kernels and looks up the array's address), further
    calls leave the device's free memory unchanged."""
    torch, table, dev = small
    q = table.queries(1, seed=10, use_aa=True, use_metadata=True)[0]
    bufs = _device_buffers(torch, table, 0)
    _load_filter(torch, dev, q, bufs)
    _enqueue(torch, dev, 0, bufs)
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info(0)[0]
    for _ in range(5):
        _enqueue(torch, dev, 0, bufs)
    torch.cuda.synchronize()
    free_after = torch.cuda.mem_get_info(0)[0]
    assert free_after == free_before
    expect, _ = dev.mutations(q, 0)
    counts, status = _result(torch, table, 0, bufs)
    assert status == 0 and np.array_equal(counts, expect)


def test_noalloc_rejects_columns_above_its_limit():
    torch = pytest.importorskip("torch")
    table = R.Table.generate(3, seed=1, genome_len=131073, pool_sites=10)
    dev = R.Device(table, 0)
    bufs = _device_buffers(torch, table, 0)
    with pytest.raises(R.RhyError) as e:
        dev.mutations_noalloc(0, bufs[0].data_ptr(), bufs[1].data_ptr(), bufs[2].data_ptr(), bufs[3].data_ptr())
    assert e.value.code == 4 and "at most 131072" in str(e.value)
    dev.close()
