"""rhy_mutations_noalloc: the Mutations pass for callers that must not allocate device memory
during a query (their HBM belongs to their own pool, or the thread may not risk the
synchronisation of cudaMalloc / cudaFree). Its working memory is a fixed array in the device
image; its output must equal rhy_mutations' bit for bit, also when called twice in a row, since
every call reuses (and must re-clear) the same array.

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
    return d_filter, d_count, d_counts


def _run(torch, dev, table, column, query, bufs):
    d_filter, d_count, d_counts = bufs
    bits, n = dev.compute_filter(query)
    d_filter.copy_(torch.from_numpy(bits.view(np.int32)))
    d_count.fill_(n)
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    dev.mutations_noalloc(column, d_filter.data_ptr(), d_count.data_ptr(), d_counts.data_ptr(), stream.cuda_stream)
    torch.cuda.synchronize()
    col = table.columns[column]
    return d_counts.cpu().numpy().view(np.uint32).reshape(col.n_symbols, col.L)


def test_noalloc_matches_mutations_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    table = R.Table.generate(70000, seed=5, genome_len=4000, pool_sites=300, n_aa_genes=2, null_fraction=0.01)
    dev = R.Device(table, 0)
    queries = table.queries(4, seed=9, use_aa=True, use_metadata=True) + ["True"]
    for column in range(table.n_seq):
        bufs = _device_buffers(torch, table, column)
        for q in queries:
            expect, _ = dev.mutations(q, column)
            first = _run(torch, dev, table, column, q, bufs)
            second = _run(torch, dev, table, column, q, bufs)
            assert np.array_equal(first, expect), (q, column)
            assert np.array_equal(second, expect), (q, column)
    dev.close()


def test_noalloc_rejects_columns_above_its_limit():
    torch = pytest.importorskip("torch")
    table = R.Table.generate(3, seed=1, genome_len=131073, pool_sites=10)
    dev = R.Device(table, 0)
    bufs = _device_buffers(torch, table, 0)
    with pytest.raises(R.RhyError) as e:
        dev.mutations_noalloc(0, bufs[0].data_ptr(), bufs[1].data_ptr(), bufs[2].data_ptr())
    assert e.value.code == 4 and "at most 131072" in str(e.value)
    dev.close()
