"""Chunk sharding across ranks on the CPU: two `gloo` ranks each hold a chunk range of one table,
evaluate the same queries on their shard (the CPU oracle stands in for each rank's GPU), and merge
through the exchange step of lapis-silo_gb300/shard.py. The merged Count, Mutations count tables,
Mutations rows and Details ids must equal the whole table's."""
import multiprocessing as mp
import os
import socket
import traceback

import numpy as np
import pytest

import rhydb_gpu as R
import shard
from rawtable import oracle_for

ROWS = 2 * 65536 + 7000   # three chunks, the last one ragged
TABLE = dict(seed=7, genome_len=600, pool_sites=120, n_aa_genes=2, null_fraction=0.002)
K = 300                   # Details: first k ids
MIN_PROPORTION = 0.05


def _table():
    return R.Table.generate(ROWS, **TABLE)


def _queries(t):
    return t.queries(24, seed=11, use_aa=True, use_metadata=True) + [
        "True", "False", "Not(HasMut(main,5))", "Maybe(SymEq(main,17,R))", "NOf(2,atleast,HasMut(main,3),"
        "HasMut(main,30),HasMut(ORF1a,7))"]


def _first_k(bits, k):
    return R.bits_to_rows(bits)[:k]


def _shard_results(t, rank, world):
    """Per-query (count, [table per column], first-k global ids) on this rank's shard."""
    raw = t.raw()
    a, b = shard.chunk_ranges(t.n_rows, world)[rank]
    ncol = len(t.columns)
    out = []
    if a == b:   # a rank without rows contributes zeros and no ids
        for _ in _queries(t):
            out.append((0, [np.zeros((c.n_symbols, c.L), np.uint32) for c in t.columns], np.zeros(0, np.uint32)))
        return out
    sr = shard.shard_raw(raw, a, b)
    st = R.Table.from_raw(sr.raw)
    orc = oracle_for(st, sr.raw)
    for q in _queries(t):
        bits, cnt = orc.compute_filter(q)
        tables = [orc.mutations(q, c)[0] for c in range(ncol)]
        out.append((cnt, tables, shard.global_ids(_first_k(bits, K), sr.first_chunk)))
    return out


def _rank_main(rank, world, port, err_dir):
    try:
        import torch.distributed as dist

        os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
        dist.init_process_group("gloo", rank=rank, world_size=world)
        t = _table()
        mine = _shard_results(t, rank, world)
        merged = []
        for cnt, tables, ids in mine:
            merged.append((shard.all_reduce_count(cnt), [shard.all_reduce_table(x) for x in tables],
                           shard.all_gather_details(ids, K)))
        if rank == 0:
            full = oracle_for(t, t.raw())
            for q, (cnt, tables, ids) in zip(_queries(t), merged):
                bits, want = full.compute_filter(q)
                assert cnt == want, (q, cnt, want)
                assert np.array_equal(ids, _first_k(bits, K)), q
                for c, got in enumerate(tables):
                    ref = full.mutations(q, c)[0]
                    assert np.array_equal(got, ref), (q, c)
                    assert t.mutation_rows(c, got, MIN_PROPORTION) == full.mutation_rows(c, ref, MIN_PROPORTION), (q, c)
        dist.barrier()
        dist.destroy_process_group()
    except BaseException:
        with open(os.path.join(err_dir, f"rank{rank}.txt"), "w") as f:
            f.write(traceback.format_exc())
        raise


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_chunk_ranges():
    assert shard.chunk_ranges(ROWS, 1) == [(0, ROWS)]
    assert shard.chunk_ranges(ROWS, 2) == [(0, 131072), (131072, ROWS)]
    assert shard.chunk_ranges(ROWS, 3) == [(0, 65536), (65536, 131072), (131072, ROWS)]
    assert shard.chunk_ranges(ROWS, 4)[3] == (ROWS, ROWS)
    assert shard.chunk_ranges(65536, 2) == [(0, 65536), (65536, 65536)]
    with pytest.raises(ValueError):
        shard.chunk_ranges(ROWS, 0)
    for world in range(1, 6):
        r = shard.chunk_ranges(ROWS, world)
        assert r[0][0] == 0 and r[-1][1] == ROWS
        assert all(r[i][1] == r[i + 1][0] for i in range(world - 1))
        assert all(a % 65536 == 0 or a == b for a, b in r)


def test_shard_raw_rejects_unaligned_ranges():
    t = R.Table.generate(1000, seed=1, genome_len=100, pool_sites=10)
    raw = t.raw()
    for a, b in [(1, 10), (0, 1001), (-1, 5)]:
        with pytest.raises(ValueError):
            shard.shard_raw(raw, a, b)


def test_merges_in_one_process_four_shards():
    """Four shards (one of them empty) merged without a process group."""
    t = _table()
    full = oracle_for(t, t.raw())
    per_rank = [_shard_results(t, r, 4) for r in range(4)]
    spanning = 0
    for i, q in enumerate(_queries(t)):
        bits, want = full.compute_filter(q)
        assert shard.merge_counts(p[i][0] for p in per_rank) == want, q
        ids = shard.merge_details([p[i][2] for p in per_rank], K)
        assert np.array_equal(ids, _first_k(bits, K)), q
        spanning += len(set((ids >> 16).tolist())) > 1
        for c in range(len(t.columns)):
            got = shard.merge_tables([p[i][1][c] for p in per_rank])
            assert np.array_equal(got, full.mutations(q, c)[0]), (q, c)
    assert spanning > 0   # some first-k lists take ids from more than one shard


def test_two_gloo_ranks_reduce_to_the_whole_table(tmp_path):
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
    for p in procs:
        if p.is_alive():
            p.kill()
            p.join()
    errors = {f.name: f.read_text() for f in tmp_path.glob("rank*.txt")}
    assert not errors, errors
    assert [p.exitcode for p in procs] == [0, 0]
