"""Chunk sharding of one table across ranks (one GPU per rank) and the one exchange step that
merges the per-shard results.

Every operator on the path is local to a 2^16-row chunk: And / Or / AndNot work key by key,
Complement works inside the chunk's own rows (reference: src/rhydb/storage/column/row_layout.cpp:18-23,
src/rhydb/query_engine/copy_on_write_bitmap.cpp:145-298), NOf counts per row. A table therefore
splits into contiguous chunk ranges, one per rank, and a query needs no exchange while it runs.
The results merge once:

* Count: the sum of the per-shard counts;
* Mutations: the element-wise sum of the per-shard count tables (|symbols| x L, u32), thresholded
  once on the merged table, since the threshold depends on the total per position
  (reference: src/rhydb/query_engine/operators/mutations_node.cpp:269-366);
* Details: the per-shard first-k ids, made global and concatenated in chunk order, first k kept.

Each shard is an ordinary table built from the rows of its range (`shard_raw`); chunk v of shard
s is chunk `first_chunk(s) + v` of the whole table, so a shard's local row id
`v << 16 | row` becomes the global id `(first_chunk + v) << 16 | row`.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

import rhydb_gpu as R

CHUNK_ROWS = 1 << 16


def chunk_ranges(n_rows: int, world: int) -> list[tuple[int, int]]:
    """Contiguous row ranges, one per rank, on chunk boundaries; chunks are dealt as evenly as
    possible (earlier ranks take the extra chunk). A rank may get an empty range."""
    if world < 1:
        raise ValueError("world size must be at least 1")
    n_chunks = (n_rows + CHUNK_ROWS - 1) // CHUNK_ROWS
    base, extra = divmod(n_chunks, world)
    out, c = [], 0
    for r in range(world):
        c1 = c + base + (1 if r < extra else 0)
        out.append((min(c * CHUNK_ROWS, n_rows), min(c1 * CHUNK_ROWS, n_rows)))
        c = c1
    return out


def _view(ptr, n: int, dtype) -> np.ndarray:
    if n == 0:
        return np.zeros(0, dtype)
    return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(np.ctypeslib.as_ctypes_type(dtype))), shape=(n,))


@dataclass
class ShardRaw:
    """A RawTable over rows [row_begin, row_end) of another RawTable, owning its buffers."""

    raw: R.RawTable
    row_begin: int
    row_end: int
    _keep: list = field(default_factory=list, repr=False)

    @property
    def first_chunk(self) -> int:
        return self.row_begin // CHUNK_ROWS


def shard_raw(raw: R.RawTable, row_begin: int, row_end: int) -> ShardRaw:
    """Copies rows [row_begin, row_end) of `raw` into a new RawTable. row_begin must sit on a chunk
    boundary so that the shard's chunks are whole chunks of the table (an empty range may sit
    anywhere). Dictionary value lists are
    shared with `raw`, which must stay alive until the shard's table is built."""
    n = raw.n_rows
    if not (0 <= row_begin <= row_end <= n) or (row_begin % CHUNK_ROWS and row_begin != row_end):
        raise ValueError(f"bad shard range [{row_begin}, {row_end}) of {n} rows")
    m = row_end - row_begin
    keep: list = []

    def own(a: np.ndarray) -> np.ndarray:
        a = np.ascontiguousarray(a).copy() if a.size else np.zeros(1, a.dtype)
        keep.append(a)
        return a

    seq = []
    for i in range(raw.n_seq):
        src = raw.seq[i]
        off = _view(src.row_off, n + 1, np.uint64)
        r0, r1 = int(off[row_begin]), int(off[row_end])
        col = R.RawSeqColumn()
        name, ref = src.name, src.reference
        keep += [name, ref]
        col.name, col.kind, col.reference, col.L = name, src.kind, ref, src.L
        col.is_null = own(_view(src.is_null, n, np.uint8)[row_begin:row_end]).ctypes.data_as(C.POINTER(C.c_uint8))
        col.row_off = own(off[row_begin:row_end + 1] - np.uint64(r0)).ctypes.data_as(C.POINTER(C.c_uint64))
        col.run_pos = own(_view(src.run_pos, r1, np.uint32)[r0:r1]).ctypes.data_as(C.POINTER(C.c_uint32))
        col.run_len = own(_view(src.run_len, r1, np.uint32)[r0:r1]).ctypes.data_as(C.POINTER(C.c_uint32))
        col.run_char = own(_view(src.run_char, r1, np.uint8)[r0:r1]).ctypes.data_as(C.POINTER(C.c_char))
        seq.append(col)
    dic = []
    for i in range(raw.n_dict):
        src = raw.dict[i]
        col = R.RawDictColumn()
        name = src.name
        keep.append(name)
        col.name, col.n_values, col.values = name, src.n_values, src.values
        col.ids = own(_view(src.ids, n, np.uint32)[row_begin:row_end]).ctypes.data_as(C.POINTER(C.c_uint32))
        dic.append(col)
    dat = []
    for i in range(raw.n_date):
        src = raw.date[i]
        col = R.RawDateColumn()
        name = src.name
        keep.append(name)
        col.name = name
        col.days = own(_view(src.days, n, np.int32)[row_begin:row_end]).ctypes.data_as(C.POINTER(C.c_int32))
        dat.append(col)

    t = R.RawTable()
    t.n_rows, t.n_seq, t.n_dict, t.n_date = m, len(seq), len(dic), len(dat)
    s = (R.RawSeqColumn * max(1, len(seq)))(*seq)
    d = (R.RawDictColumn * max(1, len(dic)))(*dic)
    e = (R.RawDateColumn * max(1, len(dat)))(*dat)
    keep += [s, d, e]
    t.seq = C.cast(s, C.POINTER(R.RawSeqColumn))
    t.dict = C.cast(d, C.POINTER(R.RawDictColumn))
    t.date = C.cast(e, C.POINTER(R.RawDateColumn))
    return ShardRaw(t, row_begin, row_end, keep)


def global_ids(local_ids, first_chunk: int) -> np.ndarray:
    """Shard-local row ids (chunk << 16 | row) to the whole table's ids."""
    ids = np.asarray(local_ids, dtype=np.uint32)
    return ids + np.uint32(first_chunk << 16)


def merge_counts(per_shard) -> int:
    return int(sum(int(c) for c in per_shard))


def merge_tables(per_shard) -> np.ndarray:
    """Element-wise sum of per-shard Mutations count tables. A position's total is at most the
    table's row count, so the u32 sum cannot wrap when every shard counts rows of one table."""
    out = None
    for t in per_shard:
        t = np.asarray(t, dtype=np.uint64)
        out = t.copy() if out is None else out + t
    if out is None:
        raise ValueError("no shards")
    if out.size and int(out.max()) > 0xFFFFFFFF:
        raise OverflowError("merged count exceeds u32")
    return out.astype(np.uint32)


def merge_details(per_shard_global_ids, k: int) -> np.ndarray:
    """First k ids of the whole table from each shard's first k (global ids, shards in chunk order)."""
    parts = [np.asarray(a, dtype=np.uint32) for a in per_shard_global_ids]
    ids = np.concatenate(parts) if parts else np.zeros(0, np.uint32)
    return ids[:k]


def all_reduce_count(count: int, group=None) -> int:
    """Count exchange over torch.distributed (any backend): the sum over ranks."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([int(count)], dtype=torch.int64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return int(t.item())


def all_reduce_table(table: np.ndarray, group=None) -> np.ndarray:
    """Mutations exchange: the element-wise sum of every rank's count table (summed in int64, checked
    against the u32 range)."""
    import torch
    import torch.distributed as dist

    t = torch.from_numpy(np.ascontiguousarray(table, dtype=np.int64))
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    out = t.numpy()
    if out.size and int(out.max()) > 0xFFFFFFFF:
        raise OverflowError("merged count exceeds u32")
    return out.astype(np.uint32)


def all_gather_details(global_ids, k: int, group=None) -> np.ndarray:
    """Details exchange: every rank's first k global ids gathered in rank (= chunk) order, first k
    kept."""
    import torch.distributed as dist

    world = dist.get_world_size(group)
    parts: list = [None] * world
    dist.all_gather_object(parts, np.asarray(global_ids, dtype=np.uint32)[:k].tolist(), group=group)
    return merge_details(parts, k)
