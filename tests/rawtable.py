"""Builds raw tables (the C-ABI input format) from literal aligned sequences, and helpers shared
by the tests: a product table plus the oracle's own image of the same input."""
from __future__ import annotations

import ctypes as C

import numpy as np

import oracle as oracle_mod
import rhydb_gpu as R


class RawBuilder:
    """Owns the buffers behind a rhydb_gpu.RawTable built from Python data."""

    def __init__(self, n_rows: int):
        self.n_rows = n_rows
        self._keep = []
        self.seq = []
        self.dict = []
        self.date = []

    def _arr(self, a):
        self._keep.append(a)
        return a

    def add_sequences(self, name: str, kind: int, reference: str, rows: list):
        """rows: aligned sequence strings of len(reference), or None for a null row."""
        assert len(rows) == self.n_rows
        L = len(reference)
        is_null = np.zeros(self.n_rows, np.uint8)
        off = [0]
        pos, lens, chars = [], [], []
        for i, s in enumerate(rows):
            if s is None:
                is_null[i] = 1
                off.append(len(pos))
                continue
            assert len(s) == L, (len(s), L)
            p = 0
            while p < L:
                if s[p] == reference[p]:
                    p += 1
                    continue
                q = p
                while q < L and s[q] == s[p] and s[q] != reference[q]:
                    q += 1
                pos.append(p)
                lens.append(q - p)
                chars.append(s[p])
                p = q
            off.append(len(pos))
        col = R.RawSeqColumn()
        col.name = self._arr(C.create_string_buffer(name.encode())).value
        self._keep.append(name.encode())
        col.name = self._keep[-1]
        col.kind = kind
        ref_b = reference.encode()
        self._keep.append(ref_b)
        col.reference = ref_b
        col.L = L
        is_null = self._arr(is_null)
        off = self._arr(np.array(off, np.uint64))
        pos = self._arr(np.array(pos or [0], np.uint32))
        lens = self._arr(np.array(lens or [0], np.uint32))
        ch = self._arr(np.frombuffer(("".join(chars) or "A").encode(), np.uint8).copy())
        col.is_null = is_null.ctypes.data_as(C.POINTER(C.c_uint8))
        col.row_off = off.ctypes.data_as(C.POINTER(C.c_uint64))
        col.run_pos = pos.ctypes.data_as(C.POINTER(C.c_uint32))
        col.run_len = lens.ctypes.data_as(C.POINTER(C.c_uint32))
        col.run_char = ch.ctypes.data_as(C.POINTER(C.c_char))
        self.seq.append(col)
        return self

    def add_dict(self, name: str, values: list):
        """values: per-row string or None."""
        dictionary = sorted({v for v in values if v is not None})
        index = {v: i for i, v in enumerate(dictionary)}
        ids = self._arr(np.array([index[v] if v is not None else 0xFFFFFFFF for v in values], np.uint32))
        vals = [v.encode() for v in dictionary]
        self._keep.append(vals)
        arr = (C.c_char_p * max(1, len(vals)))(*vals)
        self._keep.append(arr)
        col = R.RawDictColumn()
        self._keep.append(name.encode())
        col.name = self._keep[-1]
        col.n_values = len(vals)
        col.values = arr
        col.ids = ids.ctypes.data_as(C.POINTER(C.c_uint32))
        self.dict.append(col)
        return self

    def add_dates(self, name: str, days: list):
        """days: per-row int (days since 1970-01-01) or None."""
        d = self._arr(np.array([x if x is not None else -(2 ** 31) for x in days], np.int32))
        col = R.RawDateColumn()
        self._keep.append(name.encode())
        col.name = self._keep[-1]
        col.days = d.ctypes.data_as(C.POINTER(C.c_int32))
        self.date.append(col)
        return self

    def raw(self) -> R.RawTable:
        t = R.RawTable()
        t.n_rows = self.n_rows
        t.n_seq, t.n_dict, t.n_date = len(self.seq), len(self.dict), len(self.date)
        s = (R.RawSeqColumn * max(1, len(self.seq)))(*self.seq)
        d = (R.RawDictColumn * max(1, len(self.dict)))(*self.dict)
        e = (R.RawDateColumn * max(1, len(self.date)))(*self.date)
        self._keep += [s, d, e]
        t.seq = C.cast(s, C.POINTER(R.RawSeqColumn))
        t.dict = C.cast(d, C.POINTER(R.RawDictColumn))
        t.date = C.cast(e, C.POINTER(R.RawDateColumn))
        self._keep.append(t)
        return t


def oracle_for(table: R.Table, raw=None) -> oracle_mod.Oracle:
    raw = raw if raw is not None else table.raw()
    return oracle_mod.Oracle(raw, table.n_chunks, [(c.name, c.n_symbols, c.L) for c in table.columns])


def date_days(iso: str) -> int:
    import datetime

    return (datetime.date.fromisoformat(iso) - datetime.date(1970, 1, 1)).days


def accession_table(n_rows: int = 300, L: int = 120, seed: int = 5):
    """A raw table with a primary-key dictionary column "accession": sequences drawn around a random
    reference (substitutions, ambiguity codes, leading / trailing / inner N runs, gaps, null rows),
    mostly unique accessions, two accessions shared by several rows (the first row counts), one
    held by a null row, some rows without one. Returns (builder, raw, accessions)."""
    rng = np.random.default_rng(seed)
    ref = "".join(rng.choice(list("ACGT"), L))
    rows = []
    for i in range(n_rows):
        if i % 37 == 5:
            rows.append(None)
            continue
        s = list(ref)
        for p in rng.choice(L, int(rng.integers(0, 12)), replace=False):
            s[p] = "ACGTRYKMN-"[rng.integers(10)]
        if rng.random() < 0.3:  # leading missing symbols
            k = int(rng.integers(1, 20))
            s[:k] = ["N"] * k
        if rng.random() < 0.3:  # trailing
            k = int(rng.integers(1, 20))
            s[L - k:] = ["N"] * k
        if rng.random() < 0.3:  # inside
            a, k = int(rng.integers(0, L - 10)), int(rng.integers(2, 10))
            s[a: a + k] = ["N"] * k
        assert len(s) == L
        rows.append("".join(s))
    acc = [f"seq_{i:04d}" for i in range(n_rows)]
    for i in (40, 41, 90):
        acc[i] = "shared_a"
    for i in (7, 200):
        acc[i] = "shared_b"
    acc[5] = "null_row"  # row 5 has no sequence
    for i in (11, 12):
        acc[i] = None
    b = RawBuilder(n_rows).add_sequences("main", 0, ref, rows).add_dict("accession", acc)
    return b, b.raw(), acc
