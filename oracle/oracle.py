"""ctypes binding of the CPU oracle (test infrastructure only; see oracle.cpp)."""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"
_lib = None


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE), "liboracle.so"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < (HERE / "oracle.cpp").stat().st_mtime:
            build()
        L = C.CDLL(str(LIB_PATH))
        P, U32, U64, I, D, SZ = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int, C.c_double, C.c_size_t
        sig = {
            "oracle_last_error": (C.c_char_p, []),
            "oracle_build": (I, [P, C.POINTER(P)]),
            "oracle_free": (None, [P]),
            "oracle_count": (I, [P, C.c_char_p, C.POINTER(U64)]),
            "oracle_filter": (I, [P, C.c_char_p, P, C.POINTER(U64)]),
            "oracle_mutations": (I, [P, C.c_char_p, U32, P, C.POINTER(U64)]),
            "oracle_mutation_rows": (I, [P, U32, P, D, P, P, P, P, P, P, SZ, C.POINTER(SZ)]),
            "oracle_local_reference": (I, [P, U32, C.c_char_p]),
            "oracle_set_primary_key": (I, [P, C.c_char_p]),
            "oracle_vertical": (I, [P, U32, P, P, P, P, SZ, C.POINTER(SZ)]),
            "oracle_row_coverage": (I, [P, U32, U32, C.POINTER(U32), C.POINTER(U32), P, SZ, C.POINTER(SZ)]),
            "oracle_diff_string": (I, [I, C.c_char_p, C.c_char_p, C.POINTER(U32), C.POINTER(U32), P, C.POINTER(SZ), P,
                                       P, C.POINTER(SZ), SZ]),
            "oracle_operator": (I, [I, P, U32, P, P, U32, U32, U32, I, P, SZ, C.POINTER(SZ)]),
            "oracle_run_batch": (I, [P, P, P, P, U32, U32, P, P, C.POINTER(D)]),
            "oracle_check_batch": (I, [P, P, P, U32, U32, P, P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class OracleError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def _check(rc):
    if rc != 0:
        raise OracleError(rc, lib().oracle_last_error().decode(errors="replace"))


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class Oracle:
    """The oracle's own storage image, built from the raw table by its own ingestion."""

    def __init__(self, raw_table, n_chunks: int, columns):
        """raw_table: a ctypes RawTable (same layout as the product's). columns: [(name, n_symbols, L)]."""
        self._h = C.c_void_p()
        _check(lib().oracle_build(C.byref(raw_table), C.byref(self._h)))
        self.n_chunks = n_chunks
        self.columns = columns

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.oracle_free(self._h)
            self._h = None

    def count(self, expr: str) -> int:
        v = C.c_uint64()
        _check(lib().oracle_count(self._h, expr.encode(), C.byref(v)))
        return v.value

    def compute_filter(self, expr: str):
        bits = np.zeros(self.n_chunks * 2048, dtype=np.uint32)
        v = C.c_uint64()
        _check(lib().oracle_filter(self._h, expr.encode(), _p(bits), C.byref(v)))
        return bits, v.value

    def mutations(self, expr: str, column: int = 0):
        _, nsym, L = self.columns[column]
        counts = np.zeros((nsym, L), dtype=np.uint32)
        v = C.c_uint64()
        _check(lib().oracle_mutations(self._h, expr.encode(), column, _p(counts), C.byref(v)))
        return counts, v.value

    def mutation_rows(self, column: int, counts: np.ndarray, min_proportion: float):
        counts = np.ascontiguousarray(counts, dtype=np.uint32)
        n = C.c_size_t()
        z = np.zeros(1, dtype=np.uint32)
        _check(lib().oracle_mutation_rows(self._h, column, _p(counts), min_proportion, _p(z), _p(z), _p(z), _p(z),
                                          _p(z), _p(z), 0, C.byref(n)))
        m = n.value
        pos = np.zeros(max(m, 1), np.uint32)
        frm = np.zeros(max(m, 1), np.uint8)
        to = np.zeros(max(m, 1), np.uint8)
        cnt = np.zeros(max(m, 1), np.uint32)
        cov = np.zeros(max(m, 1), np.uint32)
        prop = np.zeros(max(m, 1), np.float64)
        _check(lib().oracle_mutation_rows(self._h, column, _p(counts), min_proportion, _p(pos), _p(frm), _p(to),
                                          _p(cnt), _p(cov), _p(prop), m, C.byref(n)))
        return [(int(pos[i]), chr(frm[i]), chr(to[i]), int(cnt[i]), int(cov[i]), float(prop[i])) for i in range(m)]

    def set_primary_key(self, dict_column):
        _check(lib().oracle_set_primary_key(self._h, None if dict_column is None else dict_column.encode()))

    def local_reference(self, column: int) -> str:
        L = self.columns[column][2]
        buf = C.create_string_buffer(L + 1)
        _check(lib().oracle_local_reference(self._h, column, buf))
        return buf.raw[:L].decode()

    def vertical(self, column: int):
        n = C.c_size_t()
        z = np.zeros(1, np.uint32)
        _check(lib().oracle_vertical(self._h, column, _p(z), _p(z), _p(z), _p(z), 0, C.byref(n)))
        m = n.value
        pos = np.zeros(m, np.uint32)
        v = np.zeros(m, np.uint16)
        sym = np.zeros(m, np.uint8)
        card = np.zeros(m, np.uint32)
        _check(lib().oracle_vertical(self._h, column, _p(pos), _p(v), _p(sym), _p(card), m, C.byref(n)))
        return pos, v, sym, card

    def row_coverage(self, column: int, row: int):
        s, e = C.c_uint32(), C.c_uint32()
        n = C.c_size_t()
        buf = np.zeros(2048, np.uint32)
        _check(lib().oracle_row_coverage(self._h, column, row, C.byref(s), C.byref(e), _p(buf), 2048, C.byref(n)))
        return s.value, e.value, [(int(buf[2 * i]), int(buf[2 * i + 1])) for i in range(n.value)]

    def run_batch(self, exprs, actions, columns, threads: int):
        """Times queries one per worker thread; returns (seconds, per-query ms, results)."""
        n = len(exprs)
        arr = (C.c_char_p * n)(*[e.encode() for e in exprs])
        act = np.asarray(actions, dtype=np.int32)
        col = np.asarray(columns, dtype=np.uint32)
        out = np.zeros(n, np.uint64)
        ms = np.zeros(n, np.float64)
        secs = C.c_double()
        _check(lib().oracle_run_batch(self._h, C.cast(arr, C.c_void_p), _p(act), _p(col), n, threads, _p(out),
                                      _p(ms), C.byref(secs)))
        return secs.value, ms, out

    def check_batch(self, exprs, columns=None, tables=None, threads: int = 0):
        """Counts of every expression and, for the indices in `tables`, the Mutations counts of
        columns[i], on `threads` worker threads (0: all cores). Returns (counts, {i: table})."""
        import os

        n = len(exprs)
        columns = np.zeros(n, np.uint32) if columns is None else np.asarray(columns, np.uint32)
        arr = (C.c_char_p * n)(*[e.encode() for e in exprs])
        counts = np.zeros(n, np.uint64)
        out = {}
        ptrs = (C.c_void_p * n)()
        for i in tables or ():
            _, nsym, L = self.columns[int(columns[i])]
            out[int(i)] = np.zeros((nsym, L), np.uint32)
            ptrs[int(i)] = out[int(i)].ctypes.data
        _check(lib().oracle_check_batch(self._h, C.cast(arr, C.c_void_p), _p(columns), n,
                                        threads or (os.cpu_count() or 1), _p(counts), C.cast(ptrs, C.c_void_p)))
        return counts, out


def diff_string(kind: int, seq: str, ref: str):
    """The reference's string diff: (start, end, missing positions, [(pos, symbol index)])."""
    n = len(seq)
    s, e = C.c_uint32(), C.c_uint32()
    nm, nmut = C.c_size_t(), C.c_size_t()
    miss = np.zeros(n + 1, np.uint32)
    mp = np.zeros(n + 1, np.uint32)
    ms = np.zeros(n + 1, np.uint8)
    _check(lib().oracle_diff_string(kind, seq.encode(), ref.encode(), C.byref(s), C.byref(e), _p(miss), C.byref(nm),
                                    _p(mp), _p(ms), C.byref(nmut), n + 1))
    return s.value, e.value, miss[: nm.value].tolist(), list(zip(mp[: nmut.value].tolist(), ms[: nmut.value].tolist()))


def operator(kind: int, chunk_sizes, pos_sets, neg_sets=(), n: int = 0, exact: bool = False):
    """Evaluates Threshold (0) / Intersection (1) / Union (2) / Complement (3) over explicit row sets."""
    sets = [sorted(set(s)) for s in list(pos_sets) + list(neg_sets)]
    off = np.zeros(len(sets) + 1, np.uint64)
    for i, s in enumerate(sets):
        off[i + 1] = off[i] + len(s)
    rows = np.array([x for s in sets for x in s] or [0], np.uint32)
    cs = np.asarray(chunk_sizes, np.uint32)
    out = np.zeros(1 << 20, np.uint32)
    m = C.c_size_t()
    _check(lib().oracle_operator(kind, _p(cs), len(cs), _p(rows), _p(off), len(pos_sets), len(neg_sets), n,
                                 int(exact), _p(out), out.size, C.byref(m)))
    return out[: m.value].tolist()
