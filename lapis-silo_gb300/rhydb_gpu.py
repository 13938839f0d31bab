"""Python mirror of the filter / count / mutations path over the C-ABI of librhygpu.so.

The names follow the reference's query engine: a filter expression is rewritten and compiled to
an operator tree (``Table.plan``), evaluated to a row set (``Device.compute_filter``,
reference: src/rhydb/query_engine/operators/compute_filter.cpp:14-21), counted
(``Device.count``, reference: count_filter_node.cpp:35-71), or turned into per-position symbol
counts and mutation rows (``Device.mutations``, reference: mutations_node.cpp:269-366).

There is no CPU fallback: if the compiled library is missing, importing works but every call
raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "librhygpu.so"

CHUNK_ROWS = 1 << 16
CHUNK_WORDS = CHUNK_ROWS // 32
NUC_SYMBOLS = "-ACGTRYSWKMBDHVN"
AA_SYMBOLS = "-ACDEFGHIKLMNOPQRSTUVWYBJZ*X"


class RhyError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


class IllegalQuery(RhyError):
    pass


class QueryCompilationError(RhyError):
    pass


class RawSeqColumn(C.Structure):
    _fields_ = [("name", C.c_char_p), ("kind", C.c_int), ("reference", C.c_char_p), ("L", C.c_uint32),
                ("is_null", C.POINTER(C.c_uint8)), ("row_off", C.POINTER(C.c_uint64)),
                ("run_pos", C.POINTER(C.c_uint32)), ("run_len", C.POINTER(C.c_uint32)),
                ("run_char", C.POINTER(C.c_char))]


class RawDictColumn(C.Structure):
    _fields_ = [("name", C.c_char_p), ("n_values", C.c_uint32), ("values", C.POINTER(C.c_char_p)),
                ("ids", C.POINTER(C.c_uint32))]


class RawDateColumn(C.Structure):
    _fields_ = [("name", C.c_char_p), ("days", C.POINTER(C.c_int32))]


class RawTable(C.Structure):
    _fields_ = [("n_rows", C.c_uint32), ("n_seq", C.c_uint32), ("n_dict", C.c_uint32), ("n_date", C.c_uint32),
                ("seq", C.POINTER(RawSeqColumn)), ("dict", C.POINTER(RawDictColumn)),
                ("date", C.POINTER(RawDateColumn))]


class BatchTimes(C.Structure):
    _fields_ = [("plan_ms", C.c_double), ("prepare_ms", C.c_double), ("device_ms", C.c_double),
                ("output_ms", C.c_double), ("compile_ms", C.c_double), ("predict_ms", C.c_double),
                ("lower_ms", C.c_double)]


class AggDimension(C.Structure):
    _fields_ = [("kind", C.c_int), ("column", C.c_uint32), ("position", C.c_uint32)]


class OpNode(C.Structure):
    """One node of a compiled operator tree in postorder (RhyOpNode)."""
    _fields_ = [("kind", C.c_uint32), ("n_children", C.c_uint32), ("n_negated", C.c_uint32), ("column", C.c_uint32),
                ("position", C.c_uint32), ("symbols", C.c_uint32), ("value", C.c_uint32), ("flags", C.c_uint32),
                ("date", C.c_int32), ("reserved", C.c_uint32)]


class OpProgram(C.Structure):
    _fields_ = [("nodes", C.POINTER(OpNode)), ("n_nodes", C.c_uint32), ("n_row_sets", C.c_uint32),
                ("row_sets", C.POINTER(C.c_void_p))]


# node kinds of the operator-tree entry points (the reference's Operator types)
NODE_EMPTY, NODE_FULL, NODE_SCAN_SEQ, NODE_SCAN_NULLS, NODE_SCAN_DICT, NODE_SCAN_ROWS = range(6)
NODE_INTERSECTION, NODE_UNION, NODE_COMPLEMENT, NODE_THRESHOLD, NODE_SELECTION = range(6, 11)
NODE_PRED_COVERED, NODE_PRED_DATE = 11, 12


def op_node(kind: int, **fields) -> OpNode:
    nd = OpNode()
    nd.kind = kind
    for k, v in fields.items():
        setattr(nd, k, v)
    return nd


class BatchSchedule(C.Structure):
    _fields_ = [("max_tile_bits", C.c_uint32), ("stack_kb", C.c_uint32), ("ctas_per_sm", C.c_uint32),
                ("query_major", C.c_uint32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class GenConfig(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("n_rows", C.c_uint32), ("genome_len", C.c_uint32),
                ("pool_sites", C.c_uint32), ("n_aa_genes", C.c_uint32), ("null_fraction", C.c_double),
                ("threads", C.c_uint32)]


class TableInfo(C.Structure):
    _fields_ = [("n_rows", C.c_uint32), ("n_chunks", C.c_uint32), ("n_seq", C.c_uint32), ("n_dict", C.c_uint32),
                ("n_date", C.c_uint32)]


class SeqColumnInfo(C.Structure):
    _fields_ = [("L", C.c_uint32), ("n_symbols", C.c_uint32), ("kind", C.c_uint32), ("flipped_positions", C.c_uint32),
                ("n_containers", C.c_uint64), ("payload_bytes", C.c_uint64), ("n_array", C.c_uint64),
                ("n_bitset", C.c_uint64), ("n_run", C.c_uint64), ("n_missing_intervals", C.c_uint64),
                ("n_coverage_exceptions", C.c_uint64), ("n_null_rows", C.c_uint64),
                ("n_row_index_entries", C.c_uint64)]


class BatchInfo(C.Structure):
    _fields_ = [("n_queries", C.c_uint32), ("n_mutation_slots", C.c_uint32), ("n_items", C.c_uint32),
                ("n_instr", C.c_uint32), ("max_depth", C.c_uint32), ("tile_bits", C.c_uint32), ("grid", C.c_uint32),
                ("device_bytes", C.c_uint64), ("n_filter_launches", C.c_uint32), ("filter_bytes", C.c_uint64)]


class PlannerStats(C.Structure):
    _fields_ = [("n_train", C.c_uint32), ("n_val", C.c_uint32), ("epochs", C.c_uint32),
                ("train_loss", C.c_float), ("val_loss", C.c_float),
                ("qerr_learned_median", C.c_float), ("qerr_rule_median", C.c_float),
                ("qerr_learned_p90", C.c_float), ("qerr_rule_p90", C.c_float),
                ("cost_err_median", C.c_float), ("train_ms", C.c_float), ("accepted", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class PlannerModel(C.Structure):
    _fields_ = [("weights", C.c_float * 5890), ("feature_mean", C.c_float * 24), ("feature_std", C.c_float * 24),
                ("target_mean", C.c_double * 2), ("target_std", C.c_double * 2), ("accepted", C.c_int)]


class ServerConfig(C.Structure):
    _fields_ = [("max_batch", C.c_uint32), ("streams", C.c_uint32), ("max_inflight", C.c_uint32),
                ("memory_budget", C.c_uint64), ("max_wait_ms", C.c_double), ("plain", C.c_uint32)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("rejected", C.c_uint64),
                ("batches", C.c_uint64), ("p50_ms", C.c_double), ("p99_ms", C.c_double),
                ("mean_batch", C.c_double), ("qps", C.c_double), ("peak_bytes", C.c_uint64),
                ("budget_bytes", C.c_uint64), ("peak_inflight", C.c_uint32), ("cancelled", C.c_uint64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


PLANNER_FEATURES = 24
MLP_NPARAM = 5890


class MutationRow(C.Structure):
    _fields_ = [("position", C.c_uint32), ("from_", C.c_char), ("to", C.c_char), ("count", C.c_uint32),
                ("coverage", C.c_uint32), ("proportion", C.c_double)]


_lib = None


def lib():
    """Loads librhygpu.so; raises if it was not built (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: build it with __graft_entry__.build() or lapis-silo_gb300/build.py")
    L = C.CDLL(str(LIB_PATH))
    P, U32, U64, I = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int
    sig = {
        "rhy_last_error": (C.c_char_p, []),
        "rhy_generate": (I, [C.POINTER(GenConfig), C.POINTER(P)]),
        "rhy_table_from_raw": (I, [C.POINTER(RawTable), U32, C.POINTER(P)]),
        "rhy_table_info": (I, [P, C.POINTER(TableInfo)]),
        "rhy_table_from_raw_gpu": (I, [C.POINTER(RawTable), I, U32, C.POINTER(P)]),
        "rhy_seq_column_checksum": (I, [P, U32, C.POINTER(U64)]),
        "rhy_table_set_primary_key": (I, [P, C.c_char_p]),
        "rhy_seq_column_info": (I, [P, U32, C.POINTER(SeqColumnInfo)]),
        "rhy_seq_column_name": (I, [P, U32, C.c_char_p, C.c_size_t]),
        "rhy_table_raw": (I, [P, C.POINTER(RawTable)]),
        "rhy_local_reference": (I, [P, U32, C.c_char_p, C.c_size_t]),
        "rhy_seq_containers": (I, [P, U32, P, P, P, P, P, C.c_size_t, C.POINTER(C.c_size_t)]),
        "rhy_container_pass_plan": (I, [P, U32, U32, P, C.c_size_t, C.POINTER(C.c_size_t), P, C.c_size_t,
                                        C.POINTER(C.c_size_t), P, C.c_size_t, C.POINTER(C.c_size_t)]),
        "rhy_generate_queries": (I, [P, U64, U32, U32, U32, U32, I, I, C.c_char_p, C.c_size_t, C.POINTER(C.c_size_t)]),
        "rhy_table_free": (None, [P]),
        "rhy_plan": (I, [P, C.c_char_p, C.c_char_p, C.c_size_t, C.POINTER(U32), C.POINTER(U32)]),
        "rhy_open": (I, [P, I, C.POINTER(P)]),
        "rhy_set_tile_bits": (I, [P, U32]),
        "rhy_device_bytes": (I, [P, C.POINTER(U64)]),
        "rhy_count": (I, [P, C.c_char_p, P, C.POINTER(U64)]),
        "rhy_eval": (I, [P, C.c_char_p, P, P, C.POINTER(U64)]),
        "rhy_mutations": (I, [P, C.c_char_p, U32, P, P, C.POINTER(U64)]),
        "rhy_program_from_expr": (I, [P, C.c_char_p, P, C.c_size_t, C.POINTER(C.c_size_t)]),
        "rhy_program_plan": (I, [P, P, C.c_char_p, C.c_size_t, C.POINTER(U32), C.POINTER(U32)]),
        "rhy_program_eval": (I, [P, P, P, P, C.POINTER(U64)]),
        "rhy_program_count": (I, [P, P, P, C.POINTER(U64)]),
        "rhy_program_mutations": (I, [P, P, U32, P, P, C.POINTER(U64)]),
        "rhy_mutation_rows": (I, [P, U32, P, C.c_double, C.POINTER(MutationRow), C.c_size_t, C.POINTER(C.c_size_t)]),
        "rhy_batch": (I, [P, P, P, P, U32, U32, P, P, P]),
        "rhy_batch_rows": (I, [P, P, P, P, P, U32, U32, P, P, P, C.c_size_t, P, P, C.POINTER(C.c_size_t)]),
        "rhy_batch_rows_fetch": (I, [P, P, P, C.c_size_t]),
        "rhy_batch_times": (I, [P, C.POINTER(BatchTimes)]),
        "rhy_sparse_rows": (I, [P, P, P]),
        "rhy_aggregate": (I, [P, C.c_char_p, P, U32, P, P, P, C.c_size_t, C.POINTER(C.c_size_t), C.POINTER(U64)]),
        "rhy_batch_schedule": (I, [P, C.POINTER(BatchSchedule), C.POINTER(BatchSchedule)]),
        "rhy_batch_autotune": (I, [P, P, P, P, U32, U32, P, C.POINTER(BatchSchedule), P, C.c_size_t,
                                   C.POINTER(C.c_size_t)]),
        "rhy_batch_prepare": (I, [P, P, P, P, U32, U32, U32]),
        "rhy_batch_launch": (I, [P, P, I, I]),
        "rhy_batch_capture": (I, [P, P]),
        "rhy_batch_replay": (I, [P, P]),
        "rhy_batch_results": (I, [P, P, P]),
        "rhy_batch_info": (I, [P, C.POINTER(BatchInfo)]),
        "rhy_plain_prepare": (I, [P, P, P, P, U32]),
        "rhy_plain_launch": (I, [P, U32, P]),
        "rhy_plain_launch_parts": (I, [P, U32, P, U32]),
        "rhy_mutation_bytes": (I, [P, U32, C.POINTER(U64), C.POINTER(U64)]),
        "rhy_batch_capture_ex": (I, [P, P, I, I]),
        "rhy_batch_launch_parts": (I, [P, P, U32]),
        "rhy_mutations_noalloc": (I, [P, U32, P, P, P, P, P]),
        "rhy_test_withhold_copies": (I, [P, I]),
        "rhy_plan_features": (I, [P, C.c_char_p, P, C.c_size_t, C.POINTER(C.c_size_t)]),
        "rhy_planner_collect": (I, [P, P, U32, C.POINTER(C.c_size_t)]),
        "rhy_planner_train": (I, [P, U32, U32, C.c_float, U64, C.POINTER(PlannerStats)]),
        "rhy_planner_mode": (I, [P, I]),
        "rhy_planner_samples": (I, [P, P, P, C.c_size_t, C.POINTER(C.c_size_t)]),
        "rhy_planner_weights": (I, [P, P]),
        "rhy_planner_export": (I, [P, C.POINTER(PlannerModel)]),
        "rhy_planner_import": (I, [P, C.POINTER(PlannerModel)]),
        "rhy_planner_evaluate": (I, [P, P, U32, C.POINTER(PlannerStats)]),
        "rhy_planner_predict": (I, [P, P, U32, P, P]),
        "rhy_mlp_gradient": (I, [P, P, P, P, U32, P, P, P]),
        "rhy_server_start": (I, [P, C.POINTER(ServerConfig), C.POINTER(P)]),
        "rhy_server_submit": (I, [P, C.c_char_p, I, U32, C.c_double, U32, C.POINTER(U64)]),
        "rhy_server_result": (I, [P, U64, C.c_double, C.POINTER(U64), P, C.c_size_t, C.POINTER(C.c_size_t), P,
                                  C.c_size_t, C.POINTER(C.c_size_t), C.POINTER(C.c_double)]),
        "rhy_server_stats": (I, [P, C.POINTER(ServerStats)]),
        "rhy_server_cancel": (I, [P, U64, C.POINTER(I)]),
        "rhy_server_replay": (I, [P, P, P, P, P, P, P, U32, P, C.POINTER(C.c_double)]),
        "rhy_server_stop": (None, [P]),
        "rhy_close": (None, [P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _check(rc: int):
    if rc == 0:
        return
    msg = lib().rhy_last_error().decode(errors="replace")
    if rc == 1:
        raise IllegalQuery(rc, msg)
    if rc == 2:
        raise QueryCompilationError(rc, msg)
    raise RhyError(rc, msg)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


@dataclass
class SeqColumnStats:
    name: str
    L: int
    n_symbols: int
    kind: int
    flipped_positions: int
    n_containers: int
    payload_bytes: int
    n_array: int
    n_bitset: int
    n_run: int
    n_missing_intervals: int
    n_coverage_exceptions: int
    n_null_rows: int
    n_row_index_entries: int

    @property
    def symbols(self) -> str:
        return NUC_SYMBOLS if self.kind == 0 else AA_SYMBOLS


class Table:
    """Host storage image of one partition (ingested and finalized)."""

    def __init__(self, handle):
        self._h = handle
        info = TableInfo()
        _check(lib().rhy_table_info(self._h, C.byref(info)))
        self.n_rows = info.n_rows
        self.n_chunks = info.n_chunks
        self.n_seq, self.n_dict, self.n_date = info.n_seq, info.n_dict, info.n_date
        self.columns = [self.column_stats(i) for i in range(self.n_seq)]

    @classmethod
    def generate(cls, n_rows: int, seed: int = 42, genome_len: int = 29903, pool_sites: int = 5000,
                 n_aa_genes: int = 0, null_fraction: float = 0.0, threads: int = 0) -> "Table":
        cfg = GenConfig(seed, n_rows, genome_len, pool_sites, n_aa_genes, null_fraction, threads)
        h = C.c_void_p()
        _check(lib().rhy_generate(C.byref(cfg), C.byref(h)))
        return cls(h)

    @classmethod
    def from_raw(cls, raw: RawTable, threads: int = 0) -> "Table":
        h = C.c_void_p()
        _check(lib().rhy_table_from_raw(C.byref(raw), threads, C.byref(h)))
        return cls(h)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.rhy_table_free(self._h)
            self._h = None

    @classmethod
    def from_raw_gpu(cls, raw: RawTable, device: int = 0, threads: int = 0) -> "Table":
        """The same table as from_raw, its sequence columns built on a GPU."""
        h = C.c_void_p()
        _check(lib().rhy_table_from_raw_gpu(C.byref(raw), device, threads, C.byref(h)))
        return cls(h)

    def checksum(self, column: int) -> int:
        """64-bit checksum of a sequence column's whole storage image."""
        v = C.c_uint64()
        _check(lib().rhy_seq_column_checksum(self._h, column, C.byref(v)))
        return v.value

    def set_primary_key(self, dict_column: str | None) -> None:
        """Names the dictionary column holding the primary key (MutProfileSequenceId)."""
        _check(lib().rhy_table_set_primary_key(self._h, None if dict_column is None else dict_column.encode()))

    def column_stats(self, i: int) -> SeqColumnStats:
        info = SeqColumnInfo()
        _check(lib().rhy_seq_column_info(self._h, i, C.byref(info)))
        buf = C.create_string_buffer(256)
        _check(lib().rhy_seq_column_name(self._h, i, buf, 256))
        return SeqColumnStats(buf.value.decode(), info.L, info.n_symbols, info.kind, info.flipped_positions,
                              info.n_containers, info.payload_bytes, info.n_array, info.n_bitset, info.n_run,
                              info.n_missing_intervals, info.n_coverage_exceptions, info.n_null_rows,
                              info.n_row_index_entries)

    def column_index(self, name: str) -> int:
        for i, c in enumerate(self.columns):
            if c.name == name:
                return i
        raise KeyError(name)

    def raw(self) -> RawTable:
        r = RawTable()
        _check(lib().rhy_table_raw(self._h, C.byref(r)))
        return r

    def local_reference(self, column: int) -> str:
        L = self.columns[column].L
        buf = C.create_string_buffer(L + 1)
        _check(lib().rhy_local_reference(self._h, column, buf, L + 1))
        return buf.raw[:L].decode()

    def containers(self, column: int):
        """(position, chunk, symbol, cardinality, encoding) of every vertical container."""
        n = C.c_size_t()
        _check(lib().rhy_seq_containers(self._h, column, None, None, None, None, None, 0, C.byref(n)))
        m = n.value
        pos, chunk = np.zeros(m, np.uint32), np.zeros(m, np.uint16)
        sym, card, typ = np.zeros(m, np.uint8), np.zeros(m, np.uint32), np.zeros(m, np.uint8)
        if m:
            _check(lib().rhy_seq_containers(self._h, column, _ptr(pos), _ptr(chunk), _ptr(sym), _ptr(card), _ptr(typ),
                                            m, C.byref(n)))
        return pos, chunk, sym, card, typ

    def container_pass_plan(self, column: int, ctas: int):
        """The Mutations container pass's plan for `ctas` CTAs: array units (n x 5: first element,
        elements, first descriptor, descriptors, chunk), bitset / run units (n x 4: kind, chunk,
        first element, descriptor) and CTA ranges (n x 6: a0, a1, o0, o1, v0, v1), as uint32 arrays."""
        na, no, nr = C.c_size_t(), C.c_size_t(), C.c_size_t()
        _check(lib().rhy_container_pass_plan(self._h, column, ctas, None, 0, C.byref(na), None, 0, C.byref(no), None, 0,
                                             C.byref(nr)))
        au = np.zeros((na.value, 5), np.uint32)
        ou = np.zeros((no.value, 4), np.uint32)
        rg = np.zeros((nr.value, 6), np.uint32)
        _check(lib().rhy_container_pass_plan(self._h, column, ctas, _ptr(au), max(na.value, 1), C.byref(na), _ptr(ou),
                                             max(no.value, 1), C.byref(no), _ptr(rg), max(nr.value, 1), C.byref(nr)))
        return au, ou, rg

    def queries(self, n: int, seed: int = 43, max_depth: int = 4, max_nof_children: int = 8, use_aa: bool = False,
                use_metadata: bool = False, max_leaves: int = 0) -> list[str]:
        """Seeded random filter expressions; max_leaves bounds the leaves per tree (0 = no limit)."""
        need = C.c_size_t()
        _check(lib().rhy_generate_queries(self._h, seed, n, max_depth, max_nof_children, max_leaves, int(use_aa),
                                          int(use_metadata), None, 0, C.byref(need)))
        buf = C.create_string_buffer(need.value)
        _check(lib().rhy_generate_queries(self._h, seed, n, max_depth, max_nof_children, max_leaves, int(use_aa),
                                          int(use_metadata), buf, need.value, None))
        return [q for q in buf.value.decode().split("\n") if q]

    def plan(self, expr: str) -> tuple[str, int, int]:
        """Operator tree of rewrite(NONE) + compile, program length and stack depth."""
        buf = C.create_string_buffer(1 << 20)
        n, d = C.c_uint32(), C.c_uint32()
        _check(lib().rhy_plan(self._h, expr.encode(), buf, 1 << 20, C.byref(n), C.byref(d)))
        return buf.value.decode(), n.value, d.value

    def program(self, expr: str) -> list:
        """The compiled operator tree of an expression as postorder OpNodes (rhy_program_from_expr)."""
        n = C.c_size_t()
        _check(lib().rhy_program_from_expr(self._h, expr.encode(), None, 0, C.byref(n)))
        nodes = (OpNode * max(1, n.value))()
        _check(lib().rhy_program_from_expr(self._h, expr.encode(), nodes, n.value, C.byref(n)))
        return list(nodes[: n.value])

    def program_plan(self, nodes, row_sets=None) -> tuple[str, int, int]:
        """Checks and lowers an operator tree on the host: its text, program length and stack depth."""
        prog, keep = _op_program(self, nodes, row_sets)
        buf = C.create_string_buffer(1 << 20)
        n, d = C.c_uint32(), C.c_uint32()
        _check(lib().rhy_program_plan(self._h, C.byref(prog), buf, 1 << 20, C.byref(n), C.byref(d)))
        return buf.value.decode(), n.value, d.value

    def plan_features(self, expr: str) -> np.ndarray:
        """Planner features of every operator node of the compiled expression (preorder)."""
        n = C.c_size_t()
        _check(lib().rhy_plan_features(self._h, expr.encode(), None, 0, C.byref(n)))
        x = np.zeros((max(n.value, 1), PLANNER_FEATURES), np.float32)
        _check(lib().rhy_plan_features(self._h, expr.encode(), _ptr(x), n.value, C.byref(n)))
        return x[:n.value]

    def mutation_rows(self, column: int, counts: np.ndarray, min_proportion: float):
        """Rows of the Mutations action (reference: mutations_node.cpp:292-366) from symbol counts."""
        counts = np.ascontiguousarray(counts, dtype=np.uint32)
        n = C.c_size_t()
        _check(lib().rhy_mutation_rows(self._h, column, _ptr(counts), min_proportion, None, 0, C.byref(n)))
        rows = (MutationRow * max(1, n.value))()
        _check(lib().rhy_mutation_rows(self._h, column, _ptr(counts), min_proportion, rows, n.value, C.byref(n)))
        return [(r.position, r.from_.decode(), r.to.decode(), r.count, r.coverage, r.proportion)
                for r in rows[: n.value]]


class Device:
    """A partition resident in the HBM of one GPU."""

    def __init__(self, table: Table, device: int = 0):
        self.table = table
        self._h = C.c_void_p()
        _check(lib().rhy_open(table._h, device, C.byref(self._h)))

    def close(self):
        if getattr(self, "_h", None):
            lib().rhy_close(self._h)
            self._h = None

    def __del__(self):
        if _lib is not None:
            self.close()

    def set_tile_bits(self, bits: int):
        _check(lib().rhy_set_tile_bits(self._h, bits))

    def device_bytes(self) -> int:
        v = C.c_uint64()
        _check(lib().rhy_device_bytes(self._h, C.byref(v)))
        return v.value

    def count(self, expr: str, stream=None) -> int:
        v = C.c_uint64()
        _check(lib().rhy_count(self._h, expr.encode(), stream, C.byref(v)))
        return v.value

    def compute_filter(self, expr: str, stream=None) -> tuple[np.ndarray, int]:
        """Dense row-set bitmap (n_chunks * 2048 uint32 words) and its cardinality."""
        bits = np.zeros(self.table.n_chunks * CHUNK_WORDS, dtype=np.uint32)
        v = C.c_uint64()
        _check(lib().rhy_eval(self._h, expr.encode(), stream, _ptr(bits), C.byref(v)))
        return bits, v.value

    def mutations(self, expr: str, column: int = 0, stream=None) -> tuple[np.ndarray, int]:
        """counts[symbol, position] of the filtered rows and the filter cardinality."""
        col = self.table.columns[column]
        counts = np.zeros((col.n_symbols, col.L), dtype=np.uint32)
        v = C.c_uint64()
        _check(lib().rhy_mutations(self._h, expr.encode(), column, stream, _ptr(counts), C.byref(v)))
        return counts, v.value

    # ---- compiled operator trees (Operator::evaluate and the actions over it) ----
    def _program(self, nodes, row_sets):
        return _op_program(self.table, nodes, row_sets)

    def program_eval(self, nodes, row_sets=None, stream=None) -> tuple[np.ndarray, int]:
        prog, keep = self._program(nodes, row_sets)
        bits = np.zeros(self.table.n_chunks * CHUNK_WORDS, dtype=np.uint32)
        v = C.c_uint64()
        _check(lib().rhy_program_eval(self._h, C.byref(prog), stream, _ptr(bits), C.byref(v)))
        return bits, v.value

    def program_count(self, nodes, row_sets=None, stream=None) -> int:
        prog, keep = self._program(nodes, row_sets)
        v = C.c_uint64()
        _check(lib().rhy_program_count(self._h, C.byref(prog), stream, C.byref(v)))
        return v.value

    def program_mutations(self, nodes, column: int = 0, row_sets=None, stream=None) -> tuple[np.ndarray, int]:
        prog, keep = self._program(nodes, row_sets)
        col = self.table.columns[column]
        counts = np.zeros((col.n_symbols, col.L), dtype=np.uint32)
        v = C.c_uint64()
        _check(lib().rhy_program_mutations(self._h, C.byref(prog), column, stream, _ptr(counts), C.byref(v)))
        return counts, v.value

    # ---- batched path ----
    @staticmethod
    def _query_arrays(exprs, actions, columns):
        n = len(exprs)
        arr = _text_array(exprs)
        act = np.asarray(actions if actions is not None else [0] * n, dtype=np.int32)
        col = np.asarray(columns if columns is not None else [0] * n, dtype=np.uint32)
        return n, arr, act, col

    def batch(self, exprs, actions=None, columns=None, tile_bits: int = 0, stream=None):
        """Evaluates many queries in one launch sequence. Returns (filter counts, {i: counts[symbol, position]})."""
        n, arr, act, col = self._query_arrays(exprs, actions, columns)
        counts = np.zeros(max(n, 1), np.uint64)
        outs = {}
        ptrs = (C.c_void_p * max(n, 1))()
        for i in range(n):
            if act[i] == 1:
                c = self.table.columns[int(col[i])]
                outs[i] = np.zeros((c.n_symbols, c.L), np.uint32)
                ptrs[i] = outs[i].ctypes.data
        _check(lib().rhy_batch(self._h, C.cast(arr, C.c_void_p), _ptr(act), _ptr(col), n, tile_bits, stream,
                               _ptr(counts), C.cast(ptrs, C.c_void_p)))
        return counts[:n], outs

    ROW_DTYPE = np.dtype({"names": ["position", "from_", "to", "count", "coverage", "proportion"],
                          "formats": [np.uint32, "S1", "S1", np.uint32, np.uint32, np.float64],
                          "offsets": [0, 4, 5, 8, 12, 16], "itemsize": 24})

    def batch_rows(self, exprs, actions=None, columns=None, min_proportions=None, tile_bits: int = 0, stream=None,
                   rows_cap: int = 1 << 20):
        """Batch with the Mutations output computed on the device. Returns (filter counts, rows,
        row_begin, row_count): query i's rows are rows[row_begin[i]:row_begin[i] + row_count[i]], a
        structured array with the fields of RhyMutationRow."""
        n, arr, act, col = self._query_arrays(exprs, actions, columns)
        counts = np.zeros(max(n, 1), np.uint64)
        begin = np.zeros(max(n, 1), np.uint64)
        cnt = np.zeros(max(n, 1), np.uint32)
        mp = None if min_proportions is None else np.ascontiguousarray(min_proportions, dtype=np.float64)
        rows = np.empty(max(rows_cap, 1), self.ROW_DTYPE)  # written by the library up to the row count
        total = C.c_size_t()
        _check(lib().rhy_batch_rows(self._h, C.cast(arr, C.c_void_p), _ptr(act), _ptr(col),
                                    None if mp is None else _ptr(mp), n, tile_bits, stream, _ptr(counts),
                                    rows.ctypes.data, rows_cap, _ptr(begin), _ptr(cnt), C.byref(total)))
        if total.value > rows_cap:
            rows = np.zeros(total.value, self.ROW_DTYPE)
            _check(lib().rhy_batch_rows_fetch(self._h, stream, rows.ctypes.data, total.value))
        return counts[:n], rows[:total.value], begin[:n], cnt[:n]

    def batch_times(self) -> dict:
        """Host wall time (ms) of the phases of the last batch_rows call."""
        t = BatchTimes()
        _check(lib().rhy_batch_times(self._h, C.byref(t)))
        return {k: t.__getattribute__(k) for k, _ in BatchTimes._fields_}

    def batch_prepare(self, exprs, actions=None, columns=None, tile_bits: int = 0, plan_threads: int = 0):
        n, arr, act, col = self._query_arrays(exprs, actions, columns)
        self._batch_n = n
        self._batch_act, self._batch_col = act, col
        _check(lib().rhy_batch_prepare(self._h, C.cast(arr, C.c_void_p), _ptr(act), _ptr(col), n, tile_bits,
                                       plan_threads))

    def batch_launch(self, stream=None, copy_in: bool = True, copy_out: bool = True):
        _check(lib().rhy_batch_launch(self._h, stream, int(copy_in), int(copy_out)))

    def batch_capture(self, stream=None):
        _check(lib().rhy_batch_capture(self._h, stream))

    def batch_replay(self, stream=None):
        _check(lib().rhy_batch_replay(self._h, stream))

    def batch_results(self, with_mutations: bool = True):
        n = self._batch_n
        counts = np.zeros(max(n, 1), np.uint64)
        outs = {}
        ptrs = (C.c_void_p * max(n, 1))()
        if with_mutations:
            for i in range(n):
                if self._batch_act[i] == 1:
                    c = self.table.columns[int(self._batch_col[i])]
                    outs[i] = np.zeros((c.n_symbols, c.L), np.uint32)
                    ptrs[i] = outs[i].ctypes.data
        _check(lib().rhy_batch_results(self._h, _ptr(counts), C.cast(ptrs, C.c_void_p)))
        return counts[:n], outs

    def aggregate(self, expr: str, dims, stream=None):
        """Grouped counts of the filter's rows (BitmapAggregation). dims: ("seq", column, 1-based
        position) or ("dict", column) per dimension. Returns ([(group label per dimension, count)],
        filter count) in the reference's order; labels are symbol characters or dictionary values,
        None for the null group."""
        nd = len(dims)
        arr = (AggDimension * max(nd, 1))()
        for i, d in enumerate(dims):
            if d[0] == "seq":
                arr[i] = AggDimension(0, int(d[1]), int(d[2]))
            elif d[0] == "dict":
                arr[i] = AggDimension(1, int(d[1]), 0)
            else:
                raise ValueError(f"unknown dimension kind {d[0]!r}")
        n = C.c_size_t()
        fc = C.c_uint64()
        _check(lib().rhy_aggregate(self._h, expr.encode(), arr, nd, stream, None, None, 0, C.byref(n), C.byref(fc)))
        m = n.value
        groups = np.zeros(max(m * nd, 1), np.int32)
        counts = np.zeros(max(m, 1), np.uint64)
        _check(lib().rhy_aggregate(self._h, expr.encode(), arr, nd, stream, _ptr(groups), _ptr(counts), m, C.byref(n),
                                   C.byref(fc)))
        raw = self.table.raw()
        out = []
        for i in range(m):
            labels = []
            for j, d in enumerate(dims):
                g = int(groups[i * nd + j])
                if g < 0:
                    labels.append(None)
                elif d[0] == "seq":
                    labels.append(self.table.columns[int(d[1])].symbols[g])
                else:
                    labels.append(raw.dict[int(d[1])].values[g].decode())
            out.append((tuple(labels), int(counts[i])))
        return out, fc.value

    def sparse_rows(self, plain=None, batch=None) -> tuple:
        """Row limits of the row-index Mutations path (single queries, batch slots); arguments set
        them first (0 turns the path off)."""
        cur = np.zeros(2, np.uint64)
        _check(lib().rhy_sparse_rows(self._h, None, _ptr(cur)))
        if plain is not None or batch is not None:
            new = np.array([cur[0] if plain is None else plain, cur[1] if batch is None else batch], np.uint64)
            _check(lib().rhy_sparse_rows(self._h, _ptr(new), _ptr(cur)))
        return int(cur[0]), int(cur[1])

    def batch_schedule(self, **set_fields) -> dict:
        """The schedule of the batched filter launches; keyword arguments set fields first."""
        cur = BatchSchedule()
        _check(lib().rhy_batch_schedule(self._h, None, C.byref(cur)))
        if set_fields:
            for k, v in set_fields.items():
                setattr(cur, k, v)
            _check(lib().rhy_batch_schedule(self._h, C.byref(cur), C.byref(cur)))
        return cur.as_dict()

    def batch_autotune(self, exprs, actions=None, columns=None, reps: int = 5, stream=None) -> list:
        """Times every candidate schedule on this batch and keeps the fastest; returns
        [(schedule dict, median ms)] fastest first."""
        n, arr, act, col = self._query_arrays(exprs, actions, columns)
        cap = 128
        tried = (BatchSchedule * cap)()
        ms = np.zeros(cap, np.float64)
        nt = C.c_size_t()
        _check(lib().rhy_batch_autotune(self._h, C.cast(arr, C.c_void_p), _ptr(act), _ptr(col), n, reps, stream, tried,
                                        _ptr(ms), cap, C.byref(nt)))
        return [(tried[i].as_dict(), float(ms[i])) for i in range(min(nt.value, cap))]

    def batch_info(self) -> BatchInfo:
        info = BatchInfo()
        _check(lib().rhy_batch_info(self._h, C.byref(info)))
        return info

    def plain_prepare(self, exprs, actions=None, columns=None):
        n, arr, act, col = self._query_arrays(exprs, actions, columns)
        _check(lib().rhy_plain_prepare(self._h, C.cast(arr, C.c_void_p), _ptr(act), _ptr(col), n))

    def plain_launch(self, i: int, stream=None, parts: int = 15):
        _check(lib().rhy_plain_launch_parts(self._h, i, stream, parts))

    def batch_capture_ex(self, stream=None, copy_in: bool = False, copy_out: bool = False):
        _check(lib().rhy_batch_capture_ex(self._h, stream, int(copy_in), int(copy_out)))

    def batch_launch_parts(self, parts: int, stream=None):
        _check(lib().rhy_batch_launch_parts(self._h, stream, parts))

    def mutations_noalloc(self, column: int, d_filter: int, d_filter_count: int, d_counts: int, d_status: int,
                          stream=None):
        """Mutations pass over caller-owned device buffers (addresses as ints); allocates nothing.
        Enqueued on `stream`; synchronise it before reading d_counts and the int at d_status (0
        after a completed pass)."""
        _check(lib().rhy_mutations_noalloc(self._h, column, C.c_void_p(d_filter), C.c_void_p(d_filter_count),
                                           C.c_void_p(d_counts), C.c_void_p(d_status), stream))

    def test_withhold_copies(self, on: bool, container_pass: bool = False):
        """Testing only: the filter kernels (on) and the Mutations container pass (container_pass)
        withhold the bulk copies their bounded waits expect, so those waits give up and the calls
        report device error 6 (filter) or 7 (container pass); nothing is left in flight."""
        _check(lib().rhy_test_withhold_copies(self._h, (1 if on else 0) | (2 if container_pass else 0)))

    # ---- learned planner ----
    def planner_collect(self, exprs) -> int:
        arr = _text_array(exprs)
        n = C.c_size_t()
        _check(lib().rhy_planner_collect(self._h, C.cast(arr, C.c_void_p), len(exprs), C.byref(n)))
        return n.value

    def planner_train(self, epochs: int = 60, batch: int = 1024, lr: float = 2e-3, seed: int = 1) -> dict:
        st = PlannerStats()
        _check(lib().rhy_planner_train(self._h, epochs, batch, lr, seed, C.byref(st)))
        return st.as_dict()

    def planner_mode(self, mode: int):
        _check(lib().rhy_planner_mode(self._h, mode))

    def planner_samples(self):
        n = C.c_size_t()
        _check(lib().rhy_planner_samples(self._h, None, None, 0, C.byref(n)))
        x = np.zeros((max(n.value, 1), PLANNER_FEATURES), np.float32)
        y = np.zeros((max(n.value, 1), 3), np.float32)
        _check(lib().rhy_planner_samples(self._h, _ptr(x), _ptr(y), n.value, C.byref(n)))
        return x[:n.value], y[:n.value]

    def planner_predict(self, x: np.ndarray):
        x = np.ascontiguousarray(x, np.float32)
        n = x.shape[0]
        sel = np.zeros(max(n, 1), np.float64)
        cost = np.zeros(max(n, 1), np.float64)
        _check(lib().rhy_planner_predict(self._h, _ptr(x), n, _ptr(sel), _ptr(cost)))
        return sel[:n], cost[:n]

    def planner_weights(self) -> np.ndarray:
        w = np.zeros(MLP_NPARAM, np.float32)
        _check(lib().rhy_planner_weights(self._h, _ptr(w)))
        return w

    def planner_export(self) -> PlannerModel:
        m = PlannerModel()
        _check(lib().rhy_planner_export(self._h, C.byref(m)))
        return m

    def planner_import(self, model: PlannerModel):
        _check(lib().rhy_planner_import(self._h, C.byref(model)))

    def planner_evaluate(self, exprs) -> dict:
        """Judges the current network on traces of these expressions on this device (the verdict
        replaces the acceptance)."""
        arr = _text_array(exprs)
        st = PlannerStats()
        _check(lib().rhy_planner_evaluate(self._h, C.cast(arr, C.c_void_p), len(exprs), C.byref(st)))
        return st.as_dict()

    def mlp_gradient(self, w: np.ndarray, x: np.ndarray, t: np.ndarray):
        """One forward + backward of the planner network on the device: (gradient, loss, outputs)."""
        w = np.ascontiguousarray(w, np.float32)
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        n = x.shape[0]
        grad = np.zeros(MLP_NPARAM, np.float32)
        loss = np.zeros(1, np.float32)
        y = np.zeros((max(n, 1), 2), np.float32)
        _check(lib().rhy_mlp_gradient(self._h, _ptr(w), _ptr(x), _ptr(t), n, _ptr(grad), _ptr(loss), _ptr(y)))
        return grad, float(loss[0]), y[:n]

    def mutation_bytes(self, column: int = 0) -> tuple[int, int]:
        p, d = C.c_uint64(), C.c_uint64()
        _check(lib().rhy_mutation_bytes(self._h, column, C.byref(p), C.byref(d)))
        return p.value, d.value


class Server:
    """Continuous-batching request loop over a Device (rhy_server_*)."""

    def __init__(self, device: "Device", max_batch: int = 0, streams: int = 0, max_inflight: int = 0,
                 memory_budget: int = 0, max_wait_ms: float = -1.0, plain: bool = False):
        cfg = ServerConfig(max_batch, streams, max_inflight, memory_budget, max_wait_ms, int(plain))
        h = C.c_void_p()
        _check(lib().rhy_server_start(device._h, C.byref(cfg), C.byref(h)))
        self._h = h
        self.device = device

    def submit(self, expr: str, action: int = 0, column: int = 0, min_proportion: float = 0.05, k: int = 1000) -> int:
        i = C.c_uint64()
        _check(lib().rhy_server_submit(self._h, expr.encode(), action, column, min_proportion, k, C.byref(i)))
        return i.value

    def result(self, rid: int, timeout_ms: float = -1.0) -> dict:
        rows_cap, ids_cap = 4096, 1024
        while True:
            rows = np.zeros(rows_cap, Device.ROW_DTYPE)
            ids = np.zeros(ids_cap, np.uint32)
            cnt, nr, ni, lat = C.c_uint64(), C.c_size_t(), C.c_size_t(), C.c_double()
            rc = lib().rhy_server_result(self._h, rid, timeout_ms, C.byref(cnt), rows.ctypes.data, rows_cap,
                                         C.byref(nr), ids.ctypes.data, ids_cap, C.byref(ni), C.byref(lat))
            if rc == 4 and (nr.value > rows_cap or ni.value > ids_cap):
                rows_cap, ids_cap = max(rows_cap, nr.value), max(ids_cap, ni.value)
                continue
            _check(rc)
            return {"count": cnt.value, "rows": rows[:nr.value], "ids": ids[:ni.value], "latency_ms": lat.value}

    def replay(self, exprs, actions, columns, min_proportions, ks, arrival_s):
        """Open-loop replay (native submitter thread): (latencies in ms, wall seconds)."""
        n = len(exprs)
        arr = _text_array(exprs)
        act = np.ascontiguousarray(actions, np.int32)
        col = np.ascontiguousarray(columns, np.uint32)
        mp = np.ascontiguousarray(min_proportions, np.float64)
        k = np.ascontiguousarray(ks, np.uint32)
        at = np.ascontiguousarray(arrival_s, np.float64)
        lat = np.zeros(max(n, 1), np.float64)
        wall = C.c_double()
        _check(lib().rhy_server_replay(self._h, C.cast(arr, C.c_void_p), _ptr(act), _ptr(col), _ptr(mp), _ptr(k),
                                       _ptr(at), n, _ptr(lat), C.byref(wall)))
        return lat[:n], wall.value

    def cancel(self, rid: int) -> bool:
        """Cancels a request that is not done; False if it had already finished."""
        v = C.c_int()
        _check(lib().rhy_server_cancel(self._h, rid, C.byref(v)))
        return bool(v.value)

    def stats(self) -> dict:
        st = ServerStats()
        _check(lib().rhy_server_stats(self._h, C.byref(st)))
        return st.as_dict()

    def stop(self):
        if self._h:
            lib().rhy_server_stop(self._h)
            self._h = None

    def __del__(self):
        try:
            self.stop()
        except Exception:
            pass


def _text_array(texts) -> C.Array:
    """A `const char* const*` array over the strings: one encoded buffer, pointers computed in bulk
    (keeps the buffer alive as an attribute of the array)."""
    n = len(texts)
    blob = "\0".join(texts).encode() + b"\0"
    ends = np.flatnonzero(np.frombuffer(blob, np.uint8) == 0)
    if len(ends) != max(n, 1):  # a string holding NUL: one pointer per string, cut at the NUL
        arr = (C.c_char_p * max(n, 1))(*[t.encode() for t in texts])
        return arr
    ptrs = np.zeros(len(ends), np.uint64)
    ptrs[1:] = ends[:-1] + 1
    ptrs += np.uint64(C.cast(C.c_char_p(blob), C.c_void_p).value)
    arr = (C.c_void_p * len(ptrs)).from_buffer(ptrs)
    arr._keep = (blob, ptrs)
    return arr


def bits_to_rows(bits: np.ndarray) -> np.ndarray:
    """Global row ids (chunk << 16 | row) of a dense row-set bitmap."""
    b = np.unpackbits(bits.view(np.uint8), bitorder="little")
    return np.flatnonzero(b).astype(np.uint32)


def rows_to_bits(rows, n_chunks: int) -> np.ndarray:
    """Dense row-set bitmap (n_chunks * 2048 uint32 words) of global row ids."""
    b = np.zeros(n_chunks * CHUNK_ROWS, np.uint8)
    b[np.asarray(list(rows), dtype=np.int64)] = 1
    return np.packbits(b, bitorder="little").view(np.uint32).copy()


def _op_program(table, nodes, row_sets):
    """An OpProgram over ctypes arrays; the second value keeps the arrays alive."""
    arr = (OpNode * max(1, len(nodes)))(*nodes)
    sets = [np.ascontiguousarray(r, dtype=np.uint32) for r in (row_sets or [])]
    for r in sets:
        if r.size != table.n_chunks * CHUNK_WORDS:
            raise ValueError("a row set has n_chunks * 2048 words")
    ptrs = (C.c_void_p * max(1, len(sets)))(*[r.ctypes.data for r in sets])
    prog = OpProgram(C.cast(arr, C.POINTER(OpNode)), len(nodes), len(sets), C.cast(ptrs, C.POINTER(C.c_void_p)))
    return prog, (arr, sets, ptrs)
