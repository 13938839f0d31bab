/*
 * C-ABI of the GB300 query hot path for RhyDB/SILO sequence tables.
 *
 * The entry points replace the reference's filter / count / mutations path:
 *   rhy_table_from_raw   ingestion of a partition: SequenceColumn::appendChunk + finalize
 *                        (src/rhydb/storage/column/sequence_column.cpp:100-212) and the
 *                        dictionary / date columns the metadata leaves read;
 *   rhy_open             upload of the partition image to HBM (no reference counterpart: the
 *                        reference evaluates on host memory);
 *   rhy_plan             ScalarExpression::rewrite(table, NONE) + compile(table)
 *                        (src/rhydb/query_engine/scalar_expressions/scalar_expression.h:81-90);
 *   rhy_eval             computeFilter (src/rhydb/query_engine/operators/compute_filter.cpp:14-21)
 *                        = Database::getFilteredBitmap (src/rhydb/database.cpp:259-283);
 *   rhy_count            CountFilterNode (src/rhydb/query_engine/operators/count_filter_node.cpp:35-71);
 *   rhy_mutations        calculateMutationsPerPosition
 *                        (src/rhydb/query_engine/operators/mutations_node.cpp:269-288);
 *   rhy_mutation_rows    addMutationsToOutput (mutations_node.cpp:292-366);
 *   rhy_program_eval /
 *   rhy_program_count /
 *   rhy_program_mutations the same over an already compiled operator tree
 *                        (src/rhydb/query_engine/filter/operators/operator.h:32);
 *   rhy_count_batch /
 *   rhy_mutations_batch  many queries per launch (no reference counterpart: the reference runs one
 *                        query per worker thread, app/src/api.cpp:39-51).
 *
 * Expressions are text, one function per node of the reference's expression tree (positions
 * 1-based): SymEq(col,pos,C) with C = '.' for the reference symbol, HasMut(col,pos), And(...),
 * Or(...), Not(x), NOf(n,exactly|atleast,...), Maybe(x), Exact(x), StrEq(col,value),
 * DateBetween(col,from,to) in days since 1970-01-01 with '*' for an open end, True, False, and
 * MutationProfile (scalar_expressions/mutation_profile.cpp) as MutProfile(col,distance,SEQUENCE),
 * MutProfileMutations(col,distance,pos:C,...) or MutProfileSequenceId(col,distance,id).
 *
 * Conventions: every function returns RHY_OK (0) or an error code and never throws; the message
 * of the last error on the calling thread is returned by rhy_last_error(). Output buffers are
 * owned by the caller. Calls on one device handle are serialised by the handle; `stream` is a
 * cudaStream_t or NULL for the handle's own stream. Row sets are dense bitmaps: chunk k (2^16
 * rows, global row ids k << 16 ...) occupies 2048 uint32 words.
 */
#ifndef RHYDB_GPU_H
#define RHYDB_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
   RHY_OK = 0,
   RHY_ILLEGAL_QUERY = 1,   /* IllegalQueryException in the reference */
   RHY_COMPILATION = 2,     /* QueryCompilationException in the reference */
   RHY_CUDA = 3,
   RHY_INVALID_ARGUMENT = 4,
   RHY_INTERNAL = 5,
   RHY_TIMEOUT = 6,         /* rhy_server_result: not done within the timeout */
   RHY_CANCELLED = 7        /* rhy_server_result: the request was cancelled */
};

typedef struct RhyTable RhyTable;
typedef struct RhyDevice RhyDevice;

/* Raw input: each aligned sequence is the column's reference with sorted, non-overlapping runs
 * (pos, len, char) applied; missing symbols (N / X) inside runs become coverage information. */
typedef struct {
   const char* name;
   int kind;                 /* 0 = nucleotide, 1 = amino acid */
   const char* reference;    /* L characters */
   uint32_t L;
   const uint8_t* is_null;   /* n_rows */
   const uint64_t* row_off;  /* n_rows + 1 */
   const uint32_t* run_pos;
   const uint32_t* run_len;
   const char* run_char;
} RhyRawSeqColumn;

typedef struct {
   const char* name;
   uint32_t n_values;
   const char* const* values; /* dictionary */
   const uint32_t* ids;       /* n_rows, UINT32_MAX = null */
} RhyRawDictColumn;

typedef struct {
   const char* name;
   const int32_t* days;       /* n_rows, INT32_MIN = null */
} RhyRawDateColumn;

typedef struct {
   uint32_t n_rows;
   uint32_t n_seq, n_dict, n_date;
   const RhyRawSeqColumn* seq;
   const RhyRawDictColumn* dict;
   const RhyRawDateColumn* date;
} RhyRawTable;

typedef struct {
   uint64_t seed;
   uint32_t n_rows;
   uint32_t genome_len;
   uint32_t pool_sites;
   uint32_t n_aa_genes;      /* 0 or 12 (9,700 aa) */
   double null_fraction;
   uint32_t threads;         /* 0 = all hardware threads */
} RhyGenConfig;

typedef struct {
   uint32_t n_rows;
   uint32_t n_chunks;
   uint32_t n_seq, n_dict, n_date;
} RhyTableInfo;

typedef struct {
   uint32_t L;
   uint32_t n_symbols;
   uint32_t kind;
   uint32_t flipped_positions;
   uint64_t n_containers;
   uint64_t payload_bytes;
   uint64_t n_array, n_bitset, n_run;
   uint64_t n_missing_intervals;
   uint64_t n_coverage_exceptions;
   uint64_t n_null_rows;
   uint64_t n_row_index_entries;  /* per-row entries (own symbols, coverage and missing-interval events) */
} RhySeqColumnInfo;

typedef struct {
   uint32_t position;        /* 1-based */
   char from;                /* global reference symbol */
   char to;
   uint32_t count;
   uint32_t coverage;        /* total over the valid mutation symbols */
   double proportion;
} RhyMutationRow;

const char* rhy_last_error(void);

/* ---- tables (host) ---- */
int rhy_generate(const RhyGenConfig* cfg, RhyTable** out);
int rhy_table_from_raw(const RhyRawTable* raw, uint32_t threads, RhyTable** out);
/* rhy_table_from_raw with the sequence columns built on GPU `device` (reference:
 * SequenceColumn::appendChunk + finalize, src/rhydb/storage/column/sequence_column.cpp:100-212;
 * TableInserter, src/rhydb/append/table_inserter.cpp:279-343): every row's coverage, missing
 * intervals and stored symbols, the local-reference flips, and the containers are computed on the
 * device; the rest of the image is finished on the host. The table equals rhy_table_from_raw's,
 * byte for byte (rhy_seq_column_checksum). The device memory it uses is freed before it returns. */
int rhy_table_from_raw_gpu(const RhyRawTable* raw, int device, uint32_t threads, RhyTable** out);
int rhy_table_info(const RhyTable* t, RhyTableInfo* out);
/* A 64-bit checksum of a sequence column's whole storage image (local reference, containers and
 * payload, coverage, missing intervals, events, row index), to compare two builds of a table. */
int rhy_seq_column_checksum(const RhyTable* t, uint32_t column, uint64_t* out);
/* Names the dictionary column holding the table's primary key (the schema's primary_key, used by
 * MutProfileSequenceId; reference: src/rhydb/query_engine/scalar_expressions/mutation_profile.cpp:127-150).
 * NULL clears it. Call it before queries that use it run, not concurrently with them. */
int rhy_table_set_primary_key(RhyTable* t, const char* dict_column);
int rhy_seq_column_info(const RhyTable* t, uint32_t column, RhySeqColumnInfo* out);
int rhy_seq_column_name(const RhyTable* t, uint32_t column, char* buf, size_t cap);
/* Views of the raw input of a generated table (valid until rhy_table_free). */
int rhy_table_raw(const RhyTable* t, RhyRawTable* out);
/* Local reference symbols (after adaptation) as characters, L bytes. */
int rhy_local_reference(const RhyTable* t, uint32_t column, char* out, size_t cap);
/* Vertical-index containers of a column in storage order (chunk, position, symbol): position,
 * chunk, symbol, cardinality and encoding (0 array, 1 bitset, 2 run). Pass cap = 0 to size. */
int rhy_seq_containers(const RhyTable* t, uint32_t column, uint32_t* pos, uint16_t* chunk, uint8_t* sym, uint32_t* card,
                       uint8_t* type, size_t cap, size_t* n);
/* The plan of the Mutations container pass over sequence column `column` (no counterpart in the
 * reference; for tests and tuning), for `ctas` CTAs. Array units as 5 u32 each: first payload element
 * (a multiple of 8), element count (at most 1,024), first descriptor (index in storage order, as
 * rhy_seq_containers lists them), descriptor count, chunk. Bitset and run units as 4 u32 each: kind
 * (1 bitset, 2 run), chunk, first payload element, descriptor. CTA ranges as 6 u32 each: array
 * units [a0, a1), other units [o0, o1), chunks v0 and v1. Pass all caps 0 to size. */
int rhy_container_pass_plan(const RhyTable* t, uint32_t column, uint32_t ctas, uint32_t* array_units, size_t array_cap,
                            size_t* n_array, uint32_t* other_units, size_t other_cap, size_t* n_other, uint32_t* ranges,
                            size_t range_cap, size_t* n_ranges);
/* Newline-separated seeded random filter expressions (trees of at most max_leaves leaves, 0 = no
 * limit); *needed receives the byte count (incl. NUL). */
int rhy_generate_queries(const RhyTable* t, uint64_t seed, uint32_t n, uint32_t max_depth, uint32_t max_nof_children,
                         uint32_t max_leaves, int use_aa, int use_metadata, char* buf, size_t cap, size_t* needed);
void rhy_table_free(RhyTable* t);

/* ---- planning ---- */
/* Operator tree of rewrite(NONE) + compile as text, and the device program length / stack depth. */
int rhy_plan(const RhyTable* t, const char* expr, char* tree_buf, size_t cap, uint32_t* n_instr, uint32_t* depth);

/* ---- device ---- */
int rhy_open(const RhyTable* t, int device, RhyDevice** out);
int rhy_set_tile_bits(RhyDevice* d, uint32_t tile_bits);
int rhy_device_bytes(const RhyDevice* d, uint64_t* out);
int rhy_count(RhyDevice* d, const char* expr, void* stream, uint64_t* out);
/* out_bits: n_chunks * 2048 words (may be NULL); out_count may be NULL. */
int rhy_eval(RhyDevice* d, const char* expr, void* stream, uint32_t* out_bits, uint64_t* out_count);
/* counts: n_symbols * L words, counts[symbol * L + position]; filter_count may be NULL. */
int rhy_mutations(RhyDevice* d, const char* expr, uint32_t column, void* stream, uint32_t* counts, uint64_t* filter_count);
/* ---- compiled operator trees (the reference's Operator::evaluate() -> CopyOnWriteBitmap,
 * src/rhydb/query_engine/filter/operators/operator.h:32, and the actions consuming it) ----
 * A caller that has compiled a filter into the reference's operator tree passes it as a postorder
 * node list (children before their parent), each node popping its n_children operands. Node kinds
 * follow the reference's Operator types (operator.h:11-22):
 *   RHY_NODE_EMPTY / RHY_NODE_FULL        Empty, Full (every row of each chunk)
 *   RHY_NODE_SCAN_SEQ     IndexScan over a sequence column's containers: column, position (0-based),
 *                         symbols (bit s = symbol s in the column's alphabet order; the result is the
 *                         union of the rows holding one of them, as getMatchingContainerViews)
 *   RHY_NODE_SCAN_NULLS   IndexScan of the null rows of a sequence column: column
 *   RHY_NODE_SCAN_DICT    IndexScan of a dictionary column's inverted index: column, value (id)
 *   RHY_NODE_SCAN_ROWS    IndexScan over a row set the caller passes: value = its index in row_sets
 *                         (any CopyOnWriteBitmap, e.g. of an index the device does not hold)
 *   RHY_NODE_INTERSECTION Intersection: n_children operands, the last n_negated of them negated
 *   RHY_NODE_UNION        Union: n_children operands (none: the empty set)
 *   RHY_NODE_COMPLEMENT   Complement within each chunk's rows: one operand
 *   RHY_NODE_THRESHOLD    Threshold: value = number_of_matchers, flags & 1 = match exactly;
 *                         n_children operands, the last n_negated of them negated
 *   RHY_NODE_SELECTION    Selection: n_children operands = its predicates and at most one child
 *   RHY_NODE_PRED_COVERED predicate IsInCoveredRegion: column, position, flags & 1 = IS_NOT_COVERED
 *   RHY_NODE_PRED_DATE    predicate CompareToValueSelection on a date column: column, date (days
 *                         since 1970-01-01), flags & 7 = comparator (0 ==, 1 !=, 2 <, 3 <=, 4 >, 5 >=),
 *                         flags & 8 = null dates match
 * The reference's constructor checks apply (Intersection needs a non-negated child and two
 * children, Threshold 0 < n < children): they and malformed lists return RHY_COMPILATION; unknown
 * columns, positions, symbols or value ids RHY_ILLEGAL_QUERY. RangeSelection is passed as a row set.
 * Row sets are dense bitmaps of n_chunks * 2048 words in host memory with no bit at or above the
 * table's row count. */
enum {
   RHY_NODE_EMPTY = 0,
   RHY_NODE_FULL = 1,
   RHY_NODE_SCAN_SEQ = 2,
   RHY_NODE_SCAN_NULLS = 3,
   RHY_NODE_SCAN_DICT = 4,
   RHY_NODE_SCAN_ROWS = 5,
   RHY_NODE_INTERSECTION = 6,
   RHY_NODE_UNION = 7,
   RHY_NODE_COMPLEMENT = 8,
   RHY_NODE_THRESHOLD = 9,
   RHY_NODE_SELECTION = 10,
   RHY_NODE_PRED_COVERED = 11,
   RHY_NODE_PRED_DATE = 12
};
typedef struct {
   uint32_t kind;
   uint32_t n_children;
   uint32_t n_negated;
   uint32_t column;
   uint32_t position;
   uint32_t symbols;
   uint32_t value;
   uint32_t flags;
   int32_t date;
   uint32_t reserved;
} RhyOpNode;
typedef struct {
   const RhyOpNode* nodes;
   uint32_t n_nodes;
   uint32_t n_row_sets;
   const uint32_t* const* row_sets;
} RhyOpProgram;
/* The operator tree of rewrite(NONE) + compile of an expression as a node list (host only; the
 * same tree rhy_plan prints). *n receives the node count; the first min(cap, *n) are copied.
 * Expressions holding a MutationProfile have no node form (RHY_INVALID_ARGUMENT). */
int rhy_program_from_expr(const RhyTable* t, const char* expr, RhyOpNode* nodes, size_t cap, size_t* n);
/* Checks and lowers an operator tree on the host (no device needed): the tree as rhy_plan prints
 * it, the device program length and its stack depth. Fails as the evaluating calls would. */
int rhy_program_plan(const RhyTable* t, const RhyOpProgram* prog, char* tree_buf, size_t cap, uint32_t* n_instr,
                     uint32_t* depth);
/* Operator::evaluate (operator.h:32) -> dense row set and its cardinality (out_bits may be NULL). */
int rhy_program_eval(RhyDevice* d, const RhyOpProgram* prog, void* stream, uint32_t* out_bits, uint64_t* out_count);
/* CountFilterNode over an operator tree (count_filter_node.cpp:35-71). */
int rhy_program_count(RhyDevice* d, const RhyOpProgram* prog, void* stream, uint64_t* out);
/* calculateMutationsPerPosition over an operator tree's row set (mutations_node.cpp:269-288). */
int rhy_program_mutations(RhyDevice* d, const RhyOpProgram* prog, uint32_t column, void* stream, uint32_t* counts,
                          uint64_t* filter_count);
/* Grouped counts of the filter's rows (replaces BitmapAggregationNode, reference
 * bitmap_aggregation_node.cpp:51-140): one dimension per sequence position (kind 0: column,
 * 1-based position; groups = the column's symbols in alphabet order, then null rows) or dictionary
 * column (kind 1: groups = its values in string order, then null rows). Row i of the output is one
 * nonzero combination, in the reference's depth-first order: groups[i * n_dims + d] is its group in
 * dimension d (a symbol index, a value id, or -1 for the null group), counts[i] its rows. *n_out
 * receives the number of combinations; the first min(cap, *n_out) are copied. At most 8
 * dimensions and 2^26 group combinations. */
typedef struct {
   int kind;
   uint32_t column;
   uint32_t position;
} RhyAggDimension;
int rhy_aggregate(RhyDevice* d, const char* expr, const RhyAggDimension* dims, uint32_t n_dims, void* stream,
                  int32_t* groups, uint64_t* counts, size_t cap, size_t* n_out, uint64_t* filter_count);
/* Mutations filters of 1..set[0] rows (single queries) or 1..set[1] rows (slots of a batch) are
 * counted from the row index (each filtered row adds its entries) instead of by the passes over
 * every container; 0 turns that path off. Results are the same either way. `set` and `get` point
 * to two values each and may be NULL. Defaults: rows / 32 and rows / 64. */
int rhy_sparse_rows(RhyDevice* d, const uint64_t* set, uint64_t* get);
/* ---- batched path (no reference counterpart: the reference runs one query per worker thread,
 * app/src/api.cpp:39-51) ----
 * n queries; actions[i] 0 = count, 1 = mutations of columns[i]. counts[i] receives the filter
 * cardinality; for a mutations query mut_counts[i] (n_symbols * L words) receives the symbol
 * counts (mut_counts may be NULL, entries of count queries are ignored). tile_bits 0 = default.
 * Synchronous on `stream`. */
int rhy_batch(RhyDevice* d, const char* const* exprs, const int* actions, const uint32_t* columns, uint32_t n,
              uint32_t tile_bits, void* stream, uint64_t* counts, uint32_t* const* mut_counts);

/* Mutations action output of a batch computed on the device (replaces addMutationsToOutput,
 * reference mutations_node.cpp:292-366, behind MutationsNode::addToExecPlan, :377): for every
 * Mutations query the rows (position, from, to, count, coverage, proportion) whose count exceeds
 * ceil(coverage * min_proportion) - 1 (any count > 0 when min_proportion is 0), packed in query-slot
 * order. counts[i] receives every query's filter cardinality; *n_rows the total number of rows,
 * which are copied when *n_rows <= rows_cap (otherwise rhy_batch_rows_fetch copies them without
 * recomputing). Query i's rows are rows[row_begin[i] .. row_begin[i] + row_count[i]).
 * min_proportions may be NULL (0.05 for every query); each must lie in [0, 1]. The batch is planned
 * and run in parts (the Mutations and Details queries up to 1,024 at a time, then the counts) so
 * that planning a part overlaps the device work of the ones before it; the first part is planned by
 * the rule even when the learned planner is on. Results do not depend on it. */
int rhy_batch_rows(RhyDevice* d, const char* const* exprs, const int* actions, const uint32_t* columns,
                   const double* min_proportions, uint32_t n, uint32_t tile_bits, void* stream, uint64_t* counts,
                   RhyMutationRow* rows, size_t rows_cap, uint64_t* row_begin, uint32_t* row_count, size_t* n_rows);
int rhy_batch_rows_fetch(RhyDevice* d, void* stream, RhyMutationRow* rows, size_t rows_cap);

/* Host wall time of the phases of the last rhy_batch_rows call: planning (parse, rewrite, compile,
 * estimates, lowering), staging (work items, device buffers), the batch on the device up to its
 * counts and row sizes (one synchronisation), and the packed rows with their copy to the host. */
typedef struct {
   double plan_ms, prepare_ms, device_ms, output_ms;
   double compile_ms, predict_ms, lower_ms; /* plan_ms split: parse to features, network, lowering */
} RhyBatchTimes;
int rhy_batch_times(RhyDevice* d, RhyBatchTimes* out);

typedef struct {
   uint32_t n_queries, n_mutation_slots, n_items, n_instr, max_depth, tile_bits, grid;
   uint64_t device_bytes;
   uint32_t n_filter_launches; /* persistent filter launches per batch (one for all program classes) */
   uint64_t filter_bytes;      /* algorithmic bytes of the batch's filter programs: container payloads and
                                  descriptors of their index-scan leaves, coverage and date data their
                                  leaves read, and their outputs (row sets of Mutations queries, counts) */
} RhyBatchInfo;

/* Split form of rhy_batch for callers that reuse one batch shape: prepare plans and stages the
 * batch (allocates on first use or growth), launch enqueues it without synchronising,
 * capture/replay record it once into a CUDA graph and replay it, results copies the outputs of the
 * last completed launch (the caller synchronises the stream first). */
int rhy_batch_prepare(RhyDevice* d, const char* const* exprs, const int* actions, const uint32_t* columns, uint32_t n,
                      uint32_t tile_bits, uint32_t plan_threads);
int rhy_batch_launch(RhyDevice* d, void* stream, int copy_in, int copy_out);
int rhy_batch_capture(RhyDevice* d, void* stream);
int rhy_batch_replay(RhyDevice* d, void* stream);
int rhy_batch_results(RhyDevice* d, uint64_t* counts, uint32_t* const* mut_counts);
int rhy_batch_info(RhyDevice* d, RhyBatchInfo* out);

/* Schedule of the batched filter launches (results never depend on it): the widest tile of a class
 * (bits), the stack budget that narrows a class's tile (KiB), persistent CTAs per SM (0 = as many
 * as fit) and the work-item order (0 = tile-major, 1 = every tile of one query in turn). */
typedef struct {
   uint32_t max_tile_bits, stack_kb, ctas_per_sm, query_major;
} RhyBatchSchedule;
/* Sets the schedule when `set` is not NULL, then reports the one in force when `get` is not NULL. */
int rhy_batch_schedule(RhyDevice* d, const RhyBatchSchedule* set, RhyBatchSchedule* get);
/* Autotuner: plans the batch, times its filter launches under every candidate schedule (tile widths
 * 16 / 32 / 64 Kbit x stack budgets 24 / 40 / 64 KiB x all or two CTAs per SM x both item orders;
 * `reps` timed runs each, median, CUDA events on `stream`), keeps the fastest in force and returns
 * the candidates fastest first in tried[0 .. min(cap, *n_tried)) with their milliseconds. */
int rhy_batch_autotune(RhyDevice* d, const char* const* exprs, const int* actions, const uint32_t* columns, uint32_t n,
                       uint32_t reps, void* stream, RhyBatchSchedule* tried, double* tried_ms, size_t cap,
                       size_t* n_tried);
/* Variants for timing: capture without the host copies; launch a subset of the kernels
 * (bit 0 filter, bits 1..4 transpose / container / coverage / final mutations kernels, bit 5 the
 * row-index pass of the slots whose filters have few rows; without bit 5 the dense kernels count
 * every slot). */
int rhy_batch_capture_ex(RhyDevice* d, void* stream, int copy_in, int copy_out);
int rhy_batch_launch_parts(RhyDevice* d, void* stream, uint32_t parts);

/* Plain single-query path split for timing with device-resident inputs: prepare plans the queries
 * and keeps their programs in HBM; launch enqueues query i (filter, and the mutations kernels for
 * a mutations query) into the handle's scratch without synchronising. */
int rhy_plain_prepare(RhyDevice* d, const char* const* exprs, const int* actions, const uint32_t* columns, uint32_t n);
int rhy_plain_launch(RhyDevice* d, uint32_t i, void* stream);
/* parts: bit 0 zeroing + filter kernel, bits 1..3 container / coverage / final mutations kernels,
 * bit 4 the row-index pass for filters of few rows (rhy_sparse_rows; without it the container and
 * coverage kernels count every filter). */
int rhy_plain_launch_parts(RhyDevice* d, uint32_t i, void* stream, uint32_t parts);
/* Bytes a mutations pass over `column` must read: container payloads plus descriptors. */
int rhy_mutation_bytes(const RhyDevice* d, uint32_t column, uint64_t* payload_bytes, uint64_t* descriptor_bytes);

/* Mutations pass that allocates no device memory (no counterpart in the reference, which runs on
 * host memory). For callers that may not allocate during a query: a process whose device memory
 * is owned by its own pool allocator, or a latency-critical thread that must avoid the implicit
 * synchronisation of cudaMalloc / cudaFree. The caller passes device buffers it owns: the filter
 * row set (n_chunks * 2048 words, as written by the filter kernels), its cardinality, the output
 * counts (n_symbols * L words, counts[symbol * L + position], overwritten) and one int of status,
 * which the call clears and a kernel of the pass sets to a nonzero device error code (7: a bounded
 * wait of the container pass for its bulk copies gave up); a completed pass leaves it 0. Read it
 * after synchronising the stream. Working memory is one fixed array in the library's device image
 * (1.5 MiB, held on every GPU that loads the library until the process exits), which limits the
 * column to 131,072 positions; longer columns fail with RHY_INVALID_ARGUMENT. The first call on a
 * device looks up the array's address; make that first call before any stream capture. All calls
 * on a device share the array: calls that overlap on the GPU race and must be serialised by the
 * caller. The enqueue itself is ordered with the handle's other calls. Filters of at most
 * rhy_sparse_rows' single-query limit take the row-index pass, as in rhy_mutations. The work is
 * enqueued on `stream` (NULL = the handle's stream); results are valid once that stream has been
 * synchronised. */
int rhy_mutations_noalloc(RhyDevice* d, uint32_t column, const uint32_t* d_filter, const uint64_t* d_filter_count,
                          uint32_t* d_counts, int* d_status, void* stream);
/* Testing the failure path of the bounded device waits (no counterpart in the reference): while bit
 * 0 of `on` is set, the filter kernels announce the leaf payload copies their waits expect but never
 * issue them, so a wait gives up after 1 ms and the call reports RHY_CUDA ("a bounded device wait
 * for bulk copies gave up", device error 6); bit 1 does the same for the Mutations container pass's
 * ring copies (device error 7; rhy_mutations_noalloc reports it in its status word). The withheld
 * copies never start, so no copy is left in flight and the device stays usable. Synchronises the
 * device; off (0) by default. Not for production use. */
int rhy_test_withhold_copies(RhyDevice* d, int on);

/* Formats counts like the reference's Mutations action; returns the number of rows in *n_rows. */
int rhy_mutation_rows(const RhyTable* t, uint32_t column, const uint32_t* counts, double min_proportion,
                      RhyMutationRow* rows, size_t cap, size_t* n_rows);
/* ---- learned planner (no counterpart in the reference, whose operators order children by
 * cardinality only: intersection.cpp:59-106) ----
 * The network (24 -> 64 -> 64 -> 2, BF16 weights, FP32 arithmetic) predicts per operator node the
 * natural log of its result's fraction of the rows and of its cycles per tile. collect runs each
 * expression through the single-query path in trace mode and appends one sample per operator node;
 * train fits the network on the GPU (80/20 split, Adam) and judges it on the held-out part against
 * the rule-based estimator; mode 1 plans batches with it (only once accepted), mode 0 (the
 * default) with the rule-based ordering. Plans differ only in child order and item order; results
 * are identical. */
#define RHY_PLANNER_FEATURES 24
#define RHY_MLP_NPARAM 5890 /* W1[64][24] b1[64] W2[64][64] b2[64] W3[2][64] b3[2] */
typedef struct {
   uint32_t n_train, n_val, epochs;
   float train_loss, val_loss;
   float qerr_learned_median, qerr_rule_median, qerr_learned_p90, qerr_rule_p90;
   float cost_err_median;
   float train_ms;
   int accepted;
} RhyPlannerStats;
/* Features of every operator node of the compiled expression, in preorder (host only). */
int rhy_plan_features(const RhyTable* t, const char* expr, float* x /* [n][24] */, size_t cap, size_t* n);
int rhy_planner_collect(RhyDevice* d, const char* const* exprs, uint32_t n, size_t* n_added);
int rhy_planner_train(RhyDevice* d, uint32_t epochs, uint32_t batch, float lr, uint64_t seed, RhyPlannerStats* out);
int rhy_planner_mode(RhyDevice* d, int mode);
/* Samples: x[n][24] features; y[n][3] = ln selectivity, ln cycles per tile, ln rule selectivity. */
int rhy_planner_samples(RhyDevice* d, float* x, float* y, size_t cap, size_t* n);
int rhy_planner_weights(RhyDevice* d, float* w /* RHY_MLP_NPARAM FP32 master weights */);
/* A trained planner as plain values, to train on one table and plan on another: the FP32 master
 * weights, the feature and target normalisation, and the verdict of the judge. */
typedef struct {
   float weights[RHY_MLP_NPARAM];
   float feature_mean[RHY_PLANNER_FEATURES], feature_std[RHY_PLANNER_FEATURES];
   double target_mean[2], target_std[2];
   int accepted;
} RhyPlannerModel;
int rhy_planner_export(RhyDevice* d, RhyPlannerModel* out);
int rhy_planner_import(RhyDevice* d, const RhyPlannerModel* in);
/* Traces the expressions on this device (they do not join the training samples) and judges the
 * current network on them against the rule-based estimates (q-errors in out, n_val = samples); the
 * verdict replaces the planner's acceptance, and a rejected network leaves mode 1. */
int rhy_planner_evaluate(RhyDevice* d, const char* const* exprs, uint32_t n, RhyPlannerStats* out);
/* Network predictions (GPU inference) for feature rows: selectivity (fraction of rows) and cycles
 * per tile. */
int rhy_planner_predict(RhyDevice* d, const float* x, uint32_t n, double* sel, double* cost);
/* One forward + backward of the network with the given FP32 master weights (used in BF16) on the
 * device: gradient of mean_n sum_k (y_k - t_k)^2 with respect to the BF16 weights, the loss and the
 * outputs y[n][2]. Leaves the planner untouched. */
int rhy_mlp_gradient(RhyDevice* d, const float* w, const float* x, const float* t, uint32_t n, float* grad, float* loss,
                     float* y);

/* ---- serving (continuous batching; no counterpart in the reference, which runs one query per
 * request thread, api.cpp:39-51) ----
 * A loop thread admits submitted requests into micro-batches while the in-flight queries fit
 * max_inflight and their device buffers fit memory_budget, and keeps `streams` micro-batches in
 * flight, so requests that arrive while others run are admitted as slots and memory free up and
 * overlap on the device. A partial micro-batch launches once its oldest request waited
 * max_wait_ms (at once when the device is idle). Actions: 0 Aggregated count, 1 Mutations rows
 * (min_proportion, column), 2 Details (the first k row ids, ascending). Results equal those of the
 * same query alone. */
typedef struct RhyServer RhyServer;
typedef struct {
   uint32_t max_batch;       /* queries per micro-batch (default 512) */
   uint32_t streams;         /* micro-batches in flight (default 3) */
   uint32_t max_inflight;    /* admitted, unfinished queries (default 4096) */
   uint64_t memory_budget;   /* device bytes of in-flight work; 0 = a quarter of the free memory */
   double max_wait_ms;       /* default 0.25 */
   uint32_t plain;           /* 1: no batching; each request runs alone through the single-query path
                                (rhy_count / rhy_mutations / rhy_eval) in arrival order, the way the
                                reference serves one query per request; 0 (default): continuous batching */
} RhyServerConfig;
typedef struct {
   uint64_t submitted, completed, rejected, batches;
   double p50_ms, p99_ms, mean_batch, qps;
   uint64_t peak_bytes, budget_bytes;
   uint32_t peak_inflight;
   uint64_t cancelled;
} RhyServerStats;
int rhy_server_start(RhyDevice* d, const RhyServerConfig* cfg /* NULL: defaults */, RhyServer** out);
/* Validates and queues a request (user errors are returned here). */
int rhy_server_submit(RhyServer* s, const char* expr, int action, uint32_t column, double min_proportion, uint32_t k,
                      uint64_t* id);
/* Waits for a request (timeout_ms < 0: no limit; RHY_TIMEOUT if not done) and copies its result:
 * the filter count, Mutations rows, Details ids and the latency from submission. When rows or ids
 * do not fit their caps only *n_rows / *n_ids are set, RHY_INVALID_ARGUMENT is returned and the
 * result is kept for another call; otherwise it is released. */
int rhy_server_result(RhyServer* s, uint64_t id, double timeout_ms, uint64_t* count, RhyMutationRow* rows,
                      size_t rows_cap, size_t* n_rows, uint32_t* ids, size_t ids_cap, size_t* n_ids, double* latency_ms);
int rhy_server_stats(RhyServer* s, RhyServerStats* out);
/* Cancels a request that is not done (reference: the plan-stop guard of a query that is abandoned,
 * query_plan.cpp:66-123): a queued request is dropped before admission, one already on the device
 * finishes there and its result is discarded. rhy_server_result then returns RHY_CANCELLED.
 * *was_pending (may be NULL) is 1 if the request was cancelled, 0 if it had already finished. */
int rhy_server_cancel(RhyServer* s, uint64_t id, int* was_pending);
/* Open-loop replay of a request trace: request i is submitted by a native thread at arrival_s[i]
 * seconds after the call starts; then all are awaited. latency_ms[i] receives each latency (NaN if
 * the request failed), *wall_s the time from the start to the last result. */
int rhy_server_replay(RhyServer* s, const char* const* exprs, const int* actions, const uint32_t* columns,
                      const double* min_proportions, const uint32_t* ks, const double* arrival_s, uint32_t n,
                      double* latency_ms, double* wall_s);
/* Finishes every queued request, stops the loop and frees the server. */
void rhy_server_stop(RhyServer* s);

void rhy_close(RhyDevice* d);

#ifdef __cplusplus
}
#endif

#endif /* RHYDB_GPU_H */
