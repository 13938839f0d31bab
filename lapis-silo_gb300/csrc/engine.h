// Device-resident partition and the execution of filter / count / mutations queries on it.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "aggregate.h"
#include "device.h"
#include "expr.h"
#include "planner.h"
#include "util.h"
#include "table.h"

namespace rhygpu {

struct CudaError : std::runtime_error {
   using std::runtime_error::runtime_error;
};

void cuda_check(cudaError_t e, const char* what);

// Throws the exception of a nonzero device error flag: CudaError for a bounded wait that gave up
// (DEVERR_WAIT_FILTER, DEVERR_WAIT_MUTATIONS), CompilationError for a malformed program.
[[noreturn]] void throw_device_error(int code);

// addMutationsToOutput on the host (reference: mutations_node.cpp:292-366): the rows of a column's
// dense counts (counts[symbol * L + position]) whose count exceeds ceil(total * min_proportion) - 1
// (any count > 0 when min_proportion is 0), total over the valid symbols, the global reference
// symbol skipped; proportion = count / total. Rows go to `out` (when not null) up to `cap`; returns
// their number.
size_t mutation_rows_host(const SeqColumnImage& c, const uint32_t* counts, double min_proportion, DevMutationRow* out,
                          size_t cap);

// One query of a batch. Actions: 0 = Aggregated count, 1 = Mutations of `column`, 2 = Details
// (the first k row ids of the filter, ascending).
struct BatchQuery {
   Program prog;
   int action = 0;  // 0 = count, 1 = mutations of `column`
   int column = 0;
   double min_proportion = 0.05;  // Mutations rows: minimum proportion of a reported mutation
   double cost = 0;               // predicted cycles per tile (learned planner); 0 = unknown
   uint32_t k = 1000;             // Details: number of row ids returned (the first ones)
};

// Schedule of the batched filter launches: the widest tile of a class, the stack budget that narrows
// a class's tile (deep programs get narrower tiles, so more CTAs fit per SM), persistent CTAs per SM
// (0 = as many as fit) and the order of the (query, tile) work items (tile-major interleaving, or
// every tile of one query in turn). Results never depend on it.
struct BatchSchedule {
   uint32_t max_tile_bits = 65536;
   uint32_t stack_kb = 40;
   uint32_t ctas_per_sm = 0;
   uint32_t query_major = 0;
};

// Batched path state: device buffers and pinned staging, grown on demand and reused across batches.
struct BatchState {
   // Classes of programs sharing a tile width (their work items are consecutive); one persistent
   // filter launch of `grid` CTAs with `stack_bytes` of stack takes the items of every class.
   struct FilterGroup {
      uint32_t item_off, n_items, tile_bits, max_depth;
   };
   std::vector<FilterGroup> fgroups;
   uint32_t stack_bytes = 0;
   struct ColGroup {
      int column;
      uint32_t slot_begin, n;
      size_t counts_off, scratch_off;  // u32 offsets into the arenas
      size_t lists_off;                // u32 offset of the group's slot lists (2 n + 2)
      uint32_t blk_off;                // first entry of the group's slots in the row-block table
   };
   uint32_t n_queries = 0, n_slots = 0, n_items = 0, n_code = 0, max_depth = 1, tile_bits = 16384, grid = 0;
   std::vector<ColGroup> groups;
   std::vector<uint32_t> slot_of_query;  // UINT32_MAX for count-only queries
   size_t counts_words = 0, scratch_words = 0, mask_bytes = 0;
   // pinned host staging
   Instr* h_code = nullptr;
   QueryDesc* h_q = nullptr;
   WorkItem* h_items = nullptr;
   uint32_t* h_slot_query = nullptr;
   unsigned long long* h_counts = nullptr;
   uint32_t* h_mcounts = nullptr;
   double* h_minprop = nullptr;       // per slot
   uint32_t* h_rowblk = nullptr;      // row-block offsets of the last batch_rows, n_blk + 1
   // device
   Instr* d_code = nullptr;
   QueryDesc* d_q = nullptr;
   WorkItem* d_items = nullptr;
   uint32_t* d_slot_query = nullptr;
   unsigned long long* d_counts = nullptr;
   uint32_t* d_next = nullptr;
   uint32_t* d_tiles = nullptr;
   uint32_t* d_mcounts = nullptr;
   uint32_t* d_mscratch = nullptr;
   uint16_t* d_masks = nullptr;
   uint32_t* d_lists = nullptr;       // per column group: dense and sparse slot lists, their lengths
   double* d_minprop = nullptr;
   uint32_t* d_rowblk = nullptr;
   DevMutationRow* d_rows = nullptr;
   int* d_err = nullptr;              // error flag of this batch's kernels
   int* h_err = nullptr;              // pinned
   uint32_t* d_k = nullptr;           // Details: k per slot, then offsets into the ids
   uint32_t* h_k = nullptr;
   uint32_t* d_ids = nullptr;         // Details: row ids
   uint32_t* h_ids = nullptr;
   uint32_t* d_nids = nullptr;        // Details: ids per slot
   uint32_t* h_nids = nullptr;
   uint32_t n_blk = 0;                // row-block table entries (Mutations slots)
   bool rows_in_final = false;        // the final Mutations pass also counts the rows per block
   size_t n_rows = 0;                 // rows of the last row pass
   uint32_t n_mut_slots = 0, n_details = 0, n_ids = 0;
   // MutationProfile row sets of the batch's programs (QueryDesc.aux_base numbers them)
   DevProfile* h_prof = nullptr;      // pinned; arrays point into d_prof_data
   uint32_t* h_prof_data = nullptr;   // pinned
   DevProfile* d_prof = nullptr;
   uint32_t* d_prof_data = nullptr;
   uint32_t* d_aux = nullptr;         // n_aux row sets of nchunks * CHUNK_WORDS words
   uint32_t n_aux = 0, profile_max_L = 0;
   size_t n_prof_data = 0;
   size_t hc_prof = 0, hc_prof_data = 0, dc_prof = 0, dc_prof_data = 0, dc_aux = 0;
   // capacities (elements), one per buffer
   size_t hc_code = 0, hc_q = 0, hc_items = 0, hc_slot_query = 0, hc_counts = 0, hc_mcounts = 0, hc_minprop = 0,
          hc_rowblk = 0, hc_err = 0, hc_k = 0, hc_ids = 0, hc_nids = 0;
   size_t dc_code = 0, dc_q = 0, dc_items = 0, dc_slot_query = 0, dc_counts = 0, dc_next = 0, dc_tiles = 0,
          dc_mcounts = 0, dc_mscratch = 0, dc_masks = 0, dc_minprop = 0, dc_rowblk = 0, dc_rows = 0, dc_err = 0, dc_k = 0,
          dc_ids = 0, dc_nids = 0, dc_lists = 0;
   cudaGraphExec_t graph = nullptr;
};

class Engine {
  public:
   static constexpr uint32_t BATCH_ALL = 63;  // batch_enqueue parts: the whole batch
   Engine(const TableImage& table, int device);
   ~Engine();
   Engine(const Engine&) = delete;
   Engine& operator=(const Engine&) = delete;

   const TableImage& table() const { return table_; }
   int device() const { return device_; }
   uint32_t nchunks() const { return table_.nchunks(); }
   const DevTable* d_table() const { return d_table_; }
   const DevTable& host_view() const { return view_; }
   uint64_t device_bytes() const { return device_bytes_; }
   // The stream a call runs on: the caller's, or the engine's own when the caller passed none.
   cudaStream_t stream_for(cudaStream_t s) const { return s ? s : stream_; }

   // Tile width of the filter kernel (rows per CTA). 4096 .. 65536, power of two. The single-query
   // path wants many CTAs (one per tile); the persistent batched kernel amortises each leaf's
   // latency over wider tiles. rhy_set_tile_bits sets both.
   uint32_t tile_bits = 16384;
   uint32_t batch_tile_bits = 65536;
   // Mutations filters of at most this many rows take the row-index pass instead of the dense
   // passes: single queries, and slots of a batch (0: never). Defaults: rows / SPARSE_PLAIN_DIV and
   // rows / SPARSE_BATCH_DIV.
   static constexpr uint32_t SPARSE_PLAIN_DIV = 32, SPARSE_BATCH_DIV = 64;
   uint64_t sparse_rows_plain = 0, sparse_rows_batch = 0;
   BatchSchedule batch_schedule;  // used by batch_prepare unless a tile width is requested
   // Autotuner: prepares the batch under every candidate schedule (tile widths 16, 32 and 64 Kbit,
   // stack budgets 24, 40 and 64 KiB, all or two CTAs per SM, both item orders), times its filter
   // launches `reps` times with CUDA events on `stream` and keeps the fastest as batch_schedule.
   // Returns every candidate with its median milliseconds, the chosen one first. The caller holds mu.
   std::vector<std::pair<BatchSchedule, double>> autotune_batch(const std::vector<BatchQuery>& qs, cudaStream_t stream,
                                                                uint32_t reps);

   Program plan(const std::string& expr, const LowerOptions& opt = {}, std::string* tree = nullptr) const;

   // Plain single-query path: host in, host out, synchronous on `stream` (nullptr = engine stream).
   // `literals`: the caller's row sets read by the program's ROWS leaves (host memory, nchunks * 2048
   // words each; Program::n_literals of them), or nullptr for a program without them.
   uint64_t count(const Program& p, cudaStream_t stream, const uint32_t* const* literals = nullptr);
   void eval(const Program& p, uint32_t* host_bits /* nchunks * 2048 */, uint64_t* host_count, cudaStream_t stream,
             const uint32_t* const* literals = nullptr);
   void mutations(const Program& p, int column, uint32_t* host_counts /* nsym * L */, uint64_t* filter_count,
                  cudaStream_t stream, const uint32_t* const* literals = nullptr);
   // Grouped counts of the filter's rows (BitmapAggregation): one dimension per sequence position
   // (kind AGG_SEQUENCE, 0-based position) or dictionary column (AGG_DICTIONARY). Output rows in the
   // reference's order, groups[i * dims + d] = symbol index / value id / -1 for the null group.
   struct AggSpec {
      uint32_t kind, col, pos;
   };
   void aggregate(const Program& p, const std::vector<AggSpec>& dims, std::vector<int32_t>& groups,
                  std::vector<uint64_t>& counts, uint64_t* filter_count, cudaStream_t stream);

   // Device-side building blocks (no host synchronisation); used by the timed benchmark legs.
   void upload_program(const Program& p, Instr* d_code, cudaStream_t stream);
   void launch_count(const Instr* d_code, const Program& p, unsigned long long* d_count, uint32_t* d_tiles,
                     cudaStream_t stream, const uint32_t* const* literals = nullptr);
   void launch_mutations(int column, const uint32_t* d_filter, const unsigned long long* d_count, uint32_t* d_counts,
                         uint32_t* d_scratch, cudaStream_t stream, uint32_t parts = MUT_PART_ALL);
   void check_error_flag();

   // ---- batched path ----
   // Plans every expression (host threads), lays the programs and (query, tile) work items out and
   // sizes the device buffers (may allocate; call outside timed regions).
   void batch_prepare(const std::vector<BatchQuery>& qs, uint32_t tile_bits = 0) { batch_prepare(batch_, qs, tile_bits); }
   void batch_prepare(BatchState& b, const std::vector<BatchQuery>& qs, uint32_t tile_bits = 0);
   // Device bytes a batch of these queries holds (buffers of batch_prepare and the row pass).
   size_t batch_device_bytes(const std::vector<BatchQuery>& qs, uint32_t tile_bits = 0) const;
   void batch_free(BatchState& b);
   // Stream-ordered: optional H2D of the staged programs, the persistent filter kernel, the batched
   // mutations kernels per column, optional D2H of the results into the pinned host buffers.
   // parts: bit 0 = zeroing + filter kernel, bits 1..4 = transpose, container, coverage and final
   // mutations kernels, bit 5 = the row-index pass of the slots whose filters have few rows (all set
   // = the whole batch; without bit 5 the dense passes count every slot); used to time kernels one
   // by one.
   void batch_enqueue(cudaStream_t stream, bool copy_in, bool copy_out, uint32_t parts = BATCH_ALL) {
      batch_enqueue(batch_, stream, copy_in, copy_out, parts);
   }
   void batch_enqueue(BatchState& b, cudaStream_t stream, bool copy_in, bool copy_out, uint32_t parts = BATCH_ALL);
   // Row pass of a batch in two stream-ordered phases around one host step: phase 1 enqueues the
   // batch, the D2H of the counts / Details ids and the count + scan of the rows; once the stream
   // has passed it, phase 2 sizes the rows, enqueues their write and copies them to `rows`.
   void rows_phase1(BatchState& b, cudaStream_t stream);
   size_t rows_phase2(BatchState& b, cudaStream_t stream, DevMutationRow* rows, size_t cap);
   void row_range(const BatchState& b, uint32_t query, uint64_t* begin, uint32_t* count) const;
   const uint32_t* details_ids(const BatchState& b, uint32_t query, uint32_t* n) const;  // pinned host
   void check_batch_error(BatchState& b);
   BatchState& batch_state() { return batch_; }
   uint64_t batch_state_count(const BatchState& b, uint32_t query) const { return b.h_counts[query]; }
   // Captures batch_enqueue(copy_in, copy_out) into a CUDA graph for the prepared shape.
   void batch_capture(cudaStream_t stream, bool copy_in = true, bool copy_out = true);
   void batch_replay(cudaStream_t stream);
   const BatchState& batch() const { return batch_; }
   const uint32_t* batch_mutation_counts(uint32_t query) const;  // pinned host, after the stream synced
   // Mutations action output of the prepared batch: enqueues the batch and the row passes,
   // synchronises once to size the packed rows, copies them to `rows` when they fit `cap` and
   // returns their number. Query i's rows are rows[row_begin[i] .. row_begin[i] + row_count[i])
   // (count queries: none). The filter counts are in batch_count afterwards.
   size_t batch_rows(cudaStream_t stream, DevMutationRow* rows, size_t cap, uint64_t* row_begin, uint32_t* row_count);
   // Copies the rows of the last batch_rows again (for a caller whose buffer was too small).
   void batch_rows_fetch(cudaStream_t stream, DevMutationRow* rows, size_t cap);
   // batch_rows of a whole batch given as text, planned and run in parts so that the host plans a
   // part while the device runs the ones before it: first the Mutations and Details queries in
   // parts of at most PIPELINE_HEAVY (the first quarter of the counts when there are none), then
   // the Aggregated counts in parts of about PIPELINE_COUNTS. Results equal batch_rows of the whole
   // batch; the rows come in part order. Counts fewer than PIPELINE_PART join the part before them.
   // The caller holds mu.
   static constexpr uint32_t PIPELINE_PART = 256;
   static constexpr uint32_t PIPELINE_HEAVY = 1024;
   static constexpr uint32_t PIPELINE_COUNTS = 768;
   size_t batch_rows_pipelined(const std::vector<std::string>& exprs, const int* actions, const uint32_t* columns,
                               const double* min_proportions, uint32_t tile_bits, cudaStream_t stream,
                               DevMutationRow* rows, size_t cap, uint64_t* counts, uint64_t* row_begin,
                               uint32_t* row_count);
   uint64_t batch_count(uint32_t query) const { return batch_.h_counts[query]; }
   // Host wall time of the phases of the last batch call made through the C-ABI: planning
   // (parse, rewrite, compile, estimates, lowering), staging (work items, device buffers), the
   // batch on the device up to its counts and row sizes, and the packed rows with their copy.
   // plan_ms splits into compile (parse, rewrite, compile, features), predict (network inference,
   // learned planner only) and lower.
   struct BatchTimes {
      double plan_ms = 0, prepare_ms = 0, device_ms = 0, output_ms = 0;
      double compile_ms = 0, predict_ms = 0, lower_ms = 0;
   } batch_times;
   // Tile width that fits the batch's deepest program in the shared-memory budget.
   uint32_t fit_tile_bits(uint32_t requested, uint32_t depth, bool batch = false) const;

   // ---- learned planner ----
   // Runs every expression through the single-query path in trace mode (program lowered without
   // early exits) and appends one training sample per operator node. Returns the samples added.
   size_t planner_collect(const std::vector<std::string>& exprs);
   PlannerStats planner_train(uint32_t epochs, uint32_t batch, float lr, uint64_t seed);
   // Traces the expressions (not added to the training samples) and judges the current network on
   // them against the rule; the verdict replaces the planner's acceptance (a rejected network
   // leaves the learned mode).
   PlannerStats planner_evaluate(const std::vector<std::string>& exprs);
   // 0: rule-based ordering; 1: learned (only once a trained network was accepted against the
   // rule-based ordering on held-out traces).
   void set_planner_mode(int mode);
   int planner_mode() const { return use_learned_ ? 1 : 0; }
   Planner& planner() { return planner_; }
   // Plans a batch: rule-based, or with the learned planner's estimates (one GPU inference over
   // all operator nodes of all expressions) and a predicted cost per query. `rule_only` plans with
   // the rule even when the learned planner is on. The caller holds mu.
   std::vector<BatchQuery> plan_batch(const std::vector<std::string>& exprs, uint32_t threads, bool rule_only = false);
   // The learned planner in two steps: learned_compile compiles and featurises every expression and
   // runs one network inference over all their operator nodes; learned_lower lowers a subset of
   // them with those estimates (and frees their trees). The caller holds mu.
   struct LearnedPlans {
      std::vector<OpPtr> ops;
      std::vector<std::vector<std::pair<const Op*, double>>> est;  // per query: (node, rows), by node
      std::vector<double> cost;
   };
   void learned_compile(const std::vector<std::string>& exprs, uint32_t threads, LearnedPlans& lp);
   std::vector<BatchQuery> learned_lower(LearnedPlans& lp, const std::vector<uint32_t>& idx, uint32_t threads);

   const EvItem* d_ev(int column) const { return d_ev_[column]; }
   uint32_t n_ev(int column) const { return n_ev_[column]; }
   uint64_t mutation_payload_bytes(int column) const;
   // Algorithmic bytes of one filter program over the whole table: the payloads and descriptors of
   // the containers its index-scan leaves read, the coverage exceptions and the missing intervals of
   // the position's block its coverage leaves read, the bit planes its date leaves read, the dense
   // row sets of null and aux leaves, and the output (a dense row set, or one count). Intermediates
   // between operators are not counted.
   uint64_t program_bytes(const Program& p, bool writes_rows) const;
   uint64_t instr_bytes(const Instr& in) const;  // one leaf's share of program_bytes
   // program_bytes over every program of a prepared batch (its slot queries write row sets)
   uint64_t batch_filter_bytes(const BatchState& b) const;

   // scratch of the single-query path
   uint32_t* d_filter = nullptr;      // nchunks * CHUNK_WORDS
   unsigned long long* d_count = nullptr;
   uint32_t* d_counts = nullptr;      // max nsym * L
   uint32_t* d_scratch = nullptr;     // 3 * (max L + 1)
   Instr* d_code = nullptr;           // MAX_PROGRAM
   int* d_err = nullptr;
   size_t counts_words = 0, scratch_words = 0;
   std::mutex mu;

  private:
   template <typename T>
   T* upload(const std::vector<T>& v, size_t min_elems = 1);
   void* alloc(size_t bytes);
   void upload_dates(const DateColumnImage& dc, uint32_t nchunks, DevDateCol& out);

   const TableImage& table_;
   int device_;
   cudaStream_t stream_ = nullptr;
   DevTable view_{};
   DevTable* d_table_ = nullptr;
   std::vector<void*> allocs_;
   std::vector<EvItem*> d_ev_;
   std::vector<uint32_t> n_ev_;
   std::vector<CtrUnit*> d_cu_;  // container units of the batched Mutations pass, heaviest first
   std::vector<uint32_t> n_cu_;
   Instr* h_code_ = nullptr;               // pinned staging
   unsigned long long* h_count_ = nullptr; // pinned
   int* h_err_ = nullptr;                  // pinned
   uint64_t device_bytes_ = 0;
   BatchState batch_;
   std::vector<std::unique_ptr<BatchState>> parts_;      // parts 1.. of batch_rows_pipelined
   std::vector<BatchState*> rows_parts_{&batch_};        // states holding the last rows, in row order
   void copy_details(BatchState& b, cudaStream_t s);
   Planner planner_;
   bool use_learned_ = false;
   std::unique_ptr<FeatureContext> fctx_;  // built on first use
   const FeatureContext& fctx();
   WorkerPool plan_pool_;  // planning threads, one per hardware thread
   // aggregation: per dictionary column the value id of every row and the values' string order
   std::vector<const uint32_t*> d_dict_ids_, d_dict_rank_;
   std::vector<std::vector<uint32_t>> dict_by_rank_;
   AggDim* d_agg_dims_ = nullptr;
   uint32_t* d_agg_counters_ = nullptr;
   uint32_t* d_agg_blocks_ = nullptr;
   AggCount* d_agg_out_ = nullptr;
   size_t agg_dims_cap_ = 0, agg_counters_cap_ = 0, agg_blocks_cap_ = 0, agg_out_cap_ = 0;
   // MutationProfile row sets of the single-query path
   DevProfile* d_prof_ = nullptr;
   uint32_t* d_prof_data_ = nullptr;
   uint32_t* d_aux_ = nullptr;
   size_t prof_cap_ = 0, prof_data_cap_ = 0, aux_cap_ = 0;
   // Runs the expressions through the single-query path in trace mode; one sample per node.
   size_t collect_traces(const std::vector<std::string>& exprs, std::vector<PlannerSample>& out);

};

// Occupancy of the persistent filter kernel for a given shared-memory stack size.
int filter_batch_blocks_per_sm(size_t smem_bytes);

}  // namespace rhygpu
