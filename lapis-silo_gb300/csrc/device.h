// Device-resident table image and the kernel launch interface.
//
// HBM layout of one partition (all arrays written once at open and read-only afterwards):
//   sequence column: container descriptors (16 B, sorted by chunk, position, symbol), a u16
//   payload arena (arrays, 8 KiB bitsets on 16-byte boundaries, run pairs), the (chunk, position)
//   offset table, per-chunk coverage exceptions, missing-interval buckets per 128-position block,
//   a dense null-row bitmap (8 KiB per chunk) and the local reference;
//   dictionary column: the inverted index in the same container format, keyed by value id;
//   date column: bit-sliced index (one dense bitmap per bit of date - min date) and a null bitmap.
// Row sets are dense bitmaps of 2^16 bits (8 KiB) per chunk.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "program.h"
#include "table.h"

namespace rhygpu {

constexpr int MAX_SEQ_COLS = 32;
constexpr int MAX_DICT_COLS = 8;
constexpr int MAX_DATE_COLS = 8;

// Units of the Mutations container pass (see mut_ring_kernel).
// An array unit: n <= WU elements [e0, e0 + n) of one chunk's array payloads (arrays lie back to
// back in descriptor order; e0 is a multiple of 8, so the unit starts on a 16-byte boundary;
// elements below the chunk's first array belong to no container of the unit) and the nd
// descriptors [c0, c0 + nd) that cover every array overlapping it (bitset and run descriptors
// between them are skipped). The host cuts units so that nd <= WU_DESC wherever it can.
constexpr uint32_t WU = 1024;
constexpr uint32_t WU_DESC = 64;
struct ArrUnit {
   uint32_t e0;
   uint32_t c0;
   uint16_t n, nd;
   uint32_t v;
};
static_assert(sizeof(ArrUnit) == 16, "array unit record");
// A bitset (kind SU_BITSET: its 4096 u16 at e0) or run container (SU_RUN), descriptor c.
enum : uint32_t { SU_BITSET = 1, SU_RUN = 2 };
struct OtherUnit {
   uint32_t kind;
   uint32_t v;
   uint32_t e0;
   uint32_t c;
};
// The work of one CTA of the container pass: array units [a0, a1) and other units [o0, o1), all
// of chunks v0 and v1 (v1 == v0 for one chunk).
struct StreamRange {
   uint32_t a0, a1, o0, o1, v0, v1, pad[2];
};
// CTAs of the container pass per SM (its shared-memory ring sets this); one range per CTA.
constexpr uint32_t RING_CTAS_PER_SM = 3;

struct DevSeqCol {
   const CtrDesc* ctrs;
   const uint16_t* payload;
   const uint32_t* off;        // nchunks * L + 1
   const CovExc* exc;
   const uint32_t* exc_off;    // nchunks + 1
   const NRunEntry* nblk;
   const uint32_t* nblk_off;   // nblocks * nchunks + 1
   const ArrUnit* au;          // array units of the Mutations container pass, chunk-major
   const OtherUnit* ou;        // its bitset and run units, chunk-major
   const StreamRange* ranges;  // its CTAs
   const uint32_t* exc_toff;   // nchunks * TOFF_N: tile row-range offsets into exc
   const uint32_t* nblk_toff;  // nblocks * nchunks * TOFF_N: the same into each nblk bucket
   const uint32_t* null_tiles; // nchunks * CHUNK_WORDS
   const uint8_t* local_ref;   // L
   const uint32_t* mstart;     // missing-interval start events (row << 8 | position in block)
   const uint32_t* mend;       // missing-interval end events
   const CovEvent* cstart;     // coverage starts > 0
   const CovEvent* cend;       // coverage ends < L
   const uint32_t* hrow_off;   // row index: nchunks * CHUNK_ROWS + 1 offsets into hent
   const uint32_t* hent;       // row index entries (position << 5 | code)
   uint32_t L;
   uint32_t nblocks;
   uint32_t nsym;
   uint32_t nctrs;
   uint32_t nau;
   uint32_t nranges;
   uint32_t valid_mask;        // symbols counted in a position's coverage (valid mutation symbols)
   const uint8_t* global_ref;  // L: the column's reference symbols (the "from" of a mutation)
   char chars[32];             // symbol -> character
};

// A range of events of one list for the mutations coverage pass.
enum : uint32_t { EV_MSTART = 0, EV_MEND = 1, EV_CSTART = 2, EV_CEND = 3 };
struct EvItem {
   uint32_t list;   // EV_*
   uint32_t block;  // position block (missing lists)
   uint32_t begin;
   uint32_t end;
};

struct DevDictCol {
   const CtrDesc* ctrs;
   const uint16_t* payload;
   const uint32_t* off;        // nchunks * nkeys + 1
   uint32_t nkeys;
   uint32_t pad;
};

// Date column as a bit-sliced index: plane i holds bit i of (date - base) for every row (dense,
// nchunks * CHUNK_WORDS words per plane), `nulls` the rows without a date. A range predicate then
// reads nbits + 1 bits per row instead of a 32-bit value.
constexpr uint32_t MAX_DATE_BITS = 32;
struct DevDateCol {
   const uint32_t* planes;     // nbits * nchunks * CHUNK_WORDS
   const uint32_t* nulls;      // nchunks * CHUNK_WORDS
   int64_t base;               // smallest date
   uint32_t nbits;             // 1..32
   uint32_t pad;
};

struct DevTable {
   uint32_t nchunks;
   uint32_t n_rows;
   const uint32_t* chunk_sizes;
   DevSeqCol seq[MAX_SEQ_COLS];
   DevDictCol dict[MAX_DICT_COLS];
   DevDateCol date[MAX_DATE_COLS];
};

// Per-query scratch of the mutations pass, in u32 words:
//   start_hist[L+1] | end_hist[L+1] | missing_diff[L+1] | seg_start[nseg] | seg_end[nseg] | seg_missing[nseg]
// The histograms are difference arrays over positions; the segment totals (MUT_SEG positions each)
// let every CTA of the final pass start its prefix sums without scanning the whole genome.
constexpr uint32_t MUT_SEG = 1024;
__host__ __device__ inline uint32_t mut_nseg(uint32_t L) { return (L + 1 + MUT_SEG - 1) / MUT_SEG; }
__host__ __device__ inline size_t mut_scratch_words(uint32_t L) { return 3ull * (L + 1) + 3ull * mut_nseg(L); }

// One unit of the batched filter kernel: tile `tile` of query `query`.
struct WorkItem {
   uint32_t query;
   uint32_t tile;
};

struct QueryDesc {
   uint32_t code_off;     // offset of the program in the shared instruction buffer
   uint32_t code_len;
   uint32_t out_tiles;    // 1 = write the row set to the query's output tiles
   uint32_t n_leaves;     // container leaves | coverage leaves << 16 (numbered 1.. in their c field)
   uint32_t depth;        // stack tiles the program uses; the rest of the CTA's stack stages payloads
   uint32_t aux_base;     // its PUSH_AUX row sets are aux tiles aux_base + a
   uint32_t tile_bits;    // rows per work item of this query (its class's tile width)
};

// A MutationProfile row set to compute before the filter programs (see ProfileSpec): the column,
// the distance and the counting terms in device memory, terms[p] = (mask[p], diff[p]) for
// p <= L (mask[L] = 0), so that any row-index entry needs one 8-byte load.
struct DevProfile {
   uint32_t col, distance, base, pad;
   const uint2* terms;
};
// aux[k] (nchunks * CHUNK_WORDS words each) = the rows of profiles[k] within its distance.
// max_L: the longest genome among the profiles' columns.
void launch_profiles(const DevTable* d_table, uint32_t nchunks, const DevProfile* d_profiles, uint32_t n,
                     uint32_t max_L, uint32_t* d_aux, void* stream);

// ---- launchers (kernels.cu) ----
// tile_bits: 4096, 8192, 16384, 32768 or 65536. stack_tiles: program depth. n_leaves: container
// leaves | coverage leaves << 16. d_trace (trace mode, optional): nchunks * (CHUNK_ROWS / tile_bits)
// tiles x ncode x 2 u32 (cycles, result popcount per executed instruction), zeroed by the caller.
cudaError_t launch_filter(const DevTable* d_table, uint32_t nchunks, const Instr* d_code, uint32_t ncode,
                          uint32_t n_leaves, uint32_t tile_bits, uint32_t stack_tiles, uint32_t* d_out_tiles,
                          unsigned long long* d_count, int* d_err, void* stream, uint32_t* d_trace = nullptr,
                          const uint32_t* d_aux = nullptr);

// Batched: n_items work items over the programs in d_code; CTAs pull items from *d_next. Every
// item uses its query's tile width (QueryDesc.tile_bits); stack_bytes of shared memory per CTA hold
// the program stack of any of them (depth x tile bytes) and staged payloads in the rest.
cudaError_t launch_filter_batch(const DevTable* d_table, uint32_t nchunks, const Instr* d_code, const QueryDesc* d_queries,
                         const WorkItem* d_items, uint32_t n_items, uint32_t stack_bytes,
                         uint32_t* d_out_tiles /* per query nchunks*CHUNK_WORDS */, unsigned long long* d_counts,
                         uint32_t* d_next, uint32_t grid, int* d_err, void* stream, const uint32_t* d_aux = nullptr);

// Device error codes the kernels set in their error word: a bounded wait for bulk copies gave up
// in a filter kernel (6) or in the Mutations container pass (7).
enum : int { DEVERR_WAIT_FILTER = 6, DEVERR_WAIT_MUTATIONS = 7 };

// Sets the container pass's shared-memory size on the current device (once per device, before
// its first launch).
void mutations_setup();

// Kernel selection masks (all bits set = the whole pass); used to time the kernels one by one.
enum : uint32_t { MUT_PART_CTR = 1, MUT_PART_COV = 2, MUT_PART_FINAL = 4, MUT_PART_ALL = 7 };
enum : uint32_t { BMUT_PART_TRANSPOSE = 1, BMUT_PART_CTR = 2, BMUT_PART_COV = 4, BMUT_PART_FINAL = 8, BMUT_PART_ALL = 15 };

// Mutations. counts: nsym * L u32 and scratch: mut_scratch_words(L) u32, both zeroed by the caller.
// The filter count decides on the device between the full path (|F| == rows: stored cardinalities),
// the empty path and the mixed path, so no host round trip sits between filter and mutations.
// Filters of at most sparse_max rows (0: none) take the row-index pass (part MUT_PART_SPARSE) instead
// of the container and coverage passes: their rows read their row-index entries.
enum : uint32_t { MUT_PART_SPARSE = 8 };
void launch_mutations(const DevTable* d_table, const DevSeqCol& col_host, uint32_t col, uint32_t nchunks,
                      const EvItem* d_ev, uint32_t n_ev, const uint32_t* d_filter,
                      const unsigned long long* d_filter_count, uint32_t* d_counts, uint32_t* d_scratch, int* d_err,
                      void* stream, uint32_t parts = MUT_PART_ALL | MUT_PART_SPARSE, uint64_t sparse_max = 0);
// Testing the failure path of the filter kernels' bounded waits on the current device: while on,
// the leaf payload copies they announce are never issued, so their waits give up and the kernels
// set error 6 (DEVERR_WAIT_FILTER) instead of evaluating. Nothing is left in flight.
void set_copy_withholding(bool on);
// The same for the Mutations container pass (mutations.cu): while on, its slot copies are announced
// but withheld, so its consumers' waits give up and it sets DEVERR_WAIT_MUTATIONS.
void set_ring_withholding(bool on);

// One unit of the batched container pass: the containers of position `pos` in chunks [v0, v1),
// at most CTR_UNIT_CHUNKS chunks and, unless a single chunk exceeds it, CTR_UNIT_ELEMENTS elements.
struct CtrUnit {
   uint32_t pos;
   uint16_t v0, v1;
};
constexpr uint32_t CTR_UNIT_CHUNKS = 32;
constexpr uint32_t CTR_UNIT_ELEMENTS = 4096;

// Batched mutations over nq filters (slot-major dense tiles, nchunks * CHUNK_WORDS each):
// counts[slot][nsym][L] and scratch[slot][mut_scratch_words(L)] zeroed by the caller;
// d_fcounts[d_slot_query[slot]] is the cardinality of the slot's filter; d_masks holds
// mutations_batch_mask_bytes(nq, nchunks); d_units lists the column's container units, heaviest first.
// On the device, once the filters are known, the slots split by their filter's cardinality: empty
// filters need no pass, filters of at most sparse_max rows (0: none) take the row-index pass (part
// BMUT_PART_SPARSE), the others the dense passes over the slots listed in d_lists (2 * nq + 2 u32
// of scratch: the dense and the sparse slot lists and their lengths). With d_rowblk, the final
// pass also counts every slot's Mutations output rows (minimum proportion d_min_prop[slot]) per
// block of ROWS_BLOCK positions into d_rowblk, as launch_rows_count would.
enum : uint32_t { BMUT_PART_SPARSE = 16 };
size_t mutations_batch_mask_bytes(uint32_t nq, uint32_t nchunks);
void launch_mutations_batch(const DevTable* d_table, const DevSeqCol& col_host, uint32_t col, uint32_t nchunks,
                            const uint32_t* d_filters, uint32_t nq, const unsigned long long* d_fcounts,
                            const uint32_t* d_slot_query, const EvItem* d_ev, uint32_t n_ev, const CtrUnit* d_units,
                            uint32_t n_units, uint16_t* d_masks, uint32_t* d_counts, uint32_t* d_scratch,
                            uint32_t* d_lists, uint64_t sparse_max, void* stream,
                            uint32_t parts = BMUT_PART_ALL | BMUT_PART_SPARSE, const double* d_min_prop = nullptr,
                            uint32_t* d_rowblk = nullptr);

// Output rows of the Mutations action (same layout as RhyMutationRow in the C-ABI header).
struct DevMutationRow {
   uint32_t position;  // 1-based
   char from, to;
   uint16_t pad;
   uint32_t count;
   uint32_t coverage;
   double proportion;
};
static_assert(sizeof(DevMutationRow) == 24, "row layout");

// Rows of nq query slots whose dense counts lie at d_counts + slot * nsym * L, with per-slot minimum
// proportions. The batched final pass counts them (launch_mutations_batch with d_rowblk):
// d_blk[slot * rows_blocks(L) + b] = rows of position block b; the scan turns n entries into
// exclusive offsets with the total at d_blk[n]; the write pass emits the rows at their offsets in
// (slot, position, symbol) order, skipping the blocks without rows.
constexpr uint32_t ROWS_BLOCK = 1024;
uint32_t rows_blocks(uint32_t L);
void launch_rows_scan(uint32_t* d_blk, uint32_t n, void* stream);
void launch_rows_write(const DevTable* d_table, const DevSeqCol& col_host, uint32_t col, const uint32_t* d_counts,
                       uint32_t nq, const double* d_min_prop, const uint32_t* d_blk, DevMutationRow* d_rows,
                       void* stream);

// Details: the first k_of[q] row ids (ascending) of each of nq dense row sets (nchunks * CHUNK_WORDS
// words apart) to d_ids + out_off[q]; d_n[q] receives min(k, |row set|).
void launch_first_k(const uint32_t* d_tiles, uint32_t nq, uint32_t nchunks, const uint32_t* d_k,
                    const uint32_t* d_out_off, uint32_t* d_ids, uint32_t* d_n, void* stream);

// Events per CTA of the coverage pass.
constexpr uint32_t EV_PER_CTA = 8192;

}  // namespace rhygpu
