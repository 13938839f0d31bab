// Host storage image of one table partition: what ingestion produces and what is uploaded to HBM.
//
// Sequence columns keep the reference's storage semantics:
//  * vertical index: one roaring-style container per (position, 2^16-row chunk, symbol) holding
//    the rows whose symbol differs from the local reference (reference:
//    src/rhydb/storage/column/vertical_sequence_index.h:20-113), with the missing symbol (N / X)
//    never stored there;
//  * coverage: per row the covered [start, end) and the missing positions inside it (reference:
//    src/rhydb/storage/column/horizontal_coverage_index.h:21-114);
//  * local reference: a position whose majority symbol differs from the reference is flipped at
//    finalize (reference: src/rhydb/storage/column/sequence_column.cpp:158-212,
//    vertical_sequence_index.cpp:217-283).
// Containers keep their roaring encodings (array <= 4096 sorted u16, 8 KiB bitset, or runs),
// chosen by the smallest serialized size (reference: src/rhydb/roaring_util/roaring_container.cpp:7-62).
//
// The coverage layout is redesigned for the GPU: rows whose covered region is not the whole genome
// are kept as a short per-chunk exception list, and the missing positions inside coverage are kept
// as intervals bucketed by 128-position blocks, so a coverage tile at one position reads only the
// exceptions and the intervals of one block instead of every row.
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "alphabet.h"
#include "dataset.h"

namespace rhygpu {

constexpr uint32_t CHUNK_ROWS = 1u << 16;  // rows per chunk, reference: src/rhydb/storage/column/column.h:18
constexpr uint32_t CHUNK_WORDS = CHUNK_ROWS / 32;
constexpr uint32_t NBLOCK = 128;           // positions per N-interval bucket

enum CtrType : uint8_t { CT_ARRAY = 0, CT_BITSET = 1, CT_RUN = 2 };

// 16-byte container descriptor, identical on host and device.
struct CtrDesc {
   uint32_t payload;   // offset into the u16 payload arena
   uint32_t key;       // position (sequence column) or value id (dictionary column)
   uint16_t v;         // chunk id (v_index)
   uint8_t sym;        // symbol (sequence column), 0 for dictionary columns
   uint8_t type;       // CtrType
   uint16_t nruns;     // run containers: number of (start, length-1) pairs
   uint16_t card_m1;   // cardinality - 1
};
static_assert(sizeof(CtrDesc) == 16, "descriptor layout");

struct CovExc {  // a row whose covered region is not [0, L)
   uint32_t row;   // row within chunk
   uint32_t start;
   uint32_t end;
   uint32_t pad;
};

struct CovEvent {  // coverage boundary of one row
   uint32_t row;   // global row id
   uint32_t pos;
};

constexpr uint32_t MAX_EVENT_CHUNKS = 256;  // packed mutations events hold 24-bit row ids

constexpr uint32_t TOFF_ROWS = 4096;
constexpr uint32_t TOFF_N = CHUNK_ROWS / TOFF_ROWS + 1;

struct NRunEntry {  // missing interval of one row clipped to one position block
   uint32_t row;    // global row id (chunk << 16 | row within chunk)
   uint16_t lo;     // [lo, hi) relative to the block start
   uint16_t hi;
};

// Totals over all chunks of the containers of one (key, symbol): rows, containers, bitsets.
struct KeyStats {
   uint32_t card = 0;
   uint16_t nctr = 0;
   uint16_t nbits = 0;
};
constexpr uint32_t STAT_SYMS = 32;  // stats slots per key (every alphabet has fewer symbols)

struct ContainerSet {
   std::vector<CtrDesc> ctrs;       // sorted by (v, key, sym)
   std::vector<uint16_t> payload;   // bitset payloads start on 16-byte boundaries
   std::vector<uint32_t> off;       // [nchunks * nkeys + 1]: ctrs of (v, key) are [off[v*nkeys+key], off[...+1])
   uint32_t nkeys = 0;
   std::vector<KeyStats> stats;     // [nkeys * STAT_SYMS]: planning statistics
   uint64_t payload_bytes() const;
   const KeyStats& stat(uint32_t key, uint32_t sym) const { return stats[static_cast<size_t>(key) * STAT_SYMS + sym]; }
};

struct SeqColumnImage {
   std::string name;
   SymKind kind = SymKind::NUC;
   uint32_t L = 0;
   std::string reference;              // global reference chars
   std::vector<uint8_t> global_ref;    // symbols
   std::vector<uint8_t> local_ref;     // symbols after adaptation
   ContainerSet vertical;              // keys = positions
   std::vector<uint32_t> null_rows;    // global row ids (chunk << 16 | row)
   std::vector<CovExc> cov_exc;        // sorted by (chunk, row)
   std::vector<uint32_t> cov_exc_off;  // nchunks + 1
   // Missing positions inside coverage, as intervals: per row CSR over global ids (chunk stride).
   std::vector<uint32_t> nrow_off;     // nchunks * CHUNK_ROWS + 1
   std::vector<uint32_t> nrow_start, nrow_end;
   std::vector<NRunEntry> nblk;        // bucketed by (block, chunk), sorted by row
   std::vector<uint32_t> nblk_off;     // nblocks * nchunks + 1
   // Row-range offsets for tiles: exc_toff[v * TOFF_N + k] is the index of the first coverage
   // exception of chunk v with row >= k * TOFF_ROWS, nblk_toff[(b * nchunks + v) * TOFF_N + k] the
   // same inside bucket (b, v) of nblk.
   std::vector<uint32_t> exc_toff;
   std::vector<uint32_t> nblk_toff;
   uint32_t nblocks = 0;
   // Mutations pass: the same missing intervals as start and end events, packed as
   // (global row << 8 | position within the block, 0..128) and sorted by (block, position, row),
   // so counts per position aggregate over runs of equal positions; per-block offsets.
   std::vector<uint32_t> mstart, mend;
   std::vector<uint32_t> mstart_off, mend_off;  // nblocks + 1
   // Coverage boundaries of rows whose covered region is not the whole genome, sorted by
   // position: starts above 0 and ends below L (a row without coverage has end 0).
   std::vector<CovEvent> cstart, cend;
   // Row index of the same counts, for filters of few rows: per row (global id, chunk stride) one
   // entry (position << 5 | code) per container holding the row (code = its symbol), per coverage
   // boundary above (ROW_COV_START, ROW_COV_END) and per missing interval (ROW_MISS_START at its
   // first position, ROW_MISS_END after its last). Rows of F read their entries instead of every
   // container being tested against F.
   std::vector<uint32_t> hrow_off;     // nchunks * CHUNK_ROWS + 1
   std::vector<uint32_t> hent;
   uint32_t flipped_positions = 0;
};
constexpr uint32_t ROW_COV_START = 28, ROW_COV_END = 29, ROW_MISS_START = 30, ROW_MISS_END = 31;

struct DictColumnImage {
   std::string name;
   std::vector<std::string> values;
   std::map<std::string, uint32_t> index;
   ContainerSet inverted;              // keys = value ids
};

struct DateColumnImage {
   std::string name;
   std::vector<int32_t> days;          // global-id (chunk stride) layout, INT32_MIN = null
};

struct TableImage {
   uint32_t n_rows = 0;
   std::vector<uint32_t> chunk_sizes;
   std::vector<SeqColumnImage> seq;
   std::vector<DictColumnImage> dict;
   std::vector<DateColumnImage> date;
   int primary_key = -1;  // dictionary column holding the primary key (schema primary_key), -1 = none
   uint32_t nchunks() const { return static_cast<uint32_t>(chunk_sizes.size()); }
   int find_seq(const std::string& name) const;
   int find_dict(const std::string& name) const;
   int find_date(const std::string& name) const;
};

// Ingestion: diff every row against the reference, split rows into 2^16-row chunks, build the
// vertical containers, adapt the local reference, choose container encodings.
TableImage build_table(const RawTable& raw, uint32_t threads = 0);

}  // namespace rhygpu
