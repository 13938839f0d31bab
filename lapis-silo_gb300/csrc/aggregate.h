// Grouped counts of a filter's rows by sequence positions and dictionary columns (BitmapAggregation,
// reference: src/rhydb/query_engine/operators/bitmap_aggregation_node.cpp:51-140).
#pragma once

#include <cstdint>

#include "device.h"

namespace rhygpu {

enum : uint32_t { AGG_SEQUENCE = 0, AGG_DICTIONARY = 1 };

// One grouping dimension on the device. Group indices: a sequence column's symbols (alphabet order)
// then null; a dictionary column's values in string order (rank[value id]) then null.
struct AggDim {
   uint32_t kind;            // AGG_*
   uint32_t col;             // sequence or dictionary column
   uint32_t pos;             // sequence: 0-based position
   uint32_t ngroups;         // groups of this dimension, the null group last
   uint64_t stride;          // weight of this dimension's group index in the key
   const uint32_t* ids;      // dictionary: value id per row (global id, chunk stride), UINT32_MAX = null
   const uint32_t* rank;     // dictionary: value id -> rank of the value in string order
};

struct AggCount {
   uint64_t key;
   uint32_t count;
   uint32_t pad;
};

constexpr uint32_t AGG_BLOCK = 4096;     // keys per block of the compaction
constexpr uint64_t AGG_MAX_KEYS = 1ull << 26;  // dense key space at most (256 MiB of counters)

// counters[key] += 1 for every row of the filter (dense, nchunks * CHUNK_WORDS words).
void launch_agg_keys(const DevTable* d_table, uint32_t nchunks, const uint32_t* d_filter, const AggDim* d_dims,
                     uint32_t nd, uint32_t* d_counters, void* stream);
// Nonzero counters per block of AGG_BLOCK keys, then their (key, count) at the blocks' offsets.
void launch_agg_nonzero(const uint32_t* d_counters, uint64_t keys, uint32_t* d_block_nonzero, void* stream);
void launch_agg_write(const uint32_t* d_counters, uint64_t keys, const uint32_t* d_block_off, AggCount* d_out,
                      void* stream);

}  // namespace rhygpu
