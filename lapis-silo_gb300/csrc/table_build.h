// Stages of building a table's storage image, shared by the host ingestion (table.cpp) and the GPU
// ingestion (ingest.cu): both produce, per sequence column, the same per-chunk row records and the
// same containers, and finish the column with the same host code.
#pragma once

#include <cstdint>
#include <vector>

#include "table.h"

namespace rhygpu {

// One chunk's rows of a sequence column as ingestion records them (reference: the coverage and
// mutations of extractCoverageAndMutationsFromSequence, aligned_sequence.cpp:19-122): the
// (position, symbol, row) keys of symbols other than the reference's (host ingestion only), rows
// whose covered region is not the whole genome (null and fully missing rows as {row, 0, 0}), the
// missing intervals inside each row's covered region (CSR over the chunk's rows) and the null rows
// (global ids).
struct ChunkRows {
   std::vector<uint64_t> keys;
   std::vector<CovExc> exc;
   std::vector<uint32_t> nr_off;  // chunk_size + 1
   std::vector<uint32_t> nr_s, nr_e;
   std::vector<uint32_t> nulls;
};

// Name, kind, length and reference symbols of a column (local reference = global reference).
void init_seq_column(const RawSeqColumn& raw, SeqColumnImage& col);
// Everything derived from the chunks' row records and the finished containers: the coverage
// exceptions, null rows, missing intervals (per row and bucketed by position block), the tile
// offsets, the Mutations events and the row index.
void finish_seq_column(SeqColumnImage& col, const std::vector<ChunkRows>& chunks, const std::vector<uint32_t>& chunk_sizes,
                       uint32_t threads);
// The table's row count and chunk sizes (checks every sequence column's row count).
void build_table_frame(const RawTable& raw, TableImage& t);
// The planning statistics and the (chunk, key) offset table of a container set whose descriptors
// (sorted by chunk, key, symbol) and nkeys are set.
void finish_container_set(ContainerSet& cs, uint32_t nchunks);
// Dictionary and date columns.
void build_metadata_columns(const RawTable& raw, TableImage& t, uint32_t threads);

}  // namespace rhygpu
