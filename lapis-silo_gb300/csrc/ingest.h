// Ingestion on the GPU: the storage image of a raw table built with the sequence columns' heavy
// stages on one device (reference: SequenceColumn::appendChunk + finalize,
// src/rhydb/storage/column/sequence_column.cpp:100-212, table_inserter.cpp:279-343). The result
// equals build_table's: the same containers in the same layout, the same local references, row
// records, events and row index.
#pragma once

#include <cstdint>

#include "table.h"

namespace rhygpu {

TableImage build_table_gpu(const RawTable& raw, int device, uint32_t threads = 0);

}  // namespace rhygpu
