// Mutations pass whose working memory is a fixed array in the device image (see noalloc.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "engine.h"

namespace rhygpu {

// Enqueues the Mutations pass of `column` for a filter given in device memory; allocates nothing.
// *d_status (device memory) is cleared; a kernel of the pass would set it to a device error code.
// The first call on a device looks up the array's device address (cudaGetSymbolAddress).
void mutations_noalloc(Engine& engine, uint32_t column, const uint32_t* d_filter, const unsigned long long* d_filter_count,
                       uint32_t* d_counts, int* d_status, cudaStream_t stream);

}  // namespace rhygpu
