// The row rule of the Mutations output for one position (reference: mutations_node.cpp:292-366),
// shared by the row kernels and the batched final pass, which counts the rows of its positions
// while it has their counts at hand.
#pragma once

#include <cuda_runtime.h>

#include <cmath>

#include "device.h"

namespace rhygpu {

struct PosRows {
   uint32_t n;      // rows of this position
   uint32_t total;  // coverage
   uint32_t thr;    // counts above it are reported
   uint32_t ref;    // global reference symbol
};

// total = sum of the counts of the valid symbols (0: no rows); threshold = (min_prop == 0) ? 0 :
// u32(ceil(total * min_prop) - 1); a row for every valid symbol other than the global reference
// whose count exceeds the threshold. count(s) returns the count of symbol s at p.
template <typename CountOf>
__device__ __forceinline__ PosRows position_rows(const DevSeqCol* __restrict__ cs, uint32_t p, double min_prop,
                                                 CountOf&& count) {
   PosRows r{0, 0, 0, 0};
   const uint32_t nsym = cs->nsym, valid = cs->valid_mask;
   for (uint32_t s = 0; s < nsym; ++s)
      if ((valid >> s) & 1u) r.total += count(s);
   if (r.total == 0) return r;
   r.thr = min_prop == 0.0 ? 0u : static_cast<uint32_t>(ceil(static_cast<double>(r.total) * min_prop) - 1.0);
   r.ref = __ldg(cs->global_ref + p);
   for (uint32_t s = 0; s < nsym; ++s)
      if (((valid >> s) & 1u) && s != r.ref && count(s) > r.thr) ++r.n;
   return r;
}

}  // namespace rhygpu
