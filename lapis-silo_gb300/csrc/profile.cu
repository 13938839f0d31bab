// MutationProfile row sets (reference: src/rhydb/query_engine/scalar_expressions/mutation_profile.cpp:198-257).
//
// The reference rewrites a profile into Not(NOf(distance + 1, one SymbolInSet per position)), a
// threshold over up to a genome's length of children. Here every row counts its differences from
// the row index in one pass: a covered row holding the local reference everywhere has `base`
// differences; each of its own symbols replaces the local reference's term at its position, and
// the positions it does not cover (outside its covered region or inside a missing interval) take
// the missing symbol's term instead, summed with the prefix counts. Null rows match no SymbolInSet,
// so they count no difference. A row is in the set when its count is at most the distance.
#include <cuda_runtime.h>

#include "device.h"

namespace rhygpu {

namespace {

constexpr uint32_t PT = 256;

__device__ __forceinline__ uint32_t profile_differences(const DevSeqCol* __restrict__ cs, const DevProfile& pr,
                                                        uint32_t r) {
   if ((__ldg(cs->null_tiles + (r >> 5)) >> (r & 31)) & 1u) return 0u;
   const uint32_t L = cs->L;
   const uint32_t b = __ldg(cs->hrow_off + r), e = __ldg(cs->hrow_off + r + 1);
   int64_t n = pr.base;
   uint32_t start = 0, end = L, miss_a = 0;
   auto uncovered = [&](uint32_t a, uint32_t z) {  // positions [a, z) hold the missing symbol
      n += static_cast<int64_t>(__ldg(pr.pmis + z)) - __ldg(pr.pmis + a);
      n -= static_cast<int64_t>(__ldg(pr.ploc + z)) - __ldg(pr.ploc + a);
   };
   for (uint32_t i = b; i < e; ++i) {
      const uint32_t ent = __ldg(cs->hent + i);
      const uint32_t code = ent & 31u, p = ent >> 5;
      if (code < ROW_COV_START) {
         const uint32_t m = __ldg(pr.mask + p);
         n += static_cast<int64_t>((m >> code) & 1u) - static_cast<int64_t>((m >> __ldg(cs->local_ref + p)) & 1u);
      } else if (code == ROW_COV_START) {
         start = p;
      } else if (code == ROW_COV_END) {
         end = p;
      } else if (code == ROW_MISS_START) {
         miss_a = p;
      } else {
         uncovered(miss_a, p);
      }
   }
   if (end < start) end = start;  // a row without coverage: [0, 0) covered
   uncovered(0, start);
   uncovered(end, L);
   return n < 0 ? 0u : static_cast<uint32_t>(n);
}

// grid (row words / 8, profiles): one lane per row.
__global__ void __launch_bounds__(PT) profile_kernel(const DevTable* __restrict__ tab,
                                                     const DevProfile* __restrict__ profiles,
                                                     uint32_t* __restrict__ aux) {
   const DevProfile pr = profiles[blockIdx.y];
   const DevSeqCol* cs = &tab->seq[pr.col];
   const uint32_t words = tab->nchunks * CHUNK_WORDS;
   const uint32_t lane = threadIdx.x & 31;
   const uint32_t w = (blockIdx.x * PT + threadIdx.x) >> 5;
   if (w >= words) return;  // the whole warp leaves
   const uint32_t r = 32 * w + lane;
   const bool valid = (r & (CHUNK_ROWS - 1)) < __ldg(tab->chunk_sizes + (r >> 16));
   const bool in = valid && profile_differences(cs, pr, r) <= pr.distance;
   const uint32_t bits = __ballot_sync(0xFFFFFFFFu, in);
   if (lane == 0) aux[static_cast<size_t>(blockIdx.y) * words + w] = bits;
}

}  // namespace

void launch_profiles(const DevTable* d_table, uint32_t nchunks, const DevProfile* d_profiles, uint32_t n, uint32_t* d_aux,
                     void* stream) {
   const uint32_t words = nchunks * CHUNK_WORDS;
   for (uint32_t k = 0; k < n; k += 65535) {  // grid.y is at most 65535
      const uint32_t m = n - k < 65535 ? n - k : 65535;
      profile_kernel<<<dim3((words + PT / 32 - 1) / (PT / 32), m), PT, 0, static_cast<cudaStream_t>(stream)>>>(
         d_table, d_profiles + k, d_aux + static_cast<size_t>(k) * words);
   }
}

}  // namespace rhygpu
