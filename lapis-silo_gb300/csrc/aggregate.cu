// Grouped counts of a filter's rows (BitmapAggregation, reference:
// src/rhydb/query_engine/operators/bitmap_aggregation_node.cpp:51-140).
//
//  agg_keys_kernel   one lane per filtered row: its group in every dimension, combined into one
//                    mixed-radix key (dimension 0 most significant), counted in a dense array.
//  agg_nonzero_kernel / agg_write_kernel
//                    the nonzero keys in key order, which is the reference's depth-first order
//                    over the dimensions' groups.
//
// A sequence dimension's groups are the column's symbols in alphabet order and then the null
// group. A row's symbol at the position is that of the container holding it (read from the row
// index), else the missing symbol where the row is not covered or inside a missing interval, else
// the local reference symbol; null rows form the null group. This is the partition
// compileSymbolInSet(column, position, {symbol}) makes for each symbol, with the null rows added
// last (bitmap_aggregation_node.cpp:51-84). A dictionary dimension's groups are its values in string
// order and then the null group (:237-259).
#include <cuda_runtime.h>

#include "aggregate.h"

namespace rhygpu {

namespace {

constexpr uint32_t AT = 256;

__device__ __forceinline__ uint32_t seq_group(const DevSeqCol* __restrict__ cs, uint32_t r, uint32_t pos) {
   if ((__ldg(cs->null_tiles + (r >> 5)) >> (r & 31)) & 1u) return cs->nsym;  // the null group
   const uint32_t b = __ldg(cs->hrow_off + r), e = __ldg(cs->hrow_off + r + 1);
   uint32_t sym = 0xFFFFFFFFu, start = 0, end = cs->L, miss_a = 0;
   bool missing = false;
   for (uint32_t i = b; i < e; ++i) {
      const uint32_t ent = __ldg(cs->hent + i);
      const uint32_t code = ent & 31u, p = ent >> 5;
      if (code < ROW_COV_START) {
         if (p == pos) sym = code;
      } else if (code == ROW_COV_START) {
         start = p;
      } else if (code == ROW_COV_END) {
         end = p;
      } else if (code == ROW_MISS_START) {
         miss_a = p;
      } else if (miss_a <= pos && pos < p) {  // ROW_MISS_END closes [miss_a, p)
         missing = true;
      }
   }
   if (sym != 0xFFFFFFFFu) return sym;
   if (pos < start || pos >= end || missing) return cs->nsym - 1;  // the missing symbol is the last one
   return __ldg(cs->local_ref + pos);
}

__global__ void __launch_bounds__(AT) agg_keys_kernel(const DevTable* __restrict__ tab, const uint32_t* __restrict__ F,
                                                      const AggDim* __restrict__ dims, uint32_t nd,
                                                      uint32_t* __restrict__ counters) {
   const uint32_t words = tab->nchunks * CHUNK_WORDS;
   const uint32_t lane = threadIdx.x & 31;
   const uint32_t warp = (blockIdx.x * AT + threadIdx.x) >> 5, nwarps = gridDim.x * (AT / 32);
   for (uint32_t w = warp; w < words; w += nwarps) {
      const uint32_t x = __ldg(F + w);
      if (!((x >> lane) & 1u)) continue;
      const uint32_t r = 32 * w + lane;
      uint64_t key = 0;
      for (uint32_t d = 0; d < nd; ++d) {
         const AggDim& dim = dims[d];
         uint32_t g;
         if (dim.kind == AGG_SEQUENCE) {
            g = seq_group(&tab->seq[dim.col], r, dim.pos);
         } else {
            const uint32_t id = __ldg(dim.ids + r);
            g = id == 0xFFFFFFFFu ? dim.ngroups - 1 : __ldg(dim.rank + id);
         }
         key += static_cast<uint64_t>(g) * dim.stride;
      }
      atomicAdd(counters + key, 1u);
   }
}

// Nonzero counters per block of AGG_BLOCK keys.
__global__ void __launch_bounds__(AT) agg_nonzero_kernel(const uint32_t* __restrict__ counters, uint64_t keys,
                                                         uint32_t* __restrict__ block_nonzero) {
   __shared__ uint32_t red[AT / 32];
   const uint64_t k0 = static_cast<uint64_t>(blockIdx.x) * AGG_BLOCK;
   uint32_t n = 0;
   for (uint32_t i = threadIdx.x; i < AGG_BLOCK; i += AT) n += (k0 + i < keys && counters[k0 + i] != 0u) ? 1u : 0u;
   n = __reduce_add_sync(0xFFFFFFFFu, n);
   if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = n;
   __syncthreads();
   if (threadIdx.x == 0) {
      uint32_t s = 0;
      for (uint32_t w = 0; w < AT / 32; ++w) s += red[w];
      block_nonzero[blockIdx.x] = s;
   }
}

// (key, count) of the nonzero counters of each block, at the block's offset, in key order.
__global__ void __launch_bounds__(AT) agg_write_kernel(const uint32_t* __restrict__ counters, uint64_t keys,
                                                       const uint32_t* __restrict__ block_off, AggCount* __restrict__ out) {
   __shared__ uint32_t wsum[AT / 32];
   const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
   const uint64_t k0 = static_cast<uint64_t>(blockIdx.x) * AGG_BLOCK;
   uint32_t base = block_off[blockIdx.x];
   for (uint32_t i0 = 0; i0 < AGG_BLOCK; i0 += AT) {
      const uint64_t k = k0 + i0 + threadIdx.x;
      const uint32_t c = k < keys ? counters[k] : 0u;
      const uint32_t m = __ballot_sync(0xFFFFFFFFu, c != 0u);
      if (lane == 0) wsum[warp] = __popc(m);
      __syncthreads();
      uint32_t before = 0, all = 0;
      for (uint32_t w = 0; w < AT / 32; ++w) {
         before += w < warp ? wsum[w] : 0u;
         all += wsum[w];
      }
      if (c) out[base + before + __popc(m & ((1u << lane) - 1u))] = AggCount{k, c};
      base += all;
      __syncthreads();
   }
}

}  // namespace

void launch_agg_keys(const DevTable* d_table, uint32_t nchunks, const uint32_t* d_filter, const AggDim* d_dims,
                     uint32_t nd, uint32_t* d_counters, void* stream) {
   const uint32_t words = nchunks * CHUNK_WORDS;
   const uint32_t grid = (words + AT / 32 - 1) / (AT / 32);
   agg_keys_kernel<<<grid, AT, 0, static_cast<cudaStream_t>(stream)>>>(d_table, d_filter, d_dims, nd, d_counters);
}

void launch_agg_nonzero(const uint32_t* d_counters, uint64_t keys, uint32_t* d_block_nonzero, void* stream) {
   const uint32_t blocks = static_cast<uint32_t>((keys + AGG_BLOCK - 1) / AGG_BLOCK);
   agg_nonzero_kernel<<<blocks, AT, 0, static_cast<cudaStream_t>(stream)>>>(d_counters, keys, d_block_nonzero);
}

void launch_agg_write(const uint32_t* d_counters, uint64_t keys, const uint32_t* d_block_off, AggCount* d_out,
                      void* stream) {
   const uint32_t blocks = static_cast<uint32_t>((keys + AGG_BLOCK - 1) / AGG_BLOCK);
   agg_write_kernel<<<blocks, AT, 0, static_cast<cudaStream_t>(stream)>>>(d_counters, keys, d_block_off, d_out);
}

}  // namespace rhygpu
