// Details action on the device: the first k row ids of a filter in ascending order (reference:
// TableScanNode, exec_node/table_scan.h:42-104, which walks the row set from its smallest id).
//
// One CTA per query scans the dense row set in windows of FK_T words: a block prefix sum of the
// words' population counts gives each word's first output slot, every thread writes the ids of its
// word that fall below k, and the scan stops at the window that reaches k.
#include <cuda_runtime.h>

#include "device.h"

namespace rhygpu {

namespace {

constexpr uint32_t FK_T = 256;

__global__ void __launch_bounds__(FK_T) first_k_kernel(const uint32_t* __restrict__ tiles, uint32_t words,
                                                       const uint32_t* __restrict__ k_of,
                                                       const uint32_t* __restrict__ out_off, uint32_t* __restrict__ ids,
                                                       uint32_t* __restrict__ n_out) {
   __shared__ uint32_t wsum[FK_T / 32];
   const uint32_t q = blockIdx.x, k = k_of[q];
   const uint32_t* t = tiles + static_cast<size_t>(q) * words;
   uint32_t* out = ids + out_off[q];
   const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
   uint32_t have = 0;
   for (uint32_t w0 = 0; w0 < words && have < k; w0 += FK_T) {
      const uint32_t w = w0 + threadIdx.x;
      uint32_t x = w < words ? __ldg(t + w) : 0u;
      const uint32_t c = __popc(x);
      uint32_t incl = c;
#pragma unroll
      for (uint32_t o = 1; o < 32; o <<= 1) {
         const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
         if (lane >= o) incl += y;
      }
      if (lane == 31) wsum[warp] = incl;
      __syncthreads();
      uint32_t before = 0, total = 0;
#pragma unroll
      for (uint32_t i = 0; i < FK_T / 32; ++i) {
         before += i < warp ? wsum[i] : 0u;
         total += wsum[i];
      }
      uint32_t at = have + before + incl - c;
      while (x && at < k) {
         const uint32_t b = __ffs(x) - 1;
         x &= x - 1;
         out[at++] = w * 32 + b;
      }
      have += total;
      __syncthreads();  // wsum is rewritten by the next window
   }
   if (threadIdx.x == 0) n_out[q] = have < k ? have : k;
}

}  // namespace

void launch_first_k(const uint32_t* d_tiles, uint32_t nq, uint32_t nchunks, const uint32_t* d_k,
                    const uint32_t* d_out_off, uint32_t* d_ids, uint32_t* d_n, void* stream) {
   if (nq == 0) return;
   first_k_kernel<<<nq, FK_T, 0, static_cast<cudaStream_t>(stream)>>>(d_tiles, nchunks * CHUNK_WORDS, d_k, d_out_off, d_ids,
                                                                       d_n);
}

}  // namespace rhygpu
