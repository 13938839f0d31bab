// Output rows of the Mutations action on the device (reference: mutations_node.cpp:292-366).
//
// For every query slot and position: total = sum of the counts of the valid mutation symbols;
// positions with total 0 are skipped; threshold = (min_proportion == 0) ? 0
// : u32(ceil(total * min_proportion) - 1); every valid symbol other than the global reference
// symbol whose count exceeds the threshold yields (position + 1, from, to, count, coverage = total,
// proportion = count / total). The double operations are single IEEE operations (a product, ceil,
// a quotient), so the values equal the host's bit for bit.
//
// Three steps keep the output packed and in (slot, position, symbol) order:
//   the batched final pass (mut_final_batch_kernel) counts the rows per block of ROWS_BLOCK
//                      positions of every slot, from the counts it has just completed
//   rows_scan_kernel   exclusive prefix over all (slot, block) counts; the total follows them
//   rows_write_kernel  recomputes the rows of each block that has any and writes them at their
//                      offsets (blocks without rows, most of them, read no counts)
#include <cuda_runtime.h>

#include <cmath>

#include "device.h"
#include "rows_rule.cuh"

namespace rhygpu {

namespace {

constexpr uint32_t RT = ROWS_BLOCK;  // one thread per position

__device__ __forceinline__ PosRows position_rows(const DevSeqCol* __restrict__ cs, const uint32_t* __restrict__ c,
                                                 uint32_t p, double min_prop) {
   const uint32_t L = cs->L;
   return position_rows(cs, p, min_prop, [&](uint32_t s) { return __ldg(c + static_cast<size_t>(s) * L + p); });
}

__device__ __forceinline__ uint32_t block_scan_excl(uint32_t x, uint32_t* wsum, uint32_t* total) {
   const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
   uint32_t incl = x;
#pragma unroll
   for (uint32_t o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
      if (lane >= o) incl += y;
   }
   if (lane == 31) wsum[warp] = incl;
   __syncthreads();
   uint32_t before = 0, all = 0;
   for (uint32_t w = 0; w < nw; ++w) {
      const uint32_t v = wsum[w];
      before += w < warp ? v : 0u;
      all += v;
   }
   *total = all;
   return before + incl - x;
}

// One CTA: exclusive prefix sum over n entries in place, the total written to blk[n].
__global__ void __launch_bounds__(RT) rows_scan_kernel(uint32_t* blk, uint32_t n) {
   __shared__ uint32_t wsum[RT / 32];
   const uint32_t per = (n + RT - 1) / RT;
   const uint32_t b = threadIdx.x * per, e = min(b + per, n);
   uint32_t s = 0;
   for (uint32_t i = b; i < e; ++i) s += blk[i];
   uint32_t total;
   uint32_t run = block_scan_excl(s, wsum, &total);
   for (uint32_t i = b; i < e; ++i) {
      const uint32_t x = blk[i];
      blk[i] = run;
      run += x;
   }
   if (threadIdx.x == 0) blk[n] = total;
}

__global__ void __launch_bounds__(RT) rows_write_kernel(const DevTable* __restrict__ tab, uint32_t col,
                                                        const uint32_t* __restrict__ counts,
                                                        const double* __restrict__ min_prop,
                                                        const uint32_t* __restrict__ blk, DevMutationRow* rows) {
   __shared__ uint32_t wsum[RT / 32];
   const size_t bi = static_cast<size_t>(blockIdx.y) * gridDim.x + blockIdx.x;
   const uint32_t at0 = blk[bi];
   if (blk[bi + 1] == at0) return;  // a block without rows (the scan's next entry, or its total, is equal)
   const DevSeqCol* cs = &tab->seq[col];
   const uint32_t q = blockIdx.y, p = blockIdx.x * RT + threadIdx.x;
   const uint32_t L = cs->L;
   const uint32_t* c = counts + static_cast<size_t>(q) * cs->nsym * L;
   PosRows r{0, 0, 0, 0};
   if (p < L) r = position_rows(cs, c, p, min_prop[q]);
   uint32_t total;
   uint32_t at = at0 + block_scan_excl(r.n, wsum, &total);
   if (r.n == 0) return;
   const uint32_t valid = cs->valid_mask;
   for (uint32_t s = 0; s < cs->nsym; ++s) {
      if (!((valid >> s) & 1u) || s == r.ref) continue;
      const uint32_t k = __ldg(c + static_cast<size_t>(s) * L + p);
      if (k <= r.thr) continue;
      DevMutationRow o;
      o.position = p + 1;
      o.from = cs->chars[r.ref];
      o.to = cs->chars[s];
      o.pad = 0;
      o.count = k;
      o.coverage = r.total;
      o.proportion = static_cast<double>(k) / static_cast<double>(r.total);
      rows[at++] = o;
   }
}

}  // namespace

uint32_t rows_blocks(uint32_t L) { return (L + RT - 1) / RT; }

void launch_rows_scan(uint32_t* d_blk, uint32_t n, void* stream) {
   rows_scan_kernel<<<1, RT, 0, static_cast<cudaStream_t>(stream)>>>(d_blk, n);
}

void launch_rows_write(const DevTable* d_table, const DevSeqCol& col_host, uint32_t col, const uint32_t* d_counts,
                       uint32_t nq, const double* d_min_prop, const uint32_t* d_blk, DevMutationRow* d_rows,
                       void* stream) {
   if (nq == 0) return;
   rows_write_kernel<<<dim3(rows_blocks(col_host.L), nq), RT, 0, static_cast<cudaStream_t>(stream)>>>(
      d_table, col, d_counts, d_min_prop, d_blk, d_rows);
}

}  // namespace rhygpu
