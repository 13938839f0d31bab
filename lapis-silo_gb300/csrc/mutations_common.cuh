// Device helpers shared by the single-query and batched Mutations kernels.
#pragma once

#include <cuda_runtime.h>

#include "device.h"

namespace rhygpu {

// mbarrier + TMA bulk-copy helpers. A barrier is initialised with one arrival; the issuing thread
// arrives with the expected byte count of the copies it then starts, whose completion flips the
// phase.
__device__ __forceinline__ void mbar_init(uint64_t* bar) {
   const uint32_t b = static_cast<uint32_t>(__cvta_generic_to_shared(bar));
   asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b));
   asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// One arrival that announces `bytes` of bulk copies completing on `bar`; the copies are then issued
// with bulk_copy_g2s_tx. Called by one thread.
__device__ __forceinline__ void mbar_expect(uint64_t* bar, uint32_t bytes) {
   const uint32_t b = static_cast<uint32_t>(__cvta_generic_to_shared(bar));
   asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
   asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}\n" ::"r"(b), "r"(bytes)
                : "memory");
}
__device__ __forceinline__ void bulk_copy_g2s_tx(void* smem, const void* gmem, uint32_t bytes, uint64_t* bar) {
   const uint32_t s = static_cast<uint32_t>(__cvta_generic_to_shared(smem));
   const uint32_t b = static_cast<uint32_t>(__cvta_generic_to_shared(bar));
   asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(s),
                "l"(gmem), "r"(bytes), "r"(b)
                : "memory");
}

// Nanoseconds of the GPU's global timer.
__device__ __forceinline__ uint64_t global_ns() {
   uint64_t t;
   asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
   return t;
}

// Limits of the bounded waits for bulk copies: normally 2 s (a copy lands in microseconds), 1 ms
// while a test withholds copies on purpose.
constexpr uint64_t WAIT_LIMIT_NS = 2000000000ull;
constexpr uint64_t WAIT_LIMIT_TEST_NS = 1000000ull;

// popcount of F in [a, b)
__device__ __forceinline__ uint32_t count_range(const uint32_t* F, uint32_t a, uint32_t b) {
   if (a >= b) return 0;
   const uint32_t wa = a >> 5, wb = (b - 1) >> 5;
   uint32_t s = 0;
   for (uint32_t w = wa; w <= wb; ++w) {
      uint32_t m = 0xFFFFFFFFu;
      if (w == wa) m &= 0xFFFFFFFFu << (a & 31);
      if (w == wb) m &= 0xFFFFFFFFu >> (31 - ((b - 1) & 31));
      s += __popc(F[w] & m);
   }
   return s;
}

__device__ __forceinline__ uint32_t block_incl_scan_u32(uint32_t v, uint32_t* red) {
   const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
   uint32_t x = v;
#pragma unroll
   for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
      if (static_cast<int>(lane) >= o) x += y;
   }
   __syncthreads();
   if (lane == 31) red[warp] = x;
   __syncthreads();
   uint32_t add = 0;
   for (uint32_t i = 0; i < warp; ++i) add += red[i];
   __syncthreads();
   return x + add;
}

// Final pass for positions [blockIdx.x * MUT_SEG, +MUT_SEG) of one query (blockDim.x == MUT_SEG):
//   ref(p) = |F| - #(start > p) - #(end <= p) - missing(p) - sum_s counts[s][p]
//   counts[local_ref[p]][p] += ref(p)
// All arithmetic is modulo 2^32 like the reference's uint32 vectors; the result is exact.
__device__ __forceinline__ void final_position_counts(const DevSeqCol* cs, uint32_t total, uint32_t* counts,
                                                      const uint32_t* __restrict__ scratch, uint32_t* red) {
   __shared__ uint32_t pre[4];
   const uint32_t L = cs->L, nsym = cs->nsym, nseg = mut_nseg(L);
   const uint32_t* start_hist = scratch;
   const uint32_t* end_hist = scratch + (L + 1);
   const uint32_t* ndiff = scratch + 2 * (L + 1);
   const uint32_t* seg_s = scratch + 3 * (L + 1);
   const uint32_t* seg_e = seg_s + nseg;
   const uint32_t* seg_n = seg_e + nseg;
   if (threadIdx.x < 32) {
      uint32_t ps = 0, pe = 0, pn = 0, ts = 0;
      for (uint32_t k = threadIdx.x; k < nseg; k += 32) {
         const uint32_t s = seg_s[k];
         ts += s;
         if (k < blockIdx.x) {
            ps += s;
            pe += seg_e[k];
            pn += seg_n[k];
         }
      }
      ps = __reduce_add_sync(0xFFFFFFFFu, ps);
      pe = __reduce_add_sync(0xFFFFFFFFu, pe);
      pn = __reduce_add_sync(0xFFFFFFFFu, pn);
      ts = __reduce_add_sync(0xFFFFFFFFu, ts);
      if (threadIdx.x == 0) {
         pre[0] = ps;
         pre[1] = pe;
         pre[2] = pn;
         pre[3] = ts;
      }
   }
   __syncthreads();
   const uint32_t p = blockIdx.x * MUT_SEG + threadIdx.x;
   const bool in = p < L;
   const uint32_t sl = block_incl_scan_u32(in ? start_hist[p] : 0u, red) + pre[0];
   const uint32_t el = block_incl_scan_u32(in ? end_hist[p] : 0u, red) + pre[1];
   const uint32_t nl = block_incl_scan_u32(in ? ndiff[p] : 0u, red) + pre[2];
   if (in) {  // no early return: a caller may follow with barriers
      uint32_t ref = total - (pre[3] - sl) - el - nl;
      for (uint32_t s = 0; s < nsym; ++s) ref -= counts[static_cast<size_t>(s) * L + p];
      counts[static_cast<size_t>(cs->local_ref[p]) * L + p] += ref;
   }
}

// Row-index pass over 32 words [w, w + 32) of a dense filter F (words in all): every row of F there
// adds its row-index entries, which are exactly what the container and coverage passes add for
// that row: symbol entries to counts[symbol][position]; coverage starts and ends to their
// histograms, missing-interval starts (+1) and ends (-1, modulo 2^32) to the difference array, each
// also to its segment total. The warp gathers the rows into `list` (1,024 entries), then takes them
// 32 at a time: one lane loads one row's entry range, and the rows' entries, numbered across the
// warp, are read four per lane at a time (each lane finds the row of an entry by a binary search
// over the lanes' first entry numbers). Called by a whole warp.
__device__ __forceinline__ void row_index_pass32(const DevSeqCol* __restrict__ cs, const uint32_t* __restrict__ F,
                                                 uint32_t w, uint32_t words, uint32_t* counts, uint32_t* scratch,
                                                 uint32_t* list) {
   const uint32_t lane = threadIdx.x & 31;
   const uint32_t L = cs->L, nseg = mut_nseg(L);
   uint32_t x = w + lane < words ? __ldg(F + w + lane) : 0u;
   const uint32_t c = __popc(x);
   uint32_t incl = c;
#pragma unroll
   for (uint32_t o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
      if (lane >= o) incl += y;
   }
   const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
   if (total == 0) return;
   uint32_t at = incl - c;
   while (x) {
      list[at++] = 32 * (w + lane) + (__ffs(x) - 1);
      x &= x - 1;
   }
   __syncwarp();
   uint32_t* start_hist = scratch;
   uint32_t* end_hist = scratch + (L + 1);
   uint32_t* ndiff = scratch + 2 * (L + 1);
   uint32_t* seg_s = scratch + 3 * (L + 1);
   uint32_t* seg_e = seg_s + nseg;
   uint32_t* seg_n = seg_e + nseg;
   for (uint32_t r0 = 0; r0 < total; r0 += 32) {
      const uint32_t j = r0 + lane;
      uint32_t b = 0, n = 0;
      if (j < total) {
         const uint32_t r = list[j];
         b = __ldg(cs->hrow_off + r);
         n = __ldg(cs->hrow_off + r + 1) - b;
      }
      uint32_t first = n;  // exclusive prefix of the entry counts after the scan
#pragma unroll
      for (uint32_t o = 1; o < 32; o <<= 1) {
         const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, first, o);
         if (lane >= o) first += y;
      }
      const uint32_t E = __shfl_sync(0xFFFFFFFFu, first, 31);
      first -= n;
      constexpr uint32_t U = 4;
      for (uint32_t k0 = 0; k0 < E; k0 += 32 * U) {
         uint32_t ent[U];
#pragma unroll
         for (uint32_t u = 0; u < U; ++u) {
            const uint32_t k = k0 + 32 * u + lane;
            // the last lane whose first entry number is <= k holds entry k
            uint32_t lo = 0;
#pragma unroll
            for (uint32_t step = 16; step > 0; step >>= 1) {
               const uint32_t f = __shfl_sync(0xFFFFFFFFu, first, lo + step);
               if (f <= k) lo += step;
            }
            const uint32_t bl = __shfl_sync(0xFFFFFFFFu, b, lo), fl = __shfl_sync(0xFFFFFFFFu, first, lo);
            ent[u] = k < E ? __ldg(cs->hent + bl + (k - fl)) : 0xFFFFFFFFu;
         }
#pragma unroll
         for (uint32_t u = 0; u < U; ++u) {
            if (ent[u] == 0xFFFFFFFFu) continue;
            const uint32_t code = ent[u] & 31u, pos = ent[u] >> 5;
            if (code < ROW_COV_START) {
               atomicAdd(counts + static_cast<size_t>(code) * L + pos, 1u);
            } else if (code == ROW_COV_START) {
               atomicAdd(start_hist + pos, 1u);
               atomicAdd(seg_s + pos / MUT_SEG, 1u);
            } else if (code == ROW_COV_END) {
               atomicAdd(end_hist + pos, 1u);
               atomicAdd(seg_e + pos / MUT_SEG, 1u);
            } else {
               const uint32_t d = code == ROW_MISS_START ? 1u : 0xFFFFFFFFu;
               atomicAdd(ndiff + pos, d);
               atomicAdd(seg_n + pos / MUT_SEG, d);
            }
         }
      }
   }
   __syncwarp();
}

}  // namespace rhygpu
