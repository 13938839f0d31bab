// Mutations action kernels of the plain single-query path.
//
//  mut_ctr_kernel    every vertical container once: |F ∩ container| against the filter tile of its
//                    chunk staged in shared memory; integer counts per (symbol, position)
//                    (reference: mutations_node.cpp:139-189). Payloads are read with 16-byte loads.
//  mut_cov_kernel    rows of F outside their covered region (per-chunk exception lists) and inside
//                    missing intervals (per 128-position block) as difference arrays
//                    (reference: mutations_node.cpp:51-136).
//  mut_final_kernel  prefix sums and the local-reference count per position
//                    (reference: mutations_node.cpp:192-203).
// The filter count decides on the device between the full path (|F| == rows: stored
// cardinalities, reference: mutations_node.cpp:240-266), the empty path and the mixed path.
#include <cuda_runtime.h>

#include "device.h"
#include "mutations_common.cuh"

namespace rhygpu {

namespace {

constexpr uint32_t MT = 256;
constexpr uint32_t NSPLIT = 4;  // CTAs per missing-interval block

// Warp-cooperative |F ∩ container| (all lanes return the total).
__device__ uint32_t warp_count(const CtrDesc& d, const uint32_t* F, const uint16_t* __restrict__ payload) {
   const uint32_t lane = threadIdx.x & 31;
   uint32_t c = 0;
   if (d.type == CT_ARRAY) {
      const uint32_t s = d.payload, e = s + d.card_m1 + 1u;
      const uint4* pw = reinterpret_cast<const uint4*>(payload);
      const uint32_t w0 = s >> 3, w1 = (e - 1) >> 3;
#pragma unroll 2
      for (uint32_t w = w0 + lane; w <= w1; w += 32) {
         const uint4 x = __ldg(pw + w);
#pragma unroll
         for (uint32_t t = 0; t < 8; ++t) {
            const uint32_t j = 8 * w + t;
            if (j >= s && j < e) c += test_bit(F, u16_of(x, t));
         }
      }
   } else if (d.type == CT_BITSET) {
      const uint4* b = reinterpret_cast<const uint4*>(payload + d.payload);
      const uint4* f = reinterpret_cast<const uint4*>(F);
#pragma unroll 4
      for (uint32_t k = lane; k < CHUNK_WORDS / 4; k += 32) {
         const uint4 x = __ldg(b + k);
         const uint4 y = f[k];
         c += __popc(x.x & y.x) + __popc(x.y & y.y) + __popc(x.z & y.z) + __popc(x.w & y.w);
      }
   } else {
      const uint16_t* p = payload + d.payload;
      for (uint32_t k = lane; k < d.nruns; k += 32) {
         const uint32_t s = __ldg(p + 2 * k);
         c += count_range(F, s, s + __ldg(p + 2 * k + 1) + 1u);
      }
   }
   return __reduce_add_sync(0xFFFFFFFFu, c);
}

__global__ void __launch_bounds__(MT) mut_ctr_kernel(const DevTable* __restrict__ tab, uint32_t col,
                                                     const MutPart* __restrict__ parts, uint32_t nparts,
                                                     const uint32_t* __restrict__ filter,
                                                     const unsigned long long* __restrict__ fcount, uint32_t* counts) {
   __shared__ __align__(16) uint32_t F[CHUNK_WORDS];
   const unsigned long long fc = *fcount;
   if (fc == 0) return;
   const bool full = fc == tab->n_rows;
   const DevSeqCol* cs = &tab->seq[col];
   const CtrDesc* __restrict__ ctrs = cs->ctrs;
   const uint16_t* __restrict__ payload = cs->payload;
   const uint32_t L = cs->L;
   const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
   for (uint32_t pi = blockIdx.x; pi < nparts; pi += gridDim.x) {
      const MutPart P = parts[pi];
      if (!full) {
         const uint4* src = reinterpret_cast<const uint4*>(filter + static_cast<size_t>(P.v) * CHUNK_WORDS);
         uint4* dst = reinterpret_cast<uint4*>(F);
         for (uint32_t k = threadIdx.x; k < CHUNK_WORDS / 4; k += blockDim.x) dst[k] = __ldg(src + k);
      }
      __syncthreads();
      for (uint32_t base = P.begin + warp * 32; base < P.end; base += nw * 32) {
         const uint32_t idx = base + lane;
         const bool valid = idx < P.end;
         uint4 raw = make_uint4(0, 0, 0, 0);
         if (valid) raw = __ldg(reinterpret_cast<const uint4*>(ctrs) + idx);
         const CtrDesc d = *reinterpret_cast<const CtrDesc*>(&raw);
         uint32_t cnt = 0;
         bool big = false;
         if (valid) {
            if (full) {
               cnt = d.card_m1 + 1u;
            } else if (d.type == CT_ARRAY && d.card_m1 < SMALL_ARRAY) {
               cnt = small_array_count(d, payload, F);
            } else {
               big = true;
            }
         }
         if (valid && !big && cnt) atomicAdd(&counts[static_cast<size_t>(d.sym) * L + d.key], cnt);
         uint32_t bigmask = __ballot_sync(0xFFFFFFFFu, big);
         while (bigmask) {
            const int j = __ffs(bigmask) - 1;
            bigmask &= bigmask - 1;
            const CtrDesc dj = shfl_desc(raw, j);
            const uint32_t c = warp_count(dj, F, payload);
            if (lane == 0 && c) atomicAdd(&counts[static_cast<size_t>(dj.sym) * L + dj.key], c);
         }
      }
      __syncthreads();
   }
}

__global__ void __launch_bounds__(MT) mut_cov_kernel(const DevTable* __restrict__ tab, uint32_t col,
                                                     const uint32_t* __restrict__ filter,
                                                     const unsigned long long* __restrict__ fcount, uint32_t* scratch) {
   const unsigned long long fc = *fcount;
   if (fc == 0) return;
   const bool full = fc == tab->n_rows;
   const DevSeqCol* cs = &tab->seq[col];
   const uint32_t L = cs->L, nchunks = tab->nchunks, nseg = mut_nseg(L);
   uint32_t* start_hist = scratch;
   uint32_t* end_hist = scratch + (L + 1);
   uint32_t* ndiff = scratch + 2 * (L + 1);
   uint32_t* seg_s = scratch + 3 * (L + 1);
   uint32_t* seg_e = seg_s + nseg;
   uint32_t* seg_n = seg_e + nseg;
   if (blockIdx.x < cs->nblocks * NSPLIT) {
      __shared__ int diff[NBLOCK + 1];
      __shared__ int red[2][MT / 32];
      const uint32_t b = blockIdx.x / NSPLIT, part = blockIdx.x % NSPLIT;
      for (uint32_t i = threadIdx.x; i <= NBLOCK; i += blockDim.x) diff[i] = 0;
      __syncthreads();
      // the buckets of every chunk of block b are contiguous; entries carry global row ids
      const uint32_t nb = __ldg(cs->nblk_off + static_cast<size_t>(b) * nchunks);
      const uint32_t ne = __ldg(cs->nblk_off + static_cast<size_t>(b + 1) * nchunks);
      const uint32_t per = (ne - nb + NSPLIT - 1) / NSPLIT;
      const uint32_t lo_i = nb + part * per, hi_i = min(ne, lo_i + per);
      int at_start = 0, at_end = 0;  // intervals starting at the block start / ending at the block end
      for (uint32_t i = lo_i + threadIdx.x; i < hi_i; i += blockDim.x) {
         const uint2 raw = __ldg(reinterpret_cast<const uint2*>(cs->nblk) + i);
         if (full || ((__ldg(filter + (raw.x >> 5)) >> (raw.x & 31)) & 1u)) {
            const uint32_t lo = raw.y & 0xFFFFu, hi = raw.y >> 16;
            if (lo == 0) ++at_start;
            else atomicAdd(&diff[lo], 1);
            if (hi == NBLOCK) ++at_end;
            else atomicSub(&diff[hi], 1);
         }
      }
      at_start = __reduce_add_sync(0xFFFFFFFFu, at_start);
      at_end = __reduce_add_sync(0xFFFFFFFFu, at_end);
      if ((threadIdx.x & 31) == 0) {
         red[0][threadIdx.x >> 5] = at_start;
         red[1][threadIdx.x >> 5] = at_end;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
         int a = 0, e = 0;
         for (uint32_t w = 0; w < MT / 32; ++w) {
            a += red[0][w];
            e += red[1][w];
         }
         diff[0] += a;
         diff[NBLOCK] -= e;
      }
      __syncthreads();
      for (uint32_t q = threadIdx.x; q <= NBLOCK; q += blockDim.x) {
         const int x = diff[q];
         const uint32_t p = b * NBLOCK + q;
         if (x != 0 && p <= L) {
            atomicAdd(&ndiff[p], static_cast<uint32_t>(x));
            atomicAdd(&seg_n[p / MUT_SEG], static_cast<uint32_t>(x));
         }
      }
   } else {
      const uint32_t v = blockIdx.x - cs->nblocks * NSPLIT;
      if (v >= nchunks) return;
      const uint32_t xb = __ldg(cs->exc_off + v), xe = __ldg(cs->exc_off + v + 1);
      const uint32_t* Fv = filter + static_cast<size_t>(v) * CHUNK_WORDS;
      for (uint32_t i = xb + threadIdx.x; i < xe; i += blockDim.x) {
         const uint4 raw = __ldg(reinterpret_cast<const uint4*>(cs->exc) + i);
         if (full || ((__ldg(Fv + (raw.x >> 5)) >> (raw.x & 31)) & 1u)) {
            atomicAdd(&start_hist[raw.y], 1u);
            atomicAdd(&seg_s[raw.y / MUT_SEG], 1u);
            atomicAdd(&end_hist[raw.z], 1u);
            atomicAdd(&seg_e[raw.z / MUT_SEG], 1u);
         }
      }
   }
}

__global__ void __launch_bounds__(MUT_SEG) mut_final_kernel(const DevTable* __restrict__ tab, uint32_t col,
                                                            const unsigned long long* __restrict__ fcount,
                                                            uint32_t* counts, const uint32_t* __restrict__ scratch) {
   __shared__ uint32_t red[MUT_SEG / 32];
   const DevSeqCol* cs = &tab->seq[col];
   final_position_counts(cs, static_cast<uint32_t>(*fcount), counts, scratch, red);
}

}  // namespace

void launch_mutations(const DevTable* d_table, const DevSeqCol& col_host, uint32_t col, uint32_t nchunks,
                      const MutPart* d_parts, uint32_t nparts, const uint32_t* d_filter,
                      const unsigned long long* d_filter_count, uint32_t* d_counts, uint32_t* d_scratch, void* stream,
                      uint32_t parts) {
   cudaStream_t s = static_cast<cudaStream_t>(stream);
   if (nparts > 0 && (parts & MUT_PART_CTR)) {
      const uint32_t grid = nparts < 152u * 8u ? nparts : 152u * 8u;
      mut_ctr_kernel<<<grid, MT, 0, s>>>(d_table, col, d_parts, nparts, d_filter, d_filter_count, d_counts);
   }
   if (parts & MUT_PART_COV)
      mut_cov_kernel<<<col_host.nblocks * NSPLIT + nchunks, MT, 0, s>>>(d_table, col, d_filter, d_filter_count, d_scratch);
   if (parts & MUT_PART_FINAL)
      mut_final_kernel<<<(col_host.L + MUT_SEG - 1) / MUT_SEG, MUT_SEG, 0, s>>>(d_table, col, d_filter_count, d_counts,
                                                                               d_scratch);
}

}  // namespace rhygpu
