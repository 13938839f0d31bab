// Mutations action kernels of the plain single-query path.
//
//  mut_ctr_kernel    every vertical container once: |F ∩ container| against the filter tile of its
//                    chunk staged in shared memory; integer counts per (symbol, position)
//                    (reference: mutations_node.cpp:139-189). CTAs stay on one chunk; a warp takes
//                    32 consecutive containers and streams their array payloads as one contiguous
//                    range with 16-byte loads, attributing elements to containers by offset.
//  mut_cov_kernel    rows of F outside their covered region and inside missing intervals, from
//                    position-sorted start / end events aggregated per position with warp ballots
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
constexpr uint32_t NW = MT / 32;
constexpr uint32_t CTAS_PER_CHUNK_TARGET = 1216;  // 152 SMs x 8 CTAs, divided among the chunks

// Warp-cooperative |F ∩ container| for bitset and run containers (all lanes return the total).
__device__ uint32_t warp_count_other(const CtrDesc& d, const uint32_t* F, const uint16_t* __restrict__ payload) {
   const uint32_t lane = threadIdx.x & 31;
   uint32_t c = 0;
   if (d.type == CT_BITSET) {
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

__global__ void __launch_bounds__(MT) mut_ctr_kernel(const DevTable* __restrict__ tab, uint32_t col, uint32_t K,
                                                     const uint32_t* __restrict__ filter,
                                                     const unsigned long long* __restrict__ fcount, uint32_t* counts) {
   __shared__ __align__(16) uint32_t F[CHUNK_WORDS];
   const unsigned long long fc = *fcount;
   if (fc == 0) return;
   const bool full = fc == tab->n_rows;
   const DevSeqCol* cs = &tab->seq[col];
   const CtrDesc* __restrict__ ctrs = cs->ctrs;
   const uint16_t* __restrict__ payload = cs->payload;
   const uint4* __restrict__ pw = reinterpret_cast<const uint4*>(payload);
   const uint32_t L = cs->L;
   const uint32_t v = blockIdx.x / K, k = blockIdx.x % K;
   const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
   if (!full) {
      const uint4* src = reinterpret_cast<const uint4*>(filter + static_cast<size_t>(v) * CHUNK_WORDS);
      uint4* dst = reinterpret_cast<uint4*>(F);
      for (uint32_t i = threadIdx.x; i < CHUNK_WORDS / 4; i += blockDim.x) dst[i] = __ldg(src + i);
   }
   __syncthreads();
   const uint32_t cb = __ldg(cs->off + static_cast<size_t>(v) * L), ce = __ldg(cs->off + static_cast<size_t>(v + 1) * L);
   const uint32_t nslices = (ce - cb + 31) / 32;
   for (uint32_t sl = k * NW + warp; sl < nslices; sl += K * NW) {
      const uint32_t idx = cb + sl * 32 + lane;
      const bool valid = idx < ce;
      uint4 raw = make_uint4(0, 0, 0, 0);
      if (valid) raw = __ldg(reinterpret_cast<const uint4*>(ctrs) + idx);
      const CtrDesc d = *reinterpret_cast<const CtrDesc*>(&raw);
      if (full) {
         if (valid) atomicAdd(&counts[static_cast<size_t>(d.sym) * L + d.key], d.card_m1 + 1u);
         continue;
      }
      const bool is_arr = valid && d.type == CT_ARRAY;
      const uint32_t amask = __ballot_sync(0xFFFFFFFFu, is_arr);
      const uint32_t nA = __popc(amask);
      if (nA) {
         // Lane c takes the c-th array of the slice; the arrays are back to back in the payload
         // arena, so the slice's elements are one range [P0, P1) streamed in windows of 32 words.
         const uint32_t src = lane < nA ? __fns(amask, 0, lane + 1) : 0;
         const uint32_t my_s = __shfl_sync(0xFFFFFFFFu, d.payload, src);
         const uint32_t my_e = my_s + __shfl_sync(0xFFFFFFFFu, static_cast<uint32_t>(d.card_m1), src) + 1u;
         const uint32_t P0 = __shfl_sync(0xFFFFFFFFu, my_s, 0);
         const uint32_t P1 = __shfl_sync(0xFFFFFFFFu, my_e, nA - 1);
         uint32_t acc = 0;
         for (uint32_t w0 = P0 >> 3; w0 <= (P1 - 1) >> 3; w0 += 32) {
            const uint32_t w = w0 + lane;
            uint32_t bits = 0;  // bit t: element 8w + t is in F
            if (w <= (P1 - 1) >> 3) {
               const uint4 x = __ldg(pw + w);
#pragma unroll
               for (uint32_t t = 0; t < 8; ++t) bits |= test_bit(F, u16_of(x, t)) << t;
            }
            // exclusive prefix of set bits over the window's words
            const uint32_t cnt = __popc(bits);
            uint32_t incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
               const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
               if (static_cast<int>(lane) >= o) incl += y;
            }
            const uint32_t excl = incl - cnt;
            const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
            // set bits of [8 w0, x) for x inside or at the end of the window
            const uint32_t lo8 = 8 * w0, hi8 = 8 * (w0 + 32);
            const uint32_t a = min(max(my_s, lo8), hi8), z = min(max(my_e, lo8), hi8);
            const uint32_t wa = (a - lo8) >> 3, wz = (z - lo8) >> 3;
            const uint32_t ea = __shfl_sync(0xFFFFFFFFu, excl, wa & 31), ba = __shfl_sync(0xFFFFFFFFu, bits, wa & 31);
            const uint32_t ez = __shfl_sync(0xFFFFFFFFu, excl, wz & 31), bz = __shfl_sync(0xFFFFFFFFu, bits, wz & 31);
            const uint32_t pa = wa >= 32 ? total : ea + __popc(ba & ((1u << ((a - lo8) & 7)) - 1u));
            const uint32_t pz = wz >= 32 ? total : ez + __popc(bz & ((1u << ((z - lo8) & 7)) - 1u));
            acc += pz - pa;
         }
         const uint32_t key = __shfl_sync(0xFFFFFFFFu, d.key, src);
         const uint32_t sym = __shfl_sync(0xFFFFFFFFu, static_cast<uint32_t>(d.sym), src);
         if (lane < nA && acc) atomicAdd(&counts[static_cast<size_t>(sym) * L + key], acc);
      }
      uint32_t other = __ballot_sync(0xFFFFFFFFu, valid && !is_arr);
      while (other) {
         const int j = __ffs(other) - 1;
         other &= other - 1;
         const CtrDesc dj = shfl_desc(raw, j);
         const uint32_t c = warp_count_other(dj, F, payload);
         if (lane == 0 && c) atomicAdd(&counts[static_cast<size_t>(dj.sym) * L + dj.key], c);
      }
   }
}

// One CTA per event item. Missing events add +1 (start) / -1 (end) at their position; coverage
// events count rows whose covered region starts (ends) there.
__global__ void __launch_bounds__(MT) mut_cov_kernel(const DevTable* __restrict__ tab, uint32_t col,
                                                     const EvItem* __restrict__ items,
                                                     const uint32_t* __restrict__ filter,
                                                     const unsigned long long* __restrict__ fcount, uint32_t* scratch) {
   __shared__ int cnt[NBLOCK + 1];
   const unsigned long long fc = *fcount;
   if (fc == 0) return;
   const bool full = fc == tab->n_rows;
   const DevSeqCol* cs = &tab->seq[col];
   const uint32_t L = cs->L, nseg = mut_nseg(L);
   uint32_t* start_hist = scratch;
   uint32_t* end_hist = scratch + (L + 1);
   uint32_t* ndiff = scratch + 2 * (L + 1);
   uint32_t* seg_s = scratch + 3 * (L + 1);
   uint32_t* seg_e = seg_s + nseg;
   uint32_t* seg_n = seg_e + nseg;
   const EvItem it = items[blockIdx.x];
   const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
   if (it.list <= EV_MEND) {
      for (uint32_t i = threadIdx.x; i <= NBLOCK; i += blockDim.x) cnt[i] = 0;
      __syncthreads();
      const uint32_t* ev = it.list == EV_MSTART ? cs->mstart : cs->mend;
      constexpr uint32_t U = 4;  // events per lane in flight
      for (uint32_t base = it.begin + warp * 32 * U; base < it.end; base += blockDim.x * U) {
         uint32_t e[U], bit[U];
#pragma unroll
         for (uint32_t k = 0; k < U; ++k) {
            const uint32_t i = base + 32 * k + lane;
            e[k] = i < it.end ? __ldg(ev + i) : 0xFFFFFFFFu;
         }
#pragma unroll
         for (uint32_t k = 0; k < U; ++k) {
            const uint32_t row = e[k] >> 8;
            bit[k] = (e[k] != 0xFFFFFFFFu && (full || ((__ldg(filter + (row >> 5)) >> (row & 31)) & 1u))) ? 1u : 0u;
         }
#pragma unroll
         for (uint32_t k = 0; k < U; ++k) {
            const bool active = e[k] != 0xFFFFFFFFu;
            const uint32_t pos = e[k] & 0xFFu;
            const uint32_t amask = __ballot_sync(0xFFFFFFFFu, active);
            const uint32_t bits = __ballot_sync(0xFFFFFFFFu, bit[k]);
            // lanes with equal positions form one group (events are sorted by position)
            const uint32_t grp = __match_any_sync(0xFFFFFFFFu, active ? pos : 0xFFFFu) & amask;
            if (active && lane == static_cast<uint32_t>(__ffs(grp) - 1)) {
               const uint32_t n = __popc(bits & grp);
               if (n) atomicAdd(&cnt[pos], static_cast<int>(n));
            }
         }
      }
      __syncthreads();
      const int sign = it.list == EV_MSTART ? 1 : -1;
      for (uint32_t q = threadIdx.x; q <= NBLOCK; q += blockDim.x) {
         const int x = cnt[q];
         const uint32_t p = it.block * NBLOCK + q;
         if (x != 0 && p <= L) {
            atomicAdd(&ndiff[p], static_cast<uint32_t>(sign * x));
            atomicAdd(&seg_n[p / MUT_SEG], static_cast<uint32_t>(sign * x));
         }
      }
   } else {
      const CovEvent* ev = it.list == EV_CSTART ? cs->cstart : cs->cend;
      uint32_t* hist = it.list == EV_CSTART ? start_hist : end_hist;
      uint32_t* seg = it.list == EV_CSTART ? seg_s : seg_e;
      for (uint32_t i = it.begin + threadIdx.x; i < it.end; i += blockDim.x) {
         const uint2 e = __ldg(reinterpret_cast<const uint2*>(ev) + i);
         if (full || ((__ldg(filter + (e.x >> 5)) >> (e.x & 31)) & 1u)) {
            atomicAdd(&hist[e.y], 1u);
            atomicAdd(&seg[e.y / MUT_SEG], 1u);
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
                      const EvItem* d_ev, uint32_t n_ev, const uint32_t* d_filter,
                      const unsigned long long* d_filter_count, uint32_t* d_counts, uint32_t* d_scratch, void* stream,
                      uint32_t parts) {
   cudaStream_t s = static_cast<cudaStream_t>(stream);
   if (parts & MUT_PART_CTR) {
      const uint32_t K = (CTAS_PER_CHUNK_TARGET + nchunks - 1) / nchunks;
      mut_ctr_kernel<<<nchunks * K, MT, 0, s>>>(d_table, col, K, d_filter, d_filter_count, d_counts);
   }
   if ((parts & MUT_PART_COV) && n_ev > 0)
      mut_cov_kernel<<<n_ev, MT, 0, s>>>(d_table, col, d_ev, d_filter, d_filter_count, d_scratch);
   if (parts & MUT_PART_FINAL)
      mut_final_kernel<<<(col_host.L + MUT_SEG - 1) / MUT_SEG, MUT_SEG, 0, s>>>(d_table, col, d_filter_count, d_counts,
                                                                               d_scratch);
}

}  // namespace rhygpu
