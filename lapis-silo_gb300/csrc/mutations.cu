// Mutations action kernels of the plain single-query path.
//
//  mut_chunk_kernel  every vertical container once: |F ∩ container| against the filter tile of its
//                    chunk staged in shared memory; integer counts per (symbol, position)
//                    (reference: mutations_node.cpp:139-189). Warps stream units of at most WU
//                    array elements (or one bitset / run container) into registers.
//  mut_cov_kernel    rows of F outside their covered region and inside missing intervals, from
//                    position-sorted start / end events aggregated per position with warp ballots
//                    (reference: mutations_node.cpp:51-136).
//  mut_final_kernel  prefix sums and the local-reference count per position
//                    (reference: mutations_node.cpp:192-203).
//  mut_sparse_kernel filters of few rows: each row of F adds its row-index entries, the same counts
//                    the two passes above add for it (the reference's mixed path walks the filtered
//                    rows for coverage the same way, mutations_node.cpp:111-136).
// The filter count decides on the device between the full path (|F| == rows: stored
// cardinalities, reference: mutations_node.cpp:240-266), the empty path and the mixed path.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <stdexcept>
#include <string>

#include "device.h"
#include "mutations_common.cuh"

namespace rhygpu {

namespace {

constexpr uint32_t MT = 256;
constexpr uint32_t NW = MT / 32;
constexpr uint32_t WU_VEC = WU / 8;         // uint4 of payload per array unit
constexpr uint32_t WU_GROUPS = WU_VEC / 32;  // groups of 32 uint4 (one per lane) per array unit
constexpr uint32_t TASK_UNITS = 128;         // units of a task staged in shared memory (the rest read from global)

// Container pass of the Mutations action (reference: mutations_node.cpp:139-190, full path
// :240-266). One CTA per task: a range of units of one chunk (host-built, ChunkTask). The CTA
// stages the chunk's filter tile and the task's unit records in shared memory once; then every warp
// claims units of the range from a shared counter and counts them on its own, with no further CTA
// barrier:
//   SU_ARRAYS  up to WU elements of the chunk's array payloads (arrays lie back to back in
//              descriptor order), read by 16-byte loads straight into registers, lane l holding
//              uint4 l + 32 g of group g, with the unit's first 32 descriptors loaded beside
//              them. Each element (a row of the chunk) is tested against the
//              tile; a warp prefix sum over the lanes' membership counts gives every container its
//              |F ∩ c| as the difference of two prefix values (a container cut by a unit boundary
//              adds two partial counts).
//   SU_BITSET  one bitset: AND with the tile and popcount, 16 uint4 per lane.
//   SU_RUN     one run container: the tile's popcount over each run.
// Full filters (|F| == rows) add the stored cardinalities and read no payload.
__global__ void __launch_bounds__(MT, 6) mut_chunk_kernel(const DevTable* __restrict__ tab, uint32_t col,
                                                       const uint32_t* __restrict__ filter,
                                                       const unsigned long long* __restrict__ fcount,
                                                       unsigned long long sparse_max, uint32_t* counts) {
   __shared__ __align__(16) uint32_t F[CHUNK_WORDS];
   __shared__ __align__(16) StreamUnit su[TASK_UNITS];
   __shared__ uint32_t next_unit;
   __shared__ uint16_t pre[NW][WU_GROUPS][32];  // per warp: lane's exclusive prefix within a group
   __shared__ uint8_t msk[NW][WU_GROUPS][32];   // per warp: lane's 8 membership bits within a group
   __shared__ uint32_t gpre[NW][WU_GROUPS + 1]; // per warp: exclusive prefix of the groups, then the total
   const unsigned long long fc = *fcount;
   if (fc == 0 || fc <= sparse_max) return;  // empty, or counted by the row-index pass
   const bool full = fc == tab->n_rows;
   const DevSeqCol* cs = &tab->seq[col];
   const ChunkTask task = cs->tasks[blockIdx.x];
   const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, L = cs->L;
   if (!full) {
      const uint4* src = reinterpret_cast<const uint4*>(filter + static_cast<size_t>(task.v) * CHUNK_WORDS);
      for (uint32_t i = tid; i < CHUNK_WORDS / 4; i += MT) reinterpret_cast<uint4*>(F)[i] = __ldg(src + i);
   }
   const StreamUnit* __restrict__ units = cs->su;
   for (uint32_t i = tid; i < task.u1 - task.u0 && i < TASK_UNITS; i += MT) su[i] = units[task.u0 + i];
   if (tid == 0) next_unit = task.u0;
   __syncthreads();
   const CtrDesc* __restrict__ ctrs = cs->ctrs;
   const uint4* __restrict__ pay4 = reinterpret_cast<const uint4*>(cs->payload);
   for (;;) {
      uint32_t u = 0;
      if (lane == 0) u = atomicAdd(&next_unit, 1u);
      u = __shfl_sync(0xFFFFFFFFu, u, 0);
      if (u >= task.u1) break;
      const StreamUnit U = u - task.u0 < TASK_UNITS ? su[u - task.u0] : units[u];
      if (U.kind == SU_ARRAYS) {
         if (full) {
            for (uint32_t c = U.c0 + lane; c < U.c1; c += 32) {
               const uint4 raw = __ldg(reinterpret_cast<const uint4*>(ctrs) + c);
               const CtrDesc d = *reinterpret_cast<const CtrDesc*>(&raw);
               if (d.type != CT_ARRAY) continue;
               const uint32_t s = max(d.payload, U.e0), e = min(d.payload + d.card_m1 + 1u, U.e1);
               if (s < e) atomicAdd(&counts[static_cast<size_t>(d.sym) * L + d.key], e - s);
            }
            continue;
         }
         const uint32_t n = U.e1 - U.e0;  // U.e0 is a multiple of 8 (16-byte aligned), n <= WU
         uint4 x[WU_GROUPS];
#pragma unroll
         for (uint32_t g = 0; g < WU_GROUPS; ++g) {
            const uint32_t i = 32 * g + lane;
            x[g] = 8 * i < n ? __ldg(pay4 + U.e0 / 8 + i) : make_uint4(0, 0, 0, 0);
         }
         // the unit's first 32 descriptors, loaded beside the payload (one round trip for both)
         const uint4 d0 = U.c0 + lane < U.c1 ? __ldg(reinterpret_cast<const uint4*>(ctrs) + U.c0 + lane)
                                             : make_uint4(0, 0, 0, 0);
         uint32_t run = 0;  // members in the groups before g (the same in every lane)
#pragma unroll
         for (uint32_t g = 0; g < WU_GROUPS; ++g) {
            const uint32_t i = 32 * g + lane;
            uint32_t m = 0;
#pragma unroll
            for (uint32_t t = 0; t < 8; ++t) {
               const uint32_t r = u16_of(x[g], t);
               m |= ((F[r >> 5] >> (r & 31)) & 1u) << t;
            }
            if (8 * i + 8 > n) m &= 8 * i < n ? (1u << (n - 8 * i)) - 1u : 0u;  // past the unit's end
            const uint32_t c = __popc(m);
            uint32_t incl = c;
#pragma unroll
            for (uint32_t o = 1; o < 32; o <<= 1) {
               const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
               if (lane >= o) incl += y;
            }
            pre[warp][g][lane] = static_cast<uint16_t>(incl - c);
            msk[warp][g][lane] = static_cast<uint8_t>(m);
            if (lane == 0) gpre[warp][g] = run;
            run += __shfl_sync(0xFFFFFFFFu, incl, 31);
         }
         if (lane == 0) gpre[warp][WU_GROUPS] = run;
         __syncwarp();
         auto prefix = [&](uint32_t i) -> uint32_t {  // members among the unit's elements [0, i)
            if (i >= WU) return gpre[warp][WU_GROUPS];
            const uint32_t g = i / 256, k = (i / 8) % 32, t = i % 8;
            return gpre[warp][g] + pre[warp][g][k] + __popc(msk[warp][g][k] & ((1u << t) - 1u));
         };
         for (uint32_t c = U.c0 + lane; c < U.c1; c += 32) {
            const uint4 raw = c - U.c0 < 32 ? d0 : __ldg(reinterpret_cast<const uint4*>(ctrs) + c);
            const CtrDesc d = *reinterpret_cast<const CtrDesc*>(&raw);
            if (d.type != CT_ARRAY) continue;
            const uint32_t s = max(d.payload, U.e0), e = min(d.payload + d.card_m1 + 1u, U.e1);
            if (s >= e) continue;
            const uint32_t k = prefix(e - U.e0) - prefix(s - U.e0);
            if (k) atomicAdd(&counts[static_cast<size_t>(d.sym) * L + d.key], k);
         }
         __syncwarp();  // the prefix arrays are rewritten by the warp's next unit
      } else {
         const uint4 raw = __ldg(reinterpret_cast<const uint4*>(ctrs) + U.c0);
         const CtrDesc d = *reinterpret_cast<const CtrDesc*>(&raw);
         uint32_t k = 0;
         if (full) {
            k = lane == 0 ? d.card_m1 + 1u : 0u;
         } else if (U.kind == SU_BITSET) {
            const uint4* f4 = reinterpret_cast<const uint4*>(F);
            constexpr uint32_t BV = CHUNK_WORDS / 4 / 32, BB = 4;  // uint4 per lane; loads in flight
#pragma unroll
            for (uint32_t j0 = 0; j0 < BV; j0 += BB) {
               uint4 a[BB];
#pragma unroll
               for (uint32_t j = 0; j < BB; ++j) a[j] = __ldg(pay4 + U.e0 / 8 + lane + 32 * (j0 + j));
#pragma unroll
               for (uint32_t j = 0; j < BB; ++j) {
                  const uint4 y = f4[lane + 32 * (j0 + j)];
                  k += __popc(a[j].x & y.x) + __popc(a[j].y & y.y) + __popc(a[j].z & y.z) + __popc(a[j].w & y.w);
               }
            }
         } else {
            const uint16_t* r = cs->payload + d.payload;
            for (uint32_t i = lane; i < d.nruns; i += 32) {
               const uint32_t s = __ldg(r + 2 * i);
               k += count_range(F, s, s + __ldg(r + 2 * i + 1) + 1u);
            }
         }
         k = __reduce_add_sync(0xFFFFFFFFu, k);
         if (lane == 0 && k) atomicAdd(&counts[static_cast<size_t>(d.sym) * L + d.key], k);
      }
   }
}

// One CTA per event item. Missing events add +1 (start) / -1 (end) at their position; coverage
// events count rows whose covered region starts (ends) there.
__global__ void __launch_bounds__(MT) mut_cov_kernel(const DevTable* __restrict__ tab, uint32_t col,
                                                     const EvItem* __restrict__ items,
                                                     const uint32_t* __restrict__ filter,
                                                     const unsigned long long* __restrict__ fcount,
                                                     unsigned long long sparse_max, uint32_t* scratch) {
   __shared__ int cnt[NBLOCK + 1];
   const unsigned long long fc = *fcount;
   if (fc == 0 || fc <= sparse_max) return;  // empty, or counted by the row-index pass
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

// Filters of 1..sparse_max rows: one warp per 32 filter words at a time.
__global__ void __launch_bounds__(MT) mut_sparse_kernel(const DevTable* __restrict__ tab, uint32_t col,
                                                        const uint32_t* __restrict__ filter,
                                                        const unsigned long long* __restrict__ fcount,
                                                        unsigned long long sparse_max, uint32_t* counts,
                                                        uint32_t* scratch) {
   __shared__ uint32_t list[NW][1024];
   const unsigned long long fc = *fcount;
   if (fc == 0 || fc > sparse_max) return;
   const DevSeqCol* cs = &tab->seq[col];
   const uint32_t words = tab->nchunks * CHUNK_WORDS;
   const uint32_t warp = threadIdx.x >> 5, nwarps = gridDim.x * NW;
   for (uint32_t w = (blockIdx.x * NW + warp) * 32; w < words; w += nwarps * 32)
      row_index_pass32(cs, filter, w, words, counts, scratch, list[warp]);
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
                      const unsigned long long* d_filter_count, uint32_t* d_counts, uint32_t* d_scratch, int* d_err,
                      void* stream, uint32_t parts, uint64_t sparse_max) {
   (void)d_err;  // no kernel of this pass waits on anything: none reports a device error
   cudaStream_t s = static_cast<cudaStream_t>(stream);
   if (!(parts & MUT_PART_SPARSE)) sparse_max = 0;  // the dense passes count every filter
   if (sparse_max) {
      const uint32_t groups = nchunks * CHUNK_WORDS / 32;  // 32-word groups, one per warp and step
      mut_sparse_kernel<<<std::max(1u, std::min(groups / NW, 2048u)), MT, 0, s>>>(
         d_table, col, d_filter, d_filter_count, static_cast<unsigned long long>(sparse_max), d_counts, d_scratch);
   }
   if ((parts & MUT_PART_CTR) && col_host.ntasks > 0)
      mut_chunk_kernel<<<col_host.ntasks, MT, 0, s>>>(d_table, col, d_filter, d_filter_count,
                                                      static_cast<unsigned long long>(sparse_max), d_counts);
   if ((parts & MUT_PART_COV) && n_ev > 0)
      mut_cov_kernel<<<n_ev, MT, 0, s>>>(d_table, col, d_ev, d_filter, d_filter_count,
                                         static_cast<unsigned long long>(sparse_max), d_scratch);
   if (parts & MUT_PART_FINAL)
      mut_final_kernel<<<(col_host.L + MUT_SEG - 1) / MUT_SEG, MUT_SEG, 0, s>>>(d_table, col, d_filter_count, d_counts,
                                                                               d_scratch);
}

}  // namespace rhygpu
