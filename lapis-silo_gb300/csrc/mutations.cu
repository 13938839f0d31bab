// Mutations action kernels of the plain single-query path.
//
//  mut_stream_kernel every vertical container once: |F ∩ container| against the filter tile of its
//                    chunk staged in shared memory; integer counts per (symbol, position)
//                    (reference: mutations_node.cpp:139-189). The payload arena is streamed in
//                    units of 16 KiB by TMA bulk copies into double-buffered shared memory.
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

// Testing the failure path of the bounded waits: when set (on the current device), every CTA of the
// container pass announces the bytes of its first unit's copy on its barrier but never issues the
// copy, so its wait gives up (after 1 ms) and the call reports error 7. No copy is left in
// flight: the withheld copy never starts and the CTA waits for its other copy before it returns.
// Off by default; set only through set_copy_withholding.
__device__ uint32_t g_withhold_first_copy = 0;

constexpr uint32_t MT = 256;
constexpr uint32_t NW = MT / 32;

constexpr uint32_t STAGED_UNITS = 64;  // units of one CTA staged in shared memory
constexpr uint32_t EPT = SU / MT;      // array elements per thread in a unit (16)
constexpr uint32_t DESC_CAP = 256;     // descriptors of an array unit copied beside its payload
constexpr uint32_t BUF4 = SU / 8 + DESC_CAP;  // uint4 per buffer: payload, then descriptors
static_assert(EPT == 16, "units hold 16 elements per thread");

// Block-wide exclusive prefix sum of one value per thread; *total receives the sum. Contains
// one barrier; the caller separates consecutive calls with another.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t x, uint32_t* wsum, uint32_t* total) {
   const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
   uint32_t incl = x;
#pragma unroll
   for (uint32_t o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
      if (lane >= o) incl += y;
   }
   if (lane == 31) wsum[warp] = incl;
   __syncthreads();
   uint32_t before = 0, all = 0;
#pragma unroll
   for (uint32_t w = 0; w < NW; ++w) {
      const uint32_t v = wsum[w];
      before += w < warp ? v : 0u;
      all += v;
   }
   *total = all;
   return before + incl - x;
}

// Container pass of the Mutations action, streaming the payload arena. Persistent CTAs walk a
// contiguous range of the column's stream units (chunk-major), staged in shared memory:
//   SU_ARRAYS  up to SU consecutive elements of a chunk's array payloads (arrays are stored back to
//              back in descriptor order), with the descriptor range [c0, c1) overlapping them;
//   SU_BITSET  one bitset container; SU_RUN one run container.
// Array and bitset payloads, and the first DESC_CAP descriptors of an array unit, are double-
// buffered into shared memory by TMA bulk copies completing on one mbarrier (the copy of the next
// unit is in flight while the current one is counted). For array units thread t tests elements
// EPT t .. EPT t + EPT - 1 against the filter tile of the chunk (staged in shared memory), a
// block prefix sum over the membership bits gives every container its |F ∩ c| as the difference
// of two prefix values, added to counts[symbol][position] (containers cut by a unit boundary add
// two partial counts). Full filters (|F| == rows) use the stored cardinalities
// (reference: mutations_node.cpp:139-190, full path :240-266).
__global__ void __launch_bounds__(MT, 6) mut_stream_kernel(const DevTable* __restrict__ tab, uint32_t col,
                                                        const uint32_t* __restrict__ filter,
                                                        const unsigned long long* __restrict__ fcount,
                                                        unsigned long long sparse_max, uint32_t* counts, int* err) {
   extern __shared__ __align__(128) uint4 sm4[];  // two buffers (payload + descriptors), then the filter tile
   __shared__ __align__(8) uint64_t bar[2];
   __shared__ uint32_t wsum[NW], msk[MT], exq[MT];
   __shared__ StreamUnit su[STAGED_UNITS];  // this CTA's units, staged once
   const unsigned long long fc = *fcount;
   if (fc == 0 || fc <= sparse_max) return;  // empty, or counted by the row-index pass
   const bool full = fc == tab->n_rows;
   const DevSeqCol* cs = &tab->seq[col];
   const uint32_t n_units = cs->nsu;
   const uint32_t u0 = static_cast<uint32_t>(static_cast<uint64_t>(blockIdx.x) * n_units / gridDim.x);
   const uint32_t u1 = static_cast<uint32_t>(static_cast<uint64_t>(blockIdx.x + 1) * n_units / gridDim.x);
   if (u0 >= u1) return;
   const StreamUnit* __restrict__ gunits = cs->su;
   const CtrDesc* __restrict__ ctrs = cs->ctrs;
   const uint16_t* __restrict__ payload = cs->payload;
   const uint32_t L = cs->L, tid = threadIdx.x;
   const bool withhold = *static_cast<volatile uint32_t*>(&g_withhold_first_copy) != 0;
   const uint64_t wait_limit = withhold ? WAIT_LIMIT_TEST_NS : WAIT_LIMIT_NS;
   uint32_t* F = reinterpret_cast<uint32_t*>(sm4 + 2 * BUF4);
   if (tid == 0) {
      mbar_init(&bar[0]);
      mbar_init(&bar[1]);
   }
   for (uint32_t i = tid; i < u1 - u0 && i < STAGED_UNITS; i += MT) su[i] = gunits[u0 + i];
   __syncthreads();
   auto unit = [&](uint32_t u) { return u - u0 < STAGED_UNITS ? su[u - u0] : gunits[u]; };
   auto copies = [&](const StreamUnit& U) { return !full && U.kind != SU_RUN; };
   auto issue = [&](const StreamUnit& U, uint32_t b) {  // thread 0: payload and descriptors on one barrier
      const uint32_t bytes = U.kind == SU_BITSET ? CHUNK_ROWS / 8 : ((U.e1 - U.e0) * 2u + 15u) & ~15u;
      const uint32_t nd = U.kind == SU_ARRAYS ? min(U.c1 - U.c0, DESC_CAP) : 0u;
      mbar_expect(&bar[b], bytes + nd * 16u);
      bulk_copy_g2s_tx(sm4 + b * BUF4, payload + U.e0, bytes, &bar[b]);
      if (nd) bulk_copy_g2s_tx(sm4 + b * BUF4 + SU / 8, ctrs + U.c0, nd * 16u, &bar[b]);
   };
   uint32_t issued0 = 0, issued1 = 0;  // copies issued into each buffer (the same in every thread)
   {
      const StreamUnit U = unit(u0);
      if (copies(U)) {
         if (tid == 0) {
            if (withhold) mbar_expect(&bar[0], 16u);  // announced, never issued: the wait gives up
            else issue(U, 0);
         }
         ++issued0;
      }
   }
   uint32_t cur_v = 0xFFFFFFFFu;
   bool ok = true;
   for (uint32_t u = u0; u < u1 && ok; ++u) {
      const uint32_t b = (u - u0) & 1u;
      const StreamUnit U = unit(u);
      if (!full && U.v != cur_v) {
         const uint4* src = reinterpret_cast<const uint4*>(filter + static_cast<size_t>(U.v) * CHUNK_WORDS);
         for (uint32_t i = tid; i < CHUNK_WORDS / 4; i += MT) reinterpret_cast<uint4*>(F)[i] = __ldg(src + i);
         cur_v = U.v;
      }
      if (u + 1 < u1) {
         const StreamUnit N = unit(u + 1);
         if (copies(N)) {
            if (tid == 0) issue(N, b ^ 1u);
            if (b) ++issued0;
            else ++issued1;
         }
      }
      if (copies(U)) ok = mbar_wait(&bar[b], ((b ? issued1 : issued0) - 1u) & 1u, wait_limit);
      if (!__syncthreads_and(ok)) {
         ok = false;  // in every thread: the cleanup below has a barrier
         if (tid == 0) atomicExch(err, 7);
         break;
      }
      if (U.kind == SU_ARRAYS) {
         if (full) {
            for (uint32_t c = U.c0 + tid; c < U.c1; c += MT) {
               const uint4 raw = __ldg(reinterpret_cast<const uint4*>(ctrs) + c);
               const CtrDesc d = *reinterpret_cast<const CtrDesc*>(&raw);
               if (d.type != CT_ARRAY) continue;
               const uint32_t s = max(d.payload, U.e0), e = min(d.payload + d.card_m1 + 1u, U.e1);
               if (s < e) atomicAdd(&counts[static_cast<size_t>(d.sym) * L + d.key], e - s);
            }
         } else {
            const uint4* sdesc = sm4 + b * BUF4 + SU / 8;
            const uint32_t n = U.e1 - U.e0;
            const uint4* q = sm4 + b * BUF4 + 2 * tid;
            uint32_t m = 0;
            // element r of the chunk sets mask bit k when row r is in F: the filter word holding r,
            // rotated right by (r - k) mod 32, has that row's bit at position k
            if (n == SU) {
#pragma unroll
               for (uint32_t j = 0; j < 2; ++j) {
                  const uint4 x = q[j];
#pragma unroll
                  for (uint32_t t = 0; t < 8; ++t) {
                     const uint32_t r = u16_of(x, t), k = 8 * j + t;
                     const uint32_t w = F[r >> 5];
                     m |= __funnelshift_r(w, w, r - k) & (1u << k);
                  }
               }
            } else {
#pragma unroll
               for (uint32_t j = 0; j < 2; ++j) {
                  const uint4 x = q[j];
#pragma unroll
                  for (uint32_t t = 0; t < 8; ++t) {
                     const uint32_t r = u16_of(x, t), k = 8 * j + t;
                     const uint32_t w = F[r >> 5];
                     if (EPT * tid + k < n) m |= __funnelshift_r(w, w, r - k) & (1u << k);
                  }
               }
            }
            uint32_t total;
            const uint32_t ex = block_excl_scan(__popc(m), wsum, &total);
            msk[tid] = m;
            exq[tid] = ex;
            __syncthreads();
            auto prefix = [&](uint32_t i) -> uint32_t {  // members among elements [0, i)
               if (i / EPT >= MT) return total;
               return exq[i / EPT] + __popc(msk[i / EPT] & ((1u << (i % EPT)) - 1u));
            };
            for (uint32_t c = U.c0 + tid; c < U.c1; c += MT) {
               const uint4 raw = c - U.c0 < DESC_CAP ? sdesc[c - U.c0] : __ldg(reinterpret_cast<const uint4*>(ctrs) + c);
               const CtrDesc d = *reinterpret_cast<const CtrDesc*>(&raw);
               if (d.type != CT_ARRAY) continue;
               const uint32_t s = max(d.payload, U.e0), e = min(d.payload + d.card_m1 + 1u, U.e1);
               if (s >= e) continue;
               const uint32_t k = prefix(e - U.e0) - prefix(s - U.e0);
               if (k) atomicAdd(&counts[static_cast<size_t>(d.sym) * L + d.key], k);
            }
         }
      } else {
         const uint4 raw = __ldg(reinterpret_cast<const uint4*>(ctrs) + U.c0);
         const CtrDesc d = *reinterpret_cast<const CtrDesc*>(&raw);
         uint32_t k = 0;
         if (full) {
            k = tid == 0 ? d.card_m1 + 1u : 0u;
         } else if (U.kind == SU_BITSET) {
            const uint4* x = sm4 + b * BUF4;
            const uint4* f = reinterpret_cast<const uint4*>(F);
#pragma unroll
            for (uint32_t j = 0; j < CHUNK_WORDS / 4 / MT; ++j) {
               const uint4 a = x[tid + j * MT], y = f[tid + j * MT];
               k += __popc(a.x & y.x) + __popc(a.y & y.y) + __popc(a.z & y.z) + __popc(a.w & y.w);
            }
         } else {
            const uint16_t* r = payload + d.payload;
            for (uint32_t i = tid; i < d.nruns; i += MT) {
               const uint32_t s = __ldg(r + 2 * i);
               k += count_range(F, s, s + __ldg(r + 2 * i + 1) + 1u);
            }
         }
         k = __reduce_add_sync(0xFFFFFFFFu, k);
         if ((tid & 31) == 0 && k) atomicAdd(&counts[static_cast<size_t>(d.sym) * L + d.key], k);
      }
      __syncthreads();
   }
   if (!ok) {  // let the copies still in flight land before the CTA's shared memory is released
      if (tid == 0) {
         if (issued0) mbar_wait(&bar[0], (issued0 - 1u) & 1u, wait_limit);
         if (issued1) mbar_wait(&bar[1], (issued1 - 1u) & 1u, wait_limit);
      }
      __syncthreads();
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

void set_copy_withholding(bool on) {
   const uint32_t v = on ? 1u : 0u;
   const cudaError_t e = cudaMemcpyToSymbol(g_withhold_first_copy, &v, sizeof(v));
   if (e != cudaSuccess) throw std::runtime_error(std::string("set_copy_withholding: ") + cudaGetErrorString(e));
}

void launch_mutations(const DevTable* d_table, const DevSeqCol& col_host, uint32_t col, uint32_t nchunks,
                      const EvItem* d_ev, uint32_t n_ev, const uint32_t* d_filter,
                      const unsigned long long* d_filter_count, uint32_t* d_counts, uint32_t* d_scratch, int* d_err,
                      void* stream, uint32_t parts, uint64_t sparse_max) {
   cudaStream_t s = static_cast<cudaStream_t>(stream);
   if (!(parts & MUT_PART_SPARSE)) sparse_max = 0;  // the dense passes count every filter
   if (sparse_max) {
      const uint32_t groups = nchunks * CHUNK_WORDS / 32;  // 32-word groups, one per warp and step
      mut_sparse_kernel<<<std::max(1u, std::min(groups / NW, 2048u)), MT, 0, s>>>(
         d_table, col, d_filter, d_filter_count, static_cast<unsigned long long>(sparse_max), d_counts, d_scratch);
   }
   if ((parts & MUT_PART_CTR) && col_host.nsu > 0) {
      const size_t smem = 2 * BUF4 * 16 + CHUNK_WORDS * 4;
      // resident CTAs per device, computed once per device
      static std::atomic<uint32_t> resident[64];
      int dev = 0;
      cudaGetDevice(&dev);
      uint32_t res = dev >= 0 && dev < 64 ? resident[dev].load(std::memory_order_relaxed) : 0u;
      if (res == 0) {
         int sms = 0, per_sm = 0;
         cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
         if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mut_stream_kernel, MT, smem) != cudaSuccess ||
             per_sm < 1)
            per_sm = 1;
         res = static_cast<uint32_t>(std::max(sms, 1) * per_sm);
         if (dev >= 0 && dev < 64) resident[dev].store(res, std::memory_order_relaxed);
      }
      const uint32_t grid = std::min<uint32_t>(col_host.nsu, res);
      mut_stream_kernel<<<grid, MT, smem, s>>>(d_table, col, d_filter, d_filter_count,
                                               static_cast<unsigned long long>(sparse_max), d_counts, d_err);
   }
   if ((parts & MUT_PART_COV) && n_ev > 0)
      mut_cov_kernel<<<n_ev, MT, 0, s>>>(d_table, col, d_ev, d_filter, d_filter_count,
                                         static_cast<unsigned long long>(sparse_max), d_scratch);
   if (parts & MUT_PART_FINAL)
      mut_final_kernel<<<(col_host.L + MUT_SEG - 1) / MUT_SEG, MUT_SEG, 0, s>>>(d_table, col, d_filter_count, d_counts,
                                                                               d_scratch);
}

}  // namespace rhygpu
