// Mutations action kernels of the plain single-query path.
//
//  mut_ring_kernel   every vertical container once: |F ∩ container| against the filter tile of its
//                    chunk staged in shared memory; integer counts per (symbol, position)
//                    (reference: mutations_node.cpp:139-189). A producer warp bulk-copies units of
//                    at most WU array elements into a shared-memory ring that consumer warps count.
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

// Shared-memory ring of the container pass.
constexpr uint32_t RING_SLOTS = 16;
constexpr uint32_t RING_CONSUMERS = 8;                 // consumer warps per CTA; warp 0 is the producer
constexpr uint32_t RING_T = 32 * (RING_CONSUMERS + 1);
constexpr uint32_t SLOT_HDR = 16;                      // e0, c0, n | tile << 15 | nd << 16, unit ordinal
constexpr uint32_t SLOT_PAY = 2 * WU;                  // the unit's payload (u16 row ids)
constexpr uint32_t SLOT_BYTES = SLOT_HDR + SLOT_PAY + 16 * WU_DESC;  // then its first WU_DESC descriptors
static_assert(SLOT_BYTES % 16 == 0, "slots start on 16-byte boundaries");
struct Ring {
   uint32_t F[2][CHUNK_WORDS];             // filter tiles of the range's chunks v0 and v1
   uint8_t slot[RING_SLOTS][SLOT_BYTES];
   uint64_t full[RING_SLOTS];              // a slot's copies landed (one arrival + bytes)
   uint64_t empty[RING_SLOTS];             // a slot's unit was counted (one arrival)
   uint64_t tile[2];
   uint32_t next_arr, next_oth, abort_flag;
   uint32_t issued[RING_SLOTS];            // rounds of copies issued into each slot
};
constexpr size_t RING_SMEM = sizeof(Ring);

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
   const uint32_t b = static_cast<uint32_t>(__cvta_generic_to_shared(bar));
   asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(b) : "memory");
}

// Waits for the phase of `bar` with the given parity to complete. It polls without a suspend hint
// and sleeps between polls (backing off up to max_sleep_ns), so that a warp waiting on the ring
// takes few issue slots from the warps that count. Bounded by limit_ns on the global timer and by
// 2^26 polls; false if it gave up.
__device__ __forceinline__ bool ring_wait(uint64_t* bar, uint32_t parity, uint32_t max_sleep_ns, uint64_t limit_ns) {
   const uint32_t b = static_cast<uint32_t>(__cvta_generic_to_shared(bar));
   uint64_t t0 = 0;
   uint32_t ns = 16;
   for (uint32_t i = 0; i < (1u << 26); ++i) {
      uint32_t done;
      asm volatile(
         "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
         : "=r"(done)
         : "r"(b), "r"(parity)
         : "memory");
      if (done) return true;
      const uint64_t now = global_ns();
      if (t0 == 0) t0 = now;
      else if (now - t0 > limit_ns) return false;
      __nanosleep(ns);
      ns = min(2 * ns, max_sleep_ns);
   }
   return false;
}

// Non-blocking test of the phase of `bar` with the given parity.
__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
   const uint32_t b = static_cast<uint32_t>(__cvta_generic_to_shared(bar));
   uint32_t done;
   asm volatile(
      "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(b), "r"(parity)
      : "memory");
   return done != 0;
}

// One arrival on a ring slot's full barrier that announces `bytes` of bulk copies. No proxy fence
// is needed here: the slot's previous contents were only read by generic loads of the consumer that
// released it through the empty barrier this thread waited on, and the header that this thread
// writes with generic stores is read only by generic loads.
__device__ __forceinline__ void ring_expect(uint64_t* bar, uint32_t bytes) {
   const uint32_t b = static_cast<uint32_t>(__cvta_generic_to_shared(bar));
   asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}\n" ::"r"(b), "r"(bytes)
                : "memory");
}

// Waits until the producer has written unit ordinal k into a slot header (bounded by limit_ns).
// A consumer that runs a whole ring ahead sees the previous round's ordinal until then; checking
// the ordinal first keeps its barrier wait from matching the previous round's phase.
__device__ __forceinline__ bool wait_slot_unit(const uint32_t* hdr, uint32_t k, uint64_t limit_ns) {
   uint64_t t0 = 0;
   for (uint32_t i = 0; i < (1u << 26); ++i) {
      if (*reinterpret_cast<const volatile uint32_t*>(hdr + 3) == k) return true;
      const uint64_t now = global_ns();
      if (t0 == 0) t0 = now;
      else if (now - t0 > limit_ns) return false;
      __nanosleep(64);
   }
   return false;
}

// Testing the failure path of the container pass's bounded waits: while set (on the current
// device), the producer announces each unit's copy bytes on the slot's barrier but never issues the
// copies, so the consumers' waits give up (after 1 ms) and the pass sets DEVERR_WAIT_MUTATIONS. No
// copy is left in flight: the withheld copies never start. Off by default; set only through
// set_ring_withholding.
__device__ uint32_t g_withhold_ring_copies = 0;

// 32 x 32 bit transpose across a warp: lane j returns the word whose bit l is bit j of lane l's x.
// Five exchange steps, step s swapping bit s of the lane index with bit s of the bit index.
__device__ __forceinline__ uint32_t warp_transpose32(uint32_t x, uint32_t lane) {
#pragma unroll
   for (uint32_t s = 16; s >= 1; s >>= 1) {
      const uint32_t M0 = s == 16 ? 0x0000FFFFu : s == 8 ? 0x00FF00FFu : s == 4 ? 0x0F0F0F0Fu : s == 2 ? 0x33333333u : 0x55555555u;
      const uint32_t p = __shfl_xor_sync(0xFFFFFFFFu, x, s);
      x = (lane & s) ? ((x & ~M0) | ((p >> s) & M0)) : ((x & M0) | ((p << s) & ~M0));
   }
   return x;
}

// Membership bits of a unit's row ids in the filter tile F: W[it] holds the two u16 row ids of
// elements 64 it + 2 lane and 64 it + 2 lane + 1, whose bits land at 2 it and 2 it + 1. The bit of
// row r is bit r & 31 of word r >> 5; rotating that word right by (r - k) & 31 brings it to bit k
// (the rotation takes its amount modulo 32, so neither half of W needs masking).
__device__ __forceinline__ uint32_t unit_members(const uint32_t (&W)[WU / 64], const uint32_t* __restrict__ F) {
   uint32_t m = 0;
#pragma unroll
   for (uint32_t it = 0; it < WU / 64; ++it) {
      const uint32_t w = W[it], hi = w >> 16;
      const uint32_t f0 = F[(w >> 5) & 0x7FFu], f1 = F[hi >> 5];
      m |= __funnelshift_r(f0, f0, w - 2 * it) & (1u << (2 * it));
      m |= __funnelshift_r(f1, f1, hi - (2 * it + 1)) & (2u << (2 * it));
   }
   return m;
}

// Container pass of the Mutations action (reference: mutations_node.cpp:139-190, full path
// :240-266): |F ∩ c| for every container c of the column, added to counts[symbol][position].
// One CTA per host-built range (array units and bitset / run units of at most two chunks):
//   warp 0 (producer) bulk-copies the filter tiles of the range's chunks; then its lane j keeps
//     ring slot j busy: it copies the payload (row ids, WU at most) and the first WU_DESC
//     descriptors of units j, j + RING_SLOTS, ... into the slot, each as soon as the slot's previous
//     unit was released (full / empty mbarrier pair per slot), so that up to RING_SLOTS units are in
//     flight while earlier ones are counted;
//   warps 1..8 (consumers) first count the bitset and run units straight from global memory, then
//     claim array units in order; a claimed unit moves into registers and its slot is released.
//     Lane l holds elements 64 it + 2l and 64 it + 2l + 1 of step it and sets their membership bits
//     (bits 2 it and 2 it + 1); a warp bit transpose gives lane 2q the bits of the even and lane
//     2q + 1 those of the odd elements of [64q, 64q + 64), and a prefix sum over the lanes turns
//     every descriptor's |F ∩ c| into the difference of two prefix values (a container cut by a
//     unit boundary adds two partial counts).
// Full filters (|F| == rows) add the stored cardinalities: only descriptors are copied. Every wait
// is bounded; one that gives up sets DEVERR_WAIT_MUTATIONS in *err and ends the CTA's work.
__global__ void __launch_bounds__(RING_T, RING_CTAS_PER_SM) mut_ring_kernel(const DevTable* __restrict__ tab, uint32_t col,
                                                          const uint32_t* __restrict__ filter,
                                                          const unsigned long long* __restrict__ fcount,
                                                          unsigned long long sparse_max, uint32_t* counts, int* err) {
   extern __shared__ __align__(128) uint8_t ring_raw[];
   Ring& R = *reinterpret_cast<Ring*>(ring_raw);
   const unsigned long long fc = *fcount;
   if (fc == 0 || fc <= sparse_max) return;  // empty, or counted by the row-index pass
   const bool full = fc == tab->n_rows;
   const DevSeqCol* cs = &tab->seq[col];
   const StreamRange rg = cs->ranges[blockIdx.x];
   const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, L = cs->L;
   const uint32_t na = rg.a1 - rg.a0, no = rg.o1 - rg.o0;
   const bool two = rg.v1 != rg.v0;
   const bool withhold = *static_cast<volatile uint32_t*>(&g_withhold_ring_copies) != 0;
   const uint64_t limit = withhold ? WAIT_LIMIT_TEST_NS : WAIT_LIMIT_NS;
   if (tid == 0) {
      for (uint32_t s = 0; s < RING_SLOTS; ++s) {
         mbar_init(&R.full[s]);
         mbar_init(&R.empty[s]);
      }
      mbar_init(&R.tile[0]);
      mbar_init(&R.tile[1]);
      R.next_arr = 0;
      R.next_oth = 0;
      R.abort_flag = 0;
   }
   if (tid < RING_SLOTS) {
      reinterpret_cast<uint32_t*>(R.slot[tid])[3] = 0xFFFFFFFFu;  // no unit yet
      R.issued[tid] = 0;
   }
   __syncthreads();
   const CtrDesc* __restrict__ ctrs = cs->ctrs;
   volatile uint32_t* abort_flag = &R.abort_flag;
   if (warp == 0) {
      // ---------------- producer ----------------
      if (lane == 0 && !full) {
         mbar_expect(&R.tile[0], CHUNK_WORDS * 4);
         bulk_copy_g2s_tx(R.F[0], filter + static_cast<size_t>(rg.v0) * CHUNK_WORDS, CHUNK_WORDS * 4, &R.tile[0]);
         if (two) {
            mbar_expect(&R.tile[1], CHUNK_WORDS * 4);
            bulk_copy_g2s_tx(R.F[1], filter + static_cast<size_t>(rg.v1) * CHUNK_WORDS, CHUNK_WORDS * 4, &R.tile[1]);
         }
      }
      // lane j < RING_SLOTS owns slot j and issues the units j, j + RING_SLOTS, ... into it, each as
      // soon as the consumer of the slot's previous unit has released it: one pass of the warp
      // refills every free slot
      bool ok = true;
      const uint4* recs = reinterpret_cast<const uint4*>(cs->au) + rg.a0;
      uint32_t kj = lane;  // this lane's next unit
      uint4 rec = lane < RING_SLOTS && kj < na ? __ldg(recs + kj) : make_uint4(0, 0, 0, 0);
      uint64_t t_idle = 0;
      uint32_t ns = 32;
      for (;;) {
         const bool mine = lane < RING_SLOTS && kj < na;
         if (!__any_sync(0xFFFFFFFFu, mine)) break;
         if (*abort_flag) {
            ok = false;
            break;
         }
         const uint32_t round = kj / RING_SLOTS;
         const bool ready = mine && (round == 0 || mbar_test(&R.empty[lane], (round - 1) & 1u));
         if (ready) {
            const uint32_t n = rec.z & 0xFFFFu, nd = rec.z >> 16;
            uint32_t* h = reinterpret_cast<uint32_t*>(R.slot[lane]);
            const uint32_t pay = full ? 0u : (2 * n + 15) & ~15u;
            const uint32_t dsc = 16 * min(nd, WU_DESC);
            h[0] = rec.x;
            h[1] = rec.y;
            h[2] = n | ((rec.w == rg.v0 ? 0u : 1u) << 15) | (nd << 16);
            *reinterpret_cast<volatile uint32_t*>(h + 3) = kj;
            ring_expect(&R.full[lane], pay + dsc);
            if (!withhold) {
               if (pay) bulk_copy_g2s_tx(R.slot[lane] + SLOT_HDR, cs->payload + rec.x, pay, &R.full[lane]);
               bulk_copy_g2s_tx(R.slot[lane] + SLOT_HDR + SLOT_PAY, ctrs + rec.y, dsc, &R.full[lane]);
            }
            R.issued[lane] = round + 1;
            kj += RING_SLOTS;
            rec = kj < na ? __ldg(recs + kj) : make_uint4(0, 0, 0, 0);  // in flight until the slot frees
         }
         if (__any_sync(0xFFFFFFFFu, ready)) {
            t_idle = 0;
            ns = 32;
            continue;
         }
         // no slot free: back off, bounded by the time since the last copy was issued
         const uint64_t now = global_ns();
         if (t_idle == 0) t_idle = now;
         else if (now - t_idle > limit) {
            ok = false;
            break;
         }
         __nanosleep(ns);
         ns = min(2 * ns, 256u);
      }
      if (!ok && lane == 0) {
         *abort_flag = 1;
         if (err) atomicExch(err, DEVERR_WAIT_MUTATIONS);
      }
   } else {
      // ---------------- consumers ----------------
      bool ok = full || (ring_wait(&R.tile[0], 0, 256, limit) && (!two || ring_wait(&R.tile[1], 0, 256, limit)));
      ok = __all_sync(0xFFFFFFFFu, ok);
      // bitset and run units first, straight from global memory, while the producer fills the ring
      while (ok && *abort_flag == 0) {
         uint32_t u = 0;
         if (lane == 0) u = atomicAdd(&R.next_oth, 1u);
         u = __shfl_sync(0xFFFFFFFFu, u, 0);
         if (u >= no) break;
         const uint4 uraw = __ldg(reinterpret_cast<const uint4*>(cs->ou) + rg.o0 + u);
         const OtherUnit U = *reinterpret_cast<const OtherUnit*>(&uraw);
         const uint32_t* F = R.F[U.v == rg.v0 ? 0 : 1];
         const uint4 raw = __ldg(reinterpret_cast<const uint4*>(ctrs) + U.c);
         const CtrDesc d = *reinterpret_cast<const CtrDesc*>(&raw);
         uint32_t k = 0;
         if (full) {
            k = lane == 0 ? d.card_m1 + 1u : 0u;
         } else if (U.kind == SU_BITSET) {
            const uint4* f4 = reinterpret_cast<const uint4*>(F);
            const uint4* p4 = reinterpret_cast<const uint4*>(cs->payload + U.e0);
            constexpr uint32_t BV = CHUNK_WORDS / 4 / 32, BB = 8;  // uint4 per lane; loads in flight
#pragma unroll
            for (uint32_t j0 = 0; j0 < BV; j0 += BB) {
               uint4 a[BB];
#pragma unroll
               for (uint32_t j = 0; j < BB; ++j) a[j] = __ldg(p4 + lane + 32 * (j0 + j));
#pragma unroll
               for (uint32_t j = 0; j < BB; ++j) {
                  const uint4 y = f4[lane + 32 * (j0 + j)];
                  k += __popc(a[j].x & y.x) + __popc(a[j].y & y.y) + __popc(a[j].z & y.z) + __popc(a[j].w & y.w);
               }
            }
         } else {
            const uint16_t* r = cs->payload + d.payload;
            for (uint32_t i = lane; i < d.nruns; i += 32) {
               const uint32_t s0 = __ldg(r + 2 * i);
               k += count_range(F, s0, s0 + __ldg(r + 2 * i + 1) + 1u);
            }
         }
         k = __reduce_add_sync(0xFFFFFFFFu, k);
         if (lane == 0 && k) atomicAdd(&counts[static_cast<size_t>(d.sym) * L + d.key], k);
      }
      // array units from the ring, in order of claim: the unit moves into registers and its slot is
      // released before it is counted
      while (ok && *abort_flag == 0) {
         uint32_t k = 0;
         if (lane == 0) k = atomicAdd(&R.next_arr, 1u);
         k = __shfl_sync(0xFFFFFFFFu, k, 0);
         if (k >= na) break;
         const uint32_t s = k % RING_SLOTS, round = k / RING_SLOTS;
         const uint8_t* slot = R.slot[s];
         const uint32_t* h = reinterpret_cast<const uint32_t*>(slot);
         ok = __all_sync(0xFFFFFFFFu, wait_slot_unit(h, k, limit) && ring_wait(&R.full[s], round & 1u, 128, limit));
         if (!ok) break;
         const uint32_t e0 = h[0], c0 = h[1], w2 = h[2];
         const uint32_t n = w2 & 0x7FFFu, nd = w2 >> 16, tile = (w2 >> 15) & 1u;
         uint32_t W[WU / 64];
         if (!full) {
            const uint32_t* pw = reinterpret_cast<const uint32_t*>(slot + SLOT_HDR) + lane;
#pragma unroll
            for (uint32_t it = 0; it < WU / 64; ++it) W[it] = pw[32 * it];
         }
         const uint4* dsl = reinterpret_cast<const uint4*>(slot + SLOT_HDR + SLOT_PAY);
         const uint32_t nds = min(nd, WU_DESC);
         uint4 D[WU_DESC / 32];
#pragma unroll
         for (uint32_t g = 0; g < WU_DESC / 32; ++g) D[g] = 32 * g + lane < nds ? dsl[32 * g + lane] : make_uint4(0, 0, 0, 0);
         __syncwarp();
         if (lane == 0) mbar_arrive(&R.empty[s]);
         // lane l bit 2 it + h: element 64 it + 2 l + h is in F; after the transpose lane 2q holds the
         // bits of the even and lane 2q + 1 those of the odd elements of [64q, 64q + 64)
         uint32_t T = 0, pb = 0, total = 0;
         if (!full) {
            uint32_t m = tile ? unit_members(W, R.F[1]) : unit_members(W, R.F[0]);
            if (n < WU) {  // elements past the unit's end hold stale slot contents
               uint32_t valid = 0;
#pragma unroll
               for (uint32_t it = 0; it < WU / 64; ++it) {
                  const uint32_t idx = 64 * it + 2 * lane;
                  valid |= (idx < n ? 1u : 0u) << (2 * it);
                  valid |= (idx + 1 < n ? 2u : 0u) << (2 * it);
               }
               m &= valid;
            }
            T = warp_transpose32(m, lane);
            const uint32_t c = __popc(T);
            uint32_t incl = c;
#pragma unroll
            for (uint32_t o = 1; o < 32; o <<= 1) {
               const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
               if (lane >= o) incl += y;
            }
            pb = incl - c;  // lane 2q: members before element 64q
            total = __shfl_sync(0xFFFFFFFFu, incl, 31);
         }
         auto prefix = [&](uint32_t i) -> uint32_t {  // members among the unit's elements [0, i), i <= n
            const uint32_t q = (i >> 6) & 15u, l = (i >> 1) & 31u;
            const uint32_t base = __shfl_sync(0xFFFFFFFFu, pb, 2 * q);
            const uint32_t e = __shfl_sync(0xFFFFFFFFu, T, 2 * q), o = __shfl_sync(0xFFFFFFFFu, T, 2 * q + 1);
            const uint32_t m = (1u << l) - 1u;
            const uint32_t v = base + __popc(e & m) + __popc(o & m) + ((i & 1u) ? ((e >> l) & 1u) : 0u);
            return i >= WU ? total : v;
         };
         auto count_desc = [&](const uint4& raw, uint32_t j) {  // descriptor j of the unit (lane-varying)
            uint32_t a = 0, b = 0, sym = 0, key = 0;
            if (j < nd) {
               const CtrDesc d = *reinterpret_cast<const CtrDesc*>(&raw);
               if (d.type == CT_ARRAY) {
                  const uint32_t x = max(d.payload, e0), y = min(d.payload + d.card_m1 + 1u, e0 + n);
                  if (x < y) {
                     a = x - e0;
                     b = y - e0;
                     sym = d.sym;
                     key = d.key;
                  }
               }
            }
            const uint32_t cnt = full ? b - a : prefix(b) - prefix(a);
            if (cnt) atomicAdd(&counts[static_cast<size_t>(sym) * L + key], cnt);
         };
#pragma unroll
         for (uint32_t g = 0; g < WU_DESC / 32; ++g)
            if (32 * g < nd) count_desc(D[g], 32 * g + lane);
         for (uint32_t j0 = WU_DESC; j0 < nd; j0 += 32) {  // descriptors past the slot's copy
            const uint32_t j = j0 + lane;
            count_desc(j < nd ? __ldg(reinterpret_cast<const uint4*>(ctrs) + c0 + j) : make_uint4(0, 0, 0, 0), j);
         }
      }
      if (!ok && lane == 0) {
         *abort_flag = 1;
         if (err) atomicExch(err, DEVERR_WAIT_MUTATIONS);
      }
   }
   __syncthreads();
   if (tid == 0 && *abort_flag) {
      // after a wait gave up: let the copies still in flight land before the CTA's shared memory is
      // released (the last round issued into each slot; bounded like every other wait)
      for (uint32_t s = 0; s < RING_SLOTS; ++s)
         if (R.issued[s] && !ring_wait(&R.full[s], (R.issued[s] - 1) & 1u, 256, limit)) break;
      if (!full) {
         ring_wait(&R.tile[0], 0, 256, limit);
         if (two) ring_wait(&R.tile[1], 0, 256, limit);
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

void set_ring_withholding(bool on) {
   const uint32_t v = on ? 1u : 0u;
   const cudaError_t e = cudaMemcpyToSymbol(g_withhold_ring_copies, &v, sizeof(v));
   if (e != cudaSuccess) throw std::runtime_error(std::string("set_ring_withholding: ") + cudaGetErrorString(e));
}

void mutations_setup() {
   const cudaError_t e = cudaFuncSetAttribute(mut_ring_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              static_cast<int>(RING_SMEM));
   if (e != cudaSuccess)
      throw std::runtime_error(std::string("shared memory of the Mutations container pass: ") + cudaGetErrorString(e));
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
   if ((parts & MUT_PART_CTR) && col_host.nranges > 0)
      mut_ring_kernel<<<col_host.nranges, RING_T, RING_SMEM, s>>>(
         d_table, col, d_filter, d_filter_count, static_cast<unsigned long long>(sparse_max), d_counts, d_err);
   if ((parts & MUT_PART_COV) && n_ev > 0)
      mut_cov_kernel<<<n_ev, MT, 0, s>>>(d_table, col, d_ev, d_filter, d_filter_count,
                                         static_cast<unsigned long long>(sparse_max), d_scratch);
   if (parts & MUT_PART_FINAL)
      mut_final_kernel<<<(col_host.L + MUT_SEG - 1) / MUT_SEG, MUT_SEG, 0, s>>>(d_table, col, d_filter_count, d_counts,
                                                                               d_scratch);
}

}  // namespace rhygpu
