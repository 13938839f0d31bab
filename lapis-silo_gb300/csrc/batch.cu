// Batched Mutations: many filters per pass over the vertical index and the missing-interval events.
//
// The plain path streams every container once per query. Here the filters of a batch are
// transposed into 16-bit query masks per row (bit q of group g = row in filter 16 g + q) and every
// container element and event is read once per pass of up to 256 queries. The container pass counts
// 32 queries per lane in bit-sliced counters; the event pass gives each lane one 16-query group in
// nibble counters. Results are bit-identical to the single-query kernels.
//
//   transpose_kernel       filter row sets -> masks, pass-major rows (32 B per row and pass)
//   mut_ctr_batch_kernel   container pass, one warp per (position, chunk range) unit: |F_q ∩ c|
//                          for every container c (reference: mutations_node.cpp:138-190)
//   mut_cov_batch_kernel   missing-interval and coverage boundary events (reference:
//                          mutations_node.cpp:51-136)
//   mut_final_batch_kernel prefix sums and reference counts per query
//   mut_select_kernel      splits the slots by their filter's cardinality: none for empty filters,
//                          the row-index pass for filters of at most sparse_max rows, the dense
//                          passes above (over a compacted slot list) for the others
//   mut_sparse_batch_kernel the row-index pass of the sparse slots
#include <cuda_runtime.h>

#include <algorithm>

#include "device.h"
#include "mutations_common.cuh"
#include "rows_rule.cuh"

namespace rhygpu {

constexpr uint32_t MUT_GROUP = 16;   // queries per 16-bit mask
constexpr uint32_t PASS_GROUPS = 16;  // groups per mask pass (256 queries, one 32-byte sector per row)

namespace {

constexpr uint32_t BT = 256;

// Mask layout: pass p (queries 256 p ..) holds rows x wp(p) u32, wp(p) = min(8, nqc - 8 p) with
// nqc = ceil(nq / 32); u32 c of a row holds groups 2c (low half) and 2c + 1 (high half) of the pass.
// Every pass but the last is rows x 8 u32, so pass p starts at u16 offset p * rows * 16.
__device__ __forceinline__ uint32_t pass_width_u32(uint32_t nqc, uint32_t pass) {
   return nqc - 8 * pass < 8 ? nqc - 8 * pass : 8u;
}

// A CTA covers TR_WORDS filter words (32 TR_WORDS rows); warp w turns word w of 32 filters at a
// time into 32 row masks with ballots and stages them in shared memory for coalesced row stores.
constexpr uint32_t TR_WORDS = BT / 32;
constexpr uint32_t TR_CHUNKS = 32;  // query chunks of 32 staged per round (a multiple of 8)

__global__ void __launch_bounds__(BT) transpose_kernel(const uint32_t* __restrict__ tiles,
                                                       const uint32_t* __restrict__ lists, uint32_t nq_max,
                                                       uint32_t nchunks, uint32_t* __restrict__ R) {
   __shared__ uint32_t stage[TR_WORDS * 32 * (TR_CHUNKS + 1)];
   const uint32_t nq = lists[2 * nq_max];  // dense slots: lists[0 .. nq)
   const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
   const uint32_t words = nchunks * CHUNK_WORDS;
   const uint32_t nqc = (nq + 31) / 32;
   const uint32_t w = blockIdx.x * TR_WORDS + warp;  // words is a multiple of TR_WORDS
   const size_t rows = static_cast<size_t>(words) * 32;
   const size_t row0 = static_cast<size_t>(blockIdx.x) * TR_WORDS * 32;
   for (uint32_t c0 = 0; c0 < nqc; c0 += TR_CHUNKS) {
      const uint32_t nc = nqc - c0 < TR_CHUNKS ? nqc - c0 : TR_CHUNKS;
      const uint32_t P = nc | 1u;  // odd stride: the 32 lanes of a warp hit 32 banks
      for (uint32_t c = 0; c < nc; ++c) {
         const uint32_t q = 32 * (c0 + c) + lane;
         const uint32_t x = q < nq ? __ldg(tiles + static_cast<size_t>(lists[q]) * words + w) : 0u;
         uint32_t mine = 0;
#pragma unroll
         for (uint32_t b = 0; b < 32; ++b) {
            const uint32_t m = __ballot_sync(0xFFFFFFFFu, (x >> b) & 1u);
            if (lane == b) mine = m;
         }
         stage[(warp * 32 + lane) * P + c] = mine;
      }
      __syncthreads();
      for (uint32_t pass = c0 / 8; pass * 8 < c0 + nc; ++pass) {
         const uint32_t wp = pass_width_u32(nqc, pass);
         uint32_t* dst = R + static_cast<size_t>(pass) * rows * 8 + row0 * wp;
         for (uint32_t k = threadIdx.x; k < TR_WORDS * 32 * wp; k += blockDim.x) {
            const uint32_t r = k / wp, ci = k % wp;
            dst[k] = stage[r * P + 8 * pass + ci - c0];
         }
      }
      __syncthreads();
   }
}

// Per-lane counters of the 16 queries of one group. Masks are added two at a time as one 32-bit
// word w = m1 | m2 << 16 into four words of nibble counters: nibble k of nib[j] counts query
// j + 4 (k % 4). After at most 15 additions the nibbles are drained into 32-bit counters.
struct NibbleCounter {
   uint32_t nib[4];
   uint32_t nadd;
   uint32_t c[MUT_GROUP];

   __device__ __forceinline__ void clear() {
#pragma unroll
      for (uint32_t j = 0; j < 4; ++j) nib[j] = 0;
      nadd = 0;
#pragma unroll
      for (uint32_t q = 0; q < MUT_GROUP; ++q) c[q] = 0;
   }
   __device__ __forceinline__ void drain() {
#pragma unroll
      for (uint32_t q = 0; q < MUT_GROUP; ++q) {
         const uint32_t a = nib[q & 3u], sh = 4u * (q >> 2);
         c[q] += ((a >> sh) & 0xFu) + ((a >> (sh + 16u)) & 0xFu);
      }
#pragma unroll
      for (uint32_t j = 0; j < 4; ++j) nib[j] = 0;
      nadd = 0;
   }
   __device__ __forceinline__ void add(uint32_t w) {
#pragma unroll
      for (uint32_t j = 0; j < 4; ++j) nib[j] += (w >> j) & 0x11111111u;
      if (++nadd == 15) drain();
   }
};

// Per-lane counters of the 32 queries of one mask word, as carry-save bit planes: bit q of ones,
// twos and fours holds bits 0..2 of query q's count, and byte j of eb[k] counts the eights of query
// 4k + j. Rows are added eight at a time by a Harley-Seal tree of carry-save adders (one LOP3 for
// the sum and one for the carry of three words); the tree's carry-out word, the queries whose count
// passed another multiple of eight, is spread into the byte counters (4 bits to 4 bytes by one
// multiply). At most 255 blocks of eight rows fit the bytes; the caller flushes before that.
struct BitCounter {
   uint32_t ones, twos, fours;
   uint32_t eb[8];
   uint32_t blocks;

   __device__ __forceinline__ void clear() {
      ones = twos = fours = 0;
#pragma unroll
      for (uint32_t k = 0; k < 8; ++k) eb[k] = 0;
      blocks = 0;
   }
   __device__ __forceinline__ static void csa(uint32_t& carry, uint32_t& sum, uint32_t a, uint32_t b, uint32_t c) {
      const uint32_t u = a ^ b;
      carry = (a & b) | (u & c);
      sum = u ^ c;
   }
   __device__ __forceinline__ void add8(const uint32_t (&m)[8]) {
      uint32_t twos_a, twos_b, fours_a, fours_b, eights;
      csa(twos_a, ones, ones, m[0], m[1]);
      csa(twos_b, ones, ones, m[2], m[3]);
      csa(fours_a, twos, twos, twos_a, twos_b);
      csa(twos_a, ones, ones, m[4], m[5]);
      csa(twos_b, ones, ones, m[6], m[7]);
      csa(fours_b, twos, twos, twos_a, twos_b);
      csa(eights, fours, fours, fours_a, fours_b);
#pragma unroll
      for (uint32_t k = 0; k < 8; ++k) eb[k] += (((eights >> (4 * k)) & 0xFu) * 0x00204081u) & 0x01010101u;
      ++blocks;
   }
   // query q's count: the three low planes plus eight times its byte counter
   __device__ __forceinline__ uint32_t count(uint32_t q) const {
      const uint32_t low = ((ones >> q) & 1u) | (((twos >> q) & 1u) << 1) | (((fours >> q) & 1u) << 2);
      return low + 8u * ((eb[q >> 2] >> (8 * (q & 3))) & 0xFFu);
   }
};

// Counts the rows rowbase + x_t, t < cnt, of a window held one per lane in x (warp-uniform cnt
// <= 32). Lane group g = lane / 8 takes elements g, g + 4, ..., g + 28; every lane reads word
// lane % 8 of each of its rows' masks (wp words per row, zero past wp) and adds the eight words.
__device__ __forceinline__ void count_window_bits(BitCounter& k, uint32_t x, uint32_t cnt, uint32_t rowbase,
                                                  const uint32_t* __restrict__ Rp, uint32_t wp, uint32_t lane) {
   const uint32_t g = lane >> 3, w = lane & 7u;
   uint32_t m[8];
#pragma unroll
   for (uint32_t i = 0; i < 8; ++i) {
      const uint32_t t = 4 * i + g;
      const uint32_t e = __shfl_sync(0xFFFFFFFFu, x, t);
      m[i] = (t < cnt && w < wp) ? __ldg(Rp + static_cast<size_t>(rowbase + e) * wp + w) : 0u;
   }
   k.add8(m);
}

// One warp per (unit, pass): for every symbol present at the unit's position, the containers of
// the unit's chunks are counted for all queries of the pass. Lane (g, w) = (lane / 8, lane % 8)
// adds mask word w (queries 32w .. 32w + 31 of the pass) of every fourth row of each 32-element
// window into its bit-sliced counters; the four groups' counts are summed with shuffles and added
// to counts once per symbol. Bitset containers are expanded 1024 rows at a time into a per-warp row
// list in shared memory.
__global__ void __launch_bounds__(BT, 4) mut_ctr_batch_kernel(const DevTable* __restrict__ tab, uint32_t col,
                                                           const CtrUnit* __restrict__ units, uint32_t n_units,
                                                           const uint16_t* __restrict__ R,
                                                           const uint32_t* __restrict__ lists, uint32_t nq_max,
                                                           uint32_t* __restrict__ counts) {
   __shared__ uint16_t list[BT / 32][1024];
   const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
   const uint32_t u = blockIdx.x * (BT / 32) + warp;
   const uint32_t nq = lists[2 * nq_max];  // dense slots: lists[0 .. nq)
   if (u >= n_units || blockIdx.y * PASS_GROUPS * MUT_GROUP >= nq) return;  // the whole warp leaves
   const DevSeqCol* cs = &tab->seq[col];
   const uint32_t L = cs->L;
   const size_t per_query = static_cast<size_t>(cs->nsym) * L;
   const CtrDesc* __restrict__ ctrs = cs->ctrs;
   const uint16_t* __restrict__ payload = cs->payload;
   const uint32_t pass = blockIdx.y;
   const uint32_t nqc = (nq + 31) / 32;
   const size_t rows = static_cast<size_t>(tab->nchunks) * CHUNK_ROWS;
   const uint32_t wp = pass_width_u32(nqc, pass);  // mask words per row in this pass
   const uint32_t* Rp = reinterpret_cast<const uint32_t*>(R + static_cast<size_t>(pass) * rows * 16);

   const CtrUnit unit = units[u];
   const uint32_t p = unit.pos, v0 = unit.v0, nv = unit.v1 - unit.v0;
   uint32_t cb = 0, ce = 0;  // lane i: the containers of chunk v0 + i at p
   if (lane < nv) {
      cb = __ldg(cs->off + static_cast<size_t>(v0 + lane) * L + p);
      ce = __ldg(cs->off + static_cast<size_t>(v0 + lane) * L + p + 1);
   }
   uint32_t symmask = 0;
   for (uint32_t i = cb; i < ce; ++i) symmask |= 1u << __ldg(&ctrs[i].sym);
   symmask = __reduce_or_sync(0xFFFFFFFFu, symmask);
   uint16_t* wl = list[warp];
   const uint32_t g = lane >> 3, w = lane & 7u;
   while (symmask) {
      const uint32_t s = __ffs(symmask) - 1;
      symmask &= symmask - 1;
      uint32_t idx = 0xFFFFFFFFu;
      for (uint32_t i = cb; i < ce; ++i)
         if (__ldg(&ctrs[i].sym) == s) idx = i;
      uint32_t have = __ballot_sync(0xFFFFFFFFu, idx != 0xFFFFFFFFu);
      BitCounter k;
      k.clear();
      // adds the counters of the four lane groups and the counts of this word's 32 queries to the
      // query tables, then clears (at the end of a symbol, or before the byte counters could wrap)
      auto flush = [&]() {
#pragma unroll
         for (uint32_t q = 0; q < 32; ++q) {  // unrolled: the byte counters stay in registers
            uint32_t c = k.count(q);
            c += __shfl_xor_sync(0xFFFFFFFFu, c, 8);
            c += __shfl_xor_sync(0xFFFFFFFFu, c, 16);
            const uint32_t slot = 256 * pass + 32 * w + q;
            if (g == 0 && w < wp && c && slot < nq)
               atomicAdd(counts + static_cast<size_t>(lists[slot]) * per_query + static_cast<size_t>(s) * L + p, c);
         }
         k.clear();
      };
      auto window = [&](uint32_t x, uint32_t cnt, uint32_t rowbase) {
         count_window_bits(k, x, cnt, rowbase, Rp, wp, lane);
         if (k.blocks == 255) flush();
      };
      while (have) {
         const uint32_t j = __ffs(have) - 1;
         have &= have - 1;
         const uint32_t ci = __shfl_sync(0xFFFFFFFFu, idx, j);
         const uint4 raw = __ldg(reinterpret_cast<const uint4*>(ctrs) + ci);
         const CtrDesc d = *reinterpret_cast<const CtrDesc*>(&raw);
         const uint32_t rowbase = (v0 + j) * CHUNK_ROWS;
         if (d.type == CT_ARRAY) {
            const uint32_t n = d.card_m1 + 1u;
            const uint16_t* a = payload + d.payload;
            // container payloads stream through once: read them evict-first so that the masks the
            // gathers reuse stay in L2
            for (uint32_t base = 0; base < n; base += 32) {
               const uint32_t x = base + lane < n ? __ldcs(a + base + lane) : 0u;
               window(x, n - base < 32 ? n - base : 32u, rowbase);
            }
         } else if (d.type == CT_BITSET) {
            const uint32_t* bits = reinterpret_cast<const uint32_t*>(payload + d.payload);
            for (uint32_t wb = 0; wb < CHUNK_WORDS; wb += 32) {
               uint32_t x = __ldcs(bits + wb + lane);
               const uint32_t c = __popc(x);
               uint32_t incl = c;
#pragma unroll
               for (uint32_t o = 1; o < 32; o <<= 1) {
                  const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                  if (lane >= o) incl += y;
               }
               const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
               uint32_t at = incl - c;
               while (x) {
                  const uint32_t b = __ffs(x) - 1;
                  x &= x - 1;
                  wl[at++] = static_cast<uint16_t>(32 * (wb + lane) + b);
               }
               __syncwarp();
               for (uint32_t base = 0; base < total; base += 32) {
                  const uint32_t y = base + lane < total ? wl[base + lane] : 0u;
                  window(y, total - base < 32 ? total - base : 32u, rowbase);
               }
               __syncwarp();
            }
         } else {
            const uint16_t* r = payload + d.payload;
            for (uint32_t i = 0; i < d.nruns; ++i) {
               const uint32_t s0 = __ldg(r + 2 * i), n = __ldg(r + 2 * i + 1) + 1u;
               for (uint32_t base = 0; base < n; base += 32) window(s0 + base + lane, n - base < 32 ? n - base : 32u, rowbase);
            }
         }
      }
      if (k.blocks) flush();
   }
}

// One CTA per event item and pass of up to 32 query groups (blockIdx.y). A sub-warp of gsz lanes,
// one lane per query group, streams a contiguous slice of the item's position-sorted events: each
// lane gathers its group's mask of the event's row and counts its 16 queries; when the position
// changes it adds the nonzero counts to the query's difference array (missing events: +1 start,
// -1 end) or boundary histogram (coverage events), and once per segment to the segment totals.
// Events are read once for all groups of the pass.
__global__ void __launch_bounds__(BT, 3) mut_cov_batch_kernel(const DevTable* __restrict__ tab, uint32_t col,
                                                              const EvItem* __restrict__ items,
                                                              const uint16_t* __restrict__ R,
                                                              const uint32_t* __restrict__ lists, uint32_t nq_max,
                                                              uint32_t* __restrict__ scratch) {
   const uint32_t nq = lists[2 * nq_max];  // dense slots: lists[0 .. nq)
   if (blockIdx.y * 32 * MUT_GROUP >= nq) return;
   const DevSeqCol* cs = &tab->seq[col];
   const uint32_t L = cs->L, nseg = mut_nseg(L);
   const size_t per_query = mut_scratch_words(L);
   const uint32_t ngroups = (nq + MUT_GROUP - 1) / MUT_GROUP, nqc = (nq + 31) / 32;
   const uint32_t gpass = blockIdx.y * 32;
   const uint32_t gleft = ngroups - gpass;
   uint32_t gsz = 1;
   while (gsz < gleft && gsz < 32) gsz <<= 1;
   const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
   const uint32_t g = gpass + (lane & (gsz - 1));
   const bool gvalid = g < ngroups;
   const uint32_t spw = 32 / gsz;
   const uint32_t nsub = (blockDim.x >> 5) * spw, sub = warp * spw + lane / gsz;
   const size_t rows = static_cast<size_t>(tab->nchunks) * CHUNK_ROWS;
   const uint32_t mpass = g / PASS_GROUPS;
   const uint32_t stride = gvalid ? 2 * pass_width_u32(nqc, mpass) : 0u;
   const uint16_t* Rg = R + static_cast<size_t>(mpass) * rows * 16 + g % PASS_GROUPS;
   const EvItem it = items[blockIdx.x];
   const uint32_t n = it.end - it.begin;
   const uint32_t s0 = it.begin + static_cast<uint32_t>(static_cast<uint64_t>(n) * sub / nsub);
   const uint32_t s1 = it.begin + static_cast<uint32_t>(static_cast<uint64_t>(n) * (sub + 1) / nsub);

   const bool missing = it.list <= EV_MEND;
   const uint32_t* mev = it.list == EV_MSTART ? cs->mstart : cs->mend;
   const uint2* cev = reinterpret_cast<const uint2*>(it.list == EV_CSTART ? cs->cstart : cs->cend);
   const uint32_t pbase = missing ? it.block * NBLOCK : 0u;
   const uint32_t hist = missing ? 2 * (L + 1) : (it.list == EV_CSTART ? 0u : L + 1);
   const uint32_t segb = 3 * (L + 1) + (missing ? 2 * nseg : (it.list == EV_CSTART ? 0u : nseg));
   const uint32_t sign = it.list == EV_MEND ? 0xFFFFFFFFu : 1u;  // multiplier modulo 2^32
   // scratch of query q of this lane's group: that dense slot's
   auto sc_of = [&](uint32_t q) { return scratch + static_cast<size_t>(lists[MUT_GROUP * g + q]) * per_query; };

   NibbleCounter k;
   k.clear();
   uint32_t seg[MUT_GROUP];
#pragma unroll
   for (uint32_t q = 0; q < MUT_GROUP; ++q) seg[q] = 0;
   constexpr uint32_t NONE = 0xFFFFFFFEu, INVALID = 0xFFFFFFFFu;
   uint32_t cur = NONE, curseg = NONE;

   auto flush_seg = [&]() {
      if (curseg == NONE) return;
#pragma unroll
      for (uint32_t q = 0; q < MUT_GROUP; ++q) {
         if (seg[q] && MUT_GROUP * g + q < nq) atomicAdd(sc_of(q) + segb + curseg, seg[q] * sign);
         seg[q] = 0;
      }
   };
   auto flush_pos = [&]() {
      k.drain();
      if (cur != NONE && cur <= L) {
#pragma unroll
         for (uint32_t q = 0; q < MUT_GROUP; ++q) {
            if (k.c[q] && MUT_GROUP * g + q < nq) atomicAdd(sc_of(q) + hist + cur, k.c[q] * sign);
            seg[q] += k.c[q];
         }
      }
#pragma unroll
      for (uint32_t q = 0; q < MUT_GROUP; ++q) k.c[q] = 0;
   };
   auto move_to = [&](uint32_t p) {
      flush_pos();
      cur = p;
      if (p / MUT_SEG != curseg) {
         flush_seg();
         curseg = p / MUT_SEG;
      }
   };

   constexpr uint32_t U = 4;  // events in flight per lane
   for (uint32_t i = s0; i < s1; i += U) {
      uint32_t row[U], pos[U], m[U];
#pragma unroll
      for (uint32_t u = 0; u < U; ++u) {
         row[u] = 0;
         pos[u] = INVALID;
         if (i + u < s1) {
            if (missing) {
               const uint32_t e = __ldg(mev + i + u);
               row[u] = e >> 8;
               pos[u] = pbase + (e & 0xFFu);
            } else {
               const uint2 e = __ldg(cev + i + u);
               row[u] = e.x;
               pos[u] = e.y;
            }
         }
      }
#pragma unroll
      for (uint32_t u = 0; u < U; ++u)
         m[u] = (pos[u] != INVALID && gvalid) ? __ldg(Rg + static_cast<size_t>(row[u]) * stride) : 0u;
#pragma unroll
      for (uint32_t u = 0; u < U; u += 2) {
         if (pos[u] == cur && pos[u + 1] == cur) {
            k.add(__byte_perm(m[u], m[u + 1], 0x5410));
         } else {
#pragma unroll
            for (uint32_t x = u; x < u + 2; ++x) {
               if (pos[x] == INVALID) continue;
               if (pos[x] != cur) move_to(pos[x]);
               k.add(m[x]);
            }
         }
      }
   }
   flush_pos();
   flush_seg();
}

// One CTA: the dense slot list, the sparse slot list and their lengths, in slot order.
__global__ void __launch_bounds__(1024) mut_select_kernel(const unsigned long long* __restrict__ fcounts,
                                                          const uint32_t* __restrict__ slot_query, uint32_t nq,
                                                          unsigned long long sparse_max, uint32_t* __restrict__ lists) {
   __shared__ uint32_t wd[32], wsp[32];
   const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
   uint32_t nd = 0, ns = 0;  // the same in every thread
   for (uint32_t q0 = 0; q0 < nq; q0 += blockDim.x) {
      const uint32_t q = q0 + threadIdx.x;
      const unsigned long long fc = q < nq ? fcounts[slot_query[q]] : 0ull;
      const bool dense = fc > sparse_max, sparse = fc > 0 && fc <= sparse_max;
      const uint32_t bd = __ballot_sync(0xFFFFFFFFu, dense), bs = __ballot_sync(0xFFFFFFFFu, sparse);
      if (lane == 0) {
         wd[warp] = __popc(bd);
         wsp[warp] = __popc(bs);
      }
      __syncthreads();
      uint32_t pd = 0, ps = 0, td = 0, ts = 0;
      for (uint32_t w = 0; w < nw; ++w) {
         pd += w < warp ? wd[w] : 0u;
         ps += w < warp ? wsp[w] : 0u;
         td += wd[w];
         ts += wsp[w];
      }
      const uint32_t below = (1u << lane) - 1u;
      if (dense) lists[nd + pd + __popc(bd & below)] = q;
      if (sparse) lists[nq + ns + ps + __popc(bs & below)] = q;
      nd += td;
      ns += ts;
      __syncthreads();
   }
   if (threadIdx.x == 0) {
      lists[2 * nq] = nd;
      lists[2 * nq + 1] = ns;
   }
}

// grid (CTAs per slot, nq): the row-index pass of sparse slot blockIdx.y, if there is one.
__global__ void __launch_bounds__(BT) mut_sparse_batch_kernel(const DevTable* __restrict__ tab, uint32_t col,
                                                              const uint32_t* __restrict__ filters,
                                                              const uint32_t* __restrict__ lists, uint32_t nq,
                                                              uint32_t* counts, uint32_t* scratch) {
   __shared__ uint32_t list[BT / 32][1024];
   if (blockIdx.y >= lists[2 * nq + 1]) return;
   const uint32_t slot = lists[nq + blockIdx.y];
   const DevSeqCol* cs = &tab->seq[col];
   const uint32_t words = tab->nchunks * CHUNK_WORDS;
   const uint32_t warp = threadIdx.x >> 5, nwarps = gridDim.x * (BT / 32);
   const uint32_t* F = filters + static_cast<size_t>(slot) * words;
   uint32_t* cnt = counts + static_cast<size_t>(slot) * cs->nsym * cs->L;
   uint32_t* sc = scratch + static_cast<size_t>(slot) * mut_scratch_words(cs->L);
   for (uint32_t w = (blockIdx.x * (BT / 32) + warp) * 32; w < words; w += nwarps * 32)
      row_index_pass32(cs, F, w, words, cnt, sc, list[warp]);
}

// grid (ceil(L / MUT_SEG), nq): reference counts of slot blockIdx.y. With rowblk (the Mutations
// rows are wanted), the CTA then counts the output rows of its MUT_SEG (= ROWS_BLOCK) positions
// under the slot's minimum proportion into rowblk[slot * gridDim.x + blockIdx.x], the entry
// rows_count_kernel would write, from the counts its threads just completed.
__global__ void __launch_bounds__(MUT_SEG) mut_final_batch_kernel(const DevTable* __restrict__ tab, uint32_t col,
                                                                  const unsigned long long* __restrict__ fcounts,
                                                                  const uint32_t* __restrict__ slot_query,
                                                                  uint32_t* __restrict__ counts,
                                                                  const uint32_t* __restrict__ scratch,
                                                                  const double* __restrict__ min_prop,
                                                                  uint32_t* __restrict__ rowblk) {
   static_assert(MUT_SEG == ROWS_BLOCK, "a final CTA covers one block of the row counts");
   __shared__ uint32_t red[MUT_SEG / 32];
   const DevSeqCol* cs = &tab->seq[col];
   const uint32_t q = blockIdx.y, L = cs->L;
   const uint32_t total = static_cast<uint32_t>(fcounts[slot_query[q]]);
   if (total == 0) {  // an empty filter: its counts stay zero and it has no rows
      if (rowblk != nullptr && threadIdx.x == 0) rowblk[static_cast<size_t>(q) * gridDim.x + blockIdx.x] = 0;
      return;
   }
   uint32_t* c = counts + static_cast<size_t>(q) * cs->nsym * L;
   final_position_counts(cs, total, c, scratch + static_cast<size_t>(q) * mut_scratch_words(L), red);
   if (rowblk == nullptr) return;
   // each thread reads back its own position's counts (plain loads: it has just written one)
   const uint32_t p = blockIdx.x * MUT_SEG + threadIdx.x;
   const uint32_t n =
      p < L ? position_rows(cs, p, min_prop[q], [&](uint32_t s) { return c[static_cast<size_t>(s) * L + p]; }).n : 0u;
   const uint32_t wn = __reduce_add_sync(0xFFFFFFFFu, n);
   __syncthreads();  // red is free again (final_position_counts' scans are done)
   if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = wn;
   __syncthreads();
   if (threadIdx.x == 0) {
      uint32_t sum = 0;
      for (uint32_t w = 0; w < MUT_SEG / 32; ++w) sum += red[w];
      rowblk[static_cast<size_t>(q) * gridDim.x + blockIdx.x] = sum;
   }
}

}  // namespace

size_t mutations_batch_mask_bytes(uint32_t nq, uint32_t nchunks) {
   const uint32_t nqc = (nq + 31) / 32;
   return static_cast<size_t>(nqc) * nchunks * CHUNK_ROWS * 4;
}

void launch_mutations_batch(const DevTable* d_table, const DevSeqCol& col_host, uint32_t col, uint32_t nchunks,
                            const uint32_t* d_filters, uint32_t nq, const unsigned long long* d_fcounts,
                            const uint32_t* d_slot_query, const EvItem* d_ev, uint32_t n_ev, const CtrUnit* d_units,
                            uint32_t n_units, uint16_t* d_masks, uint32_t* d_counts, uint32_t* d_scratch,
                            uint32_t* d_lists, uint64_t sparse_max, void* stream, uint32_t parts,
                            const double* d_min_prop, uint32_t* d_rowblk) {
   if (nq == 0) return;
   cudaStream_t s = static_cast<cudaStream_t>(stream);
   const uint32_t ngroups = (nq + MUT_GROUP - 1) / MUT_GROUP;  // grids for the largest dense list
   // the slot lists are made with the transpose part, which every timed part follows; the split
   // does not depend on which parts run (without the row-index part its slots stay uncounted)
   if (parts & BMUT_PART_TRANSPOSE) {
      mut_select_kernel<<<1, 1024, 0, s>>>(d_fcounts, d_slot_query, nq, static_cast<unsigned long long>(sparse_max),
                                           d_lists);
      transpose_kernel<<<nchunks * CHUNK_WORDS / TR_WORDS, BT, 0, s>>>(d_filters, d_lists, nq, nchunks,
                                                                       reinterpret_cast<uint32_t*>(d_masks));
   }
   if ((parts & BMUT_PART_CTR) && n_units > 0) {
      const dim3 grid((n_units + BT / 32 - 1) / (BT / 32), (ngroups + PASS_GROUPS - 1) / PASS_GROUPS);
      mut_ctr_batch_kernel<<<grid, BT, 0, s>>>(d_table, col, d_units, n_units, d_masks, d_lists, nq, d_counts);
   }
   if ((parts & BMUT_PART_COV) && n_ev > 0)
      mut_cov_batch_kernel<<<dim3(n_ev, (ngroups + 31) / 32), BT, 0, s>>>(d_table, col, d_ev, d_masks, d_lists, nq,
                                                                          d_scratch);
   if ((parts & BMUT_PART_SPARSE) && sparse_max > 0) {
      const uint32_t per_slot = std::max(1u, std::min(nchunks * CHUNK_WORDS / 32 / (BT / 32), 64u));
      mut_sparse_batch_kernel<<<dim3(per_slot, nq), BT, 0, s>>>(d_table, col, d_filters, d_lists, nq, d_counts,
                                                                d_scratch);
   }
   if (parts & BMUT_PART_FINAL) {
      dim3 fin((col_host.L + MUT_SEG - 1) / MUT_SEG, nq);
      mut_final_batch_kernel<<<fin, MUT_SEG, 0, s>>>(d_table, col, d_fcounts, d_slot_query, d_counts, d_scratch,
                                                     d_min_prop, d_rowblk);
   }
}

}  // namespace rhygpu
