// sm_103a kernels of the filter and Count path (the Mutations kernels are in mutations.cu and
// batch.cu, the output rows in rows.cu, Details in details.cu).
//
//  filter_kernel        one CTA per (chunk, tile of W rows): runs the postorder filter program over a
//                       stack of W-bit tiles in shared memory; leaves expand array / bitset / run
//                       containers straight into shared memory; writes the row-set tile and/or adds
//                       its popcount (Count action, reference: copy_on_write_bitmap.cpp:108-118).
//                       With a trace buffer it records every instruction's cycles and result size
//                       (planner training).
//  filter_batch_kernel  persistent variant: CTAs pull (query, tile) work items from a counter.
// All arithmetic is integer; results are bit-exact with the CPU operators.
#include <cuda_runtime.h>

#include <stdexcept>
#include <string>

#include "device.h"

namespace rhygpu {

namespace {

constexpr uint32_t FT = 256;  // threads per filter CTA

__device__ __forceinline__ uint32_t valid_word(uint32_t w, uint32_t nvalid) {
   const uint32_t b = w * 32;
   if (b + 32 <= nvalid) return 0xFFFFFFFFu;
   if (b >= nvalid) return 0u;
   return (1u << (nvalid - b)) - 1u;
}

// Sets bits [a, b) of a shared-memory tile.
__device__ __forceinline__ void set_range(uint32_t* t, uint32_t a, uint32_t b) {
   if (a >= b) return;
   const uint32_t wa = a >> 5, wb = (b - 1) >> 5;
   for (uint32_t w = wa; w <= wb; ++w) {
      uint32_t m = 0xFFFFFFFFu;
      if (w == wa) m &= 0xFFFFFFFFu << (a & 31);
      if (w == wb) m &= 0xFFFFFFFFu >> (31 - ((b - 1) & 31));
      atomicOr(&t[w], m);
   }
}

// ORs the rows of one container that fall in [row0, row0 + W) into tile t.
__device__ __forceinline__ void or_container(uint32_t* t, const CtrDesc& d, const uint16_t* __restrict__ payload,
                                             uint32_t row0, uint32_t W) {
   const uint16_t* p = payload + d.payload;
   if (d.type == CT_ARRAY) {
      const uint32_t card = d.card_m1 + 1u;
      for (uint32_t i = threadIdx.x; i < card; i += blockDim.x) {
         const uint32_t r = static_cast<uint32_t>(__ldg(p + i)) - row0;
         if (r < W) atomicOr(&t[r >> 5], 1u << (r & 31));
      }
   } else if (d.type == CT_BITSET) {
      const uint4* b = reinterpret_cast<const uint4*>(p) + (row0 >> 7);
      for (uint32_t i = threadIdx.x; i < (W >> 7); i += blockDim.x) {
         const uint4 x = __ldg(b + i);
         if (x.x) atomicOr(&t[4 * i + 0], x.x);
         if (x.y) atomicOr(&t[4 * i + 1], x.y);
         if (x.z) atomicOr(&t[4 * i + 2], x.z);
         if (x.w) atomicOr(&t[4 * i + 3], x.w);
      }
   } else {
      for (uint32_t i = threadIdx.x; i < d.nruns; i += blockDim.x) {
         const uint32_t s = __ldg(p + 2 * i);
         const uint32_t e = s + __ldg(p + 2 * i + 1) + 1u;  // run covers [s, e)
         const uint32_t a = max(s, row0), b = min(e, row0 + W);
         if (a < b) set_range(t, a - row0, b - row0);
      }
   }
}

struct TileCtx {
   const DevTable* __restrict__ tab;
   uint32_t v;
   uint32_t row0;
   uint32_t W;
   uint32_t nvalid;
   const uint32_t* aux;  // the query's precomputed row sets (PUSH_AUX), nchunks * CHUNK_WORDS words each
};

// Per-item staging of the program's leaves for the chunk and row range of the current tile:
//  - container leaves (PUSH_SCAN / PUSH_DICT, c = ordinal + 1): the slot offsets of all leaves are
//    read in one round of loads and their descriptors in a second, so a leaf then costs one round
//    trip (its payload) instead of three;
//  - coverage leaves (PUSH_COVERED, c = ordinal + 1): the tile's ranges of coverage exceptions and
//    missing intervals.
// Array payloads of at most LC_SMALL rows are copied into shared memory by TMA bulk copies; every
// other staged payload and range is handed to the TMA engine as a bulk L2 prefetch, so the leaves
// find their data in L2 when the program reaches them.
constexpr uint32_t LC_LEAVES = 128;
constexpr uint32_t LC_DESCS = 256;
constexpr uint32_t LC_COV = 64;
constexpr uint32_t LC_NONE = 0xFFFFFFFFu;
constexpr uint32_t LC_PAY = 2048;   // u16 of small-array payloads copied into shared memory per item
constexpr uint32_t LC_SMALL = 64;   // arrays up to this cardinality are copied
constexpr uint16_t LC_NOPAY = 0xFFFF;
constexpr uint32_t LC_BIG = 0x80000000u;
constexpr uint32_t LC_OWNER_MAX = 256;  // leaves of at most this many copied rows are set by their words' owners

struct LeafCache {
   uint4 desc[LC_DESCS];
   uint4 pay4[LC_PAY / 8];   // small-array payloads (TMA bulk copies, 16-byte aligned runs)
   uint16_t poff[LC_DESCS];  // descriptor i's first element: u16 offset into pay4 (below LC_PAY), or
                             // LC_PAY + offset into ext; LC_NOPAY when not copied
   uint8_t dleaf[LC_DESCS];  // leaf (0-based) of staged descriptor i
   uint32_t nstaged;         // staged descriptors: the staged leaves are a prefix of the leaves
   uint32_t pay_used;        // u16 of pay4 reserved by this item's copies
   uint16_t* ext;            // the stack tiles the item's program leaves free (16-byte aligned)
   uint32_t ext_cap;         // their size in u16
   uint32_t ext_used;        // u16 of ext reserved by this item's copies
   uint64_t bar;             // completes the item's payload copies
   const uint4* src[LC_LEAVES];
   const uint16_t* pay[LC_LEAVES];
   uint32_t n[LC_LEAVES];
   uint32_t symmask[LC_LEAVES];  // symbols the leaf ORs (every container for dictionary leaves)
   uint32_t match[LC_LEAVES];    // staged leaves of at most 32 descriptors: bit i = descriptor i matches
   uint32_t tot[LC_LEAVES];      // rows of the leaf's matching containers copied into shared memory;
                                 // LC_BIG set when a matching container was not copied
   uint32_t beg[LC_LEAVES];  // LC_NONE: not staged (the leaf reads its descriptors from global memory)
   uint4 cov[LC_COV];        // exception range (x, y) and missing-interval range (z, w) of the tile
   uint32_t nl;              // container leaves 1..nl are described by the table
   uint32_t ncov;            // coverage leaves 1..ncov
};

// Bulk prefetch of global bytes [a, b) into L2; a is rounded down and b up to 16 bytes, so the
// caller guarantees the rounded range stays inside the allocation.
__device__ __forceinline__ void prefetch_l2(const void* a, const void* b) {
   const uintptr_t s = reinterpret_cast<uintptr_t>(a) & ~static_cast<uintptr_t>(15);
   const uintptr_t e = (reinterpret_cast<uintptr_t>(b) + 15) & ~static_cast<uintptr_t>(15);
   if (e <= s) return;
   const uint32_t n = static_cast<uint32_t>(min(e - s, static_cast<uintptr_t>(32768)));
   asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(s), "r"(n) : "memory");
}

// Once per CTA, before the first item: the barrier of the payload copies.
__device__ __forceinline__ void init_leaves(LeafCache& lc) {
   if (threadIdx.x == 0) {
      const uint32_t b = static_cast<uint32_t>(__cvta_generic_to_shared(&lc.bar));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b));
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
   }
}

// Clears the leaf tables for nl container and ncov coverage leaves; a barrier must follow.
__device__ __forceinline__ void clear_leaves(LeafCache& lc, uint32_t nl, uint32_t ncov, uint16_t* ext = nullptr,
                                             uint32_t ext_cap = 0) {
   if (threadIdx.x == 0) {
      lc.nl = nl;
      lc.ncov = ncov;
      lc.pay_used = 0;
      lc.ext = ext;
      lc.ext_cap = ext ? ext_cap : 0u;
      lc.ext_used = 0;
   }
   for (uint32_t k = threadIdx.x; k < nl; k += blockDim.x) {
      lc.n[k] = 0;
      lc.src[k] = nullptr;
      lc.match[k] = 0;
      lc.tot[k] = 0;
   }
   for (uint32_t k = threadIdx.x; k < ncov; k += blockDim.x) lc.cov[k] = make_uint4(0, 0, 0, 0);
}

// The tile's ranges in the coverage exceptions of chunk v and in the missing-interval bucket of
// position pos (both lists are sorted by row; TOFF_ROWS divides every tile boundary).
__device__ __forceinline__ uint4 cover_ranges(const DevTable* __restrict__ tab, const DevSeqCol* __restrict__ col,
                                              uint32_t v, uint32_t row0, uint32_t W, uint32_t pos) {
   const uint32_t k0 = row0 / TOFF_ROWS, k1 = (row0 + W) / TOFF_ROWS;
   const uint32_t* xo = col->exc_toff + static_cast<size_t>(v) * TOFF_N;
   const uint32_t* no = col->nblk_toff + (static_cast<size_t>(pos / NBLOCK) * tab->nchunks + v) * TOFF_N;
   return make_uint4(__ldg(xo + k0), __ldg(xo + k1), __ldg(no + k0), __ldg(no + k1));
}

// Testing the failure path of the bounded waits: while set (on the current device), the threads that
// stage leaf payloads announce their bytes on the item's barrier but never issue the bulk copies,
// so the item's wait gives up (after 1 ms) and the kernel sets error 6 (DEVERR_WAIT_FILTER). No
// copy is left in flight: the withheld copies never start. Off by default; set only through
// set_copy_withholding.
__device__ uint32_t g_withhold_leaf_copies = 0;

// Waits for phase `parity` of the copies' barrier, bounded by `limit_ns` on the GPU's global timer
// (2 s: a copy lands in microseconds) and, as a second bound, by 2^26 polls of at most about 1 us
// each; false if it gave up.
__device__ __forceinline__ bool wait_copies(LeafCache& lc, uint32_t parity, uint64_t limit_ns) {
   const uint32_t b = static_cast<uint32_t>(__cvta_generic_to_shared(&lc.bar));
   uint64_t t0 = 0;
   for (uint32_t i = 0; i < (1u << 26); ++i) {
      uint32_t done;
      asm volatile(
         "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
         : "=r"(done)
         : "r"(b), "r"(parity), "r"(1000u)
         : "memory");
      if (done) return true;
      uint64_t now;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
      if (t0 == 0) t0 = now;
      else if (now - t0 > limit_ns) return false;
   }
   return false;
}

// Stages the item's leaves (see LeafCache). Array containers of at most LC_SMALL rows are also
// copied into shared memory by TMA bulk copies: each issuing thread announces its bytes on the
// barrier (expect_tx) before starting its copy, and one thread arrives after every announcement,
// so the phase completes when the last copy lands. `phase` is the parity of this item's wait,
// flipped when copies were made. Returns false (error flag set) if the copies did not land.
__device__ bool stage_leaves(LeafCache& lc, const TileCtx& c, const Instr* __restrict__ code, uint32_t ncode,
                             uint32_t& phase, int* err) {
   const DevTable* __restrict__ tab = c.tab;
   const uint32_t nl = lc.nl, ncov = lc.ncov;
   const bool withhold = *static_cast<volatile uint32_t*>(&g_withhold_leaf_copies) != 0;
   // this thread's earlier shared-memory accesses (stack tiles, staged payloads of the previous
   // item) are ordered before the bulk copies into the same memory issued after the next barrier
   asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
   for (uint32_t i = threadIdx.x; i < ncode; i += blockDim.x) {
      const uint4 raw = __ldg(reinterpret_cast<const uint4*>(code) + i);
      const Instr in = *reinterpret_cast<const Instr*>(&raw);
      if (in.op == OP_PUSH_COVERED) {
         if (in.c == 0 || in.c > ncov) continue;
         const DevSeqCol* col = &tab->seq[in.col];
         const uint4 r = cover_ranges(tab, col, c.v, c.row0, c.W, in.a);
         lc.cov[in.c - 1] = r;
         prefetch_l2(col->exc + r.x, col->exc + r.y);
         prefetch_l2(col->nblk + r.z, col->nblk + (r.w & ~1u));  // stays inside the 8-byte-entry array
         continue;
      }
      if ((in.op != OP_PUSH_SCAN && in.op != OP_PUSH_DICT) || in.c == 0 || in.c > nl) continue;
      const CtrDesc* ctrs;
      const uint32_t* off;
      const uint16_t* payload;
      size_t slot;
      if (in.op == OP_PUSH_SCAN) {
         const DevSeqCol* col = &tab->seq[in.col];
         ctrs = col->ctrs;
         off = col->off;
         payload = col->payload;
         slot = static_cast<size_t>(c.v) * col->L + in.a;
      } else {
         const DevDictCol* col = &tab->dict[in.col];
         ctrs = col->ctrs;
         off = col->off;
         payload = col->payload;
         slot = static_cast<size_t>(c.v) * col->nkeys + in.a;
      }
      const uint32_t b = __ldg(off + slot), e = __ldg(off + slot + 1);
      lc.src[in.c - 1] = reinterpret_cast<const uint4*>(ctrs) + b;
      lc.pay[in.c - 1] = payload;
      lc.n[in.c - 1] = e - b;
      lc.symmask[in.c - 1] = in.op == OP_PUSH_SCAN ? in.b : 0xFFFFFFFFu;
   }
   __syncthreads();
   if (threadIdx.x < 32) {  // exclusive scan of the counts; leaves that do not fit stay unstaged
      const uint32_t lane = threadIdx.x;
      uint32_t carry = 0, staged = 0;
      for (uint32_t k0 = 0; k0 < nl; k0 += 32) {
         const uint32_t k = k0 + lane;
         const uint32_t x = k < nl ? lc.n[k] : 0u;
         uint32_t incl = x;
#pragma unroll
         for (uint32_t o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += y;
         }
         const uint32_t ex = carry + incl - x;
         const bool fits = x > 0 && ex + x <= LC_DESCS;  // the leaves that fit are a prefix of them
         if (k < nl) lc.beg[k] = fits ? ex : LC_NONE;
         if (fits) {
            for (uint32_t i = 0; i < x; ++i) lc.dleaf[ex + i] = static_cast<uint8_t>(k);
         }
         staged = max(staged, __reduce_max_sync(0xFFFFFFFFu, fits ? ex + x : 0u));
         carry += __shfl_sync(0xFFFFFFFFu, incl, 31);
      }
      if (lane == 0) lc.nstaged = staged;
   }
   __syncthreads();
   // one staged descriptor per thread: its load, and the copy or prefetch of its payload
   const uint32_t bar = static_cast<uint32_t>(__cvta_generic_to_shared(&lc.bar));
   for (uint32_t j = threadIdx.x; j < lc.nstaged; j += blockDim.x) {
      const uint32_t k = lc.dleaf[j];
      const uint4 raw = __ldg(lc.src[k] + (j - lc.beg[k]));
      lc.desc[j] = raw;
      lc.poff[j] = LC_NOPAY;
      const CtrDesc d = *reinterpret_cast<const CtrDesc*>(&raw);
      if (!((lc.symmask[k] >> d.sym) & 1u)) continue;  // a symbol the leaf does not OR: no payload
      if (lc.n[k] <= 32) atomicOr(&lc.match[k], 1u << (j - lc.beg[k]));
      // the arena ends with 16 spare bytes, so rounding the end up stays inside it
      const uint16_t* p = lc.pay[k] + d.payload;
      if (d.type == CT_ARRAY) {  // small arrays into pay4, any array into the free stack tiles
         const uintptr_t a = reinterpret_cast<uintptr_t>(p);
         const uintptr_t a0 = a & ~static_cast<uintptr_t>(15);
         const uint32_t bytes = static_cast<uint32_t>(((a + 2u * (d.card_m1 + 1u) + 15) & ~static_cast<uintptr_t>(15)) - a0);
         uint32_t dst = 0, po = LC_NOPAY;
         if (d.card_m1 < LC_SMALL) {
            const uint32_t at = atomicAdd(&lc.pay_used, bytes / 2);
            if (at + bytes / 2 <= LC_PAY) {
               po = at + static_cast<uint32_t>(a - a0) / 2;
               dst = static_cast<uint32_t>(__cvta_generic_to_shared(lc.pay4)) + 2 * at;
            }
         }
         if (po == LC_NOPAY && lc.ext_cap) {
            const uint32_t at = atomicAdd(&lc.ext_used, bytes / 2);
            if (at + bytes / 2 <= lc.ext_cap) {
               po = LC_PAY + at + static_cast<uint32_t>(a - a0) / 2;
               dst = static_cast<uint32_t>(__cvta_generic_to_shared(lc.ext)) + 2 * at;
            }
         }
         if (po != LC_NOPAY) {
            lc.poff[j] = static_cast<uint16_t>(po);
            atomicAdd(&lc.tot[k], d.card_m1 + 1u);
            asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
            if (!withhold)
               asm volatile(
                  "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                  "l"(a0), "r"(bytes), "r"(bar)
                  : "memory");
            continue;
         }
      }
      atomicOr(&lc.tot[k], LC_BIG);
      if (d.type == CT_ARRAY) prefetch_l2(p, p + d.card_m1 + 1u);
      else if (d.type == CT_BITSET) prefetch_l2(p + (c.row0 >> 4), p + ((c.row0 + c.W) >> 4));
      else prefetch_l2(p, p + 2u * d.nruns);
   }
   __syncthreads();
   if (lc.pay_used == 0 && lc.ext_used == 0) return true;  // no copies this item
   if (threadIdx.x == 0)
      asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(bar) : "memory");
   const uint64_t limit = withhold ? 1000000ull : 2000000000ull;
   bool ok = wait_copies(lc, phase, limit);
   if (!ok) ok = wait_copies(lc, phase, limit);  // once more before giving up with copies possibly in flight
   phase ^= 1u;
   if (!__syncthreads_and(ok)) {
      if (threadIdx.x == 0) atomicExch(err, 6);
      return false;
   }
   return true;
}

// OR of the containers of one slot whose symbol is in `mask` (all of them when !use_mask), from
// the staged descriptors when the leaf was staged.
__device__ void push_containers(uint32_t* t, const TileCtx& c, const CtrDesc* __restrict__ ctrs,
                                const uint16_t* __restrict__ payload, const uint32_t* __restrict__ off, size_t slot,
                                uint32_t mask, bool use_mask, const LeafCache& lc, uint32_t leaf) {
   const uint4* src;
   uint32_t n;
   if (leaf >= 1 && leaf <= lc.nl && lc.beg[leaf - 1] != LC_NONE) {
      src = lc.desc + lc.beg[leaf - 1];
      n = lc.n[leaf - 1];
   } else {
      const uint32_t b = __ldg(off + slot), e = __ldg(off + slot + 1);
      src = reinterpret_cast<const uint4*>(ctrs) + b;
      n = e - b;
   }
   const bool staged = leaf >= 1 && leaf <= lc.nl && lc.beg[leaf - 1] != LC_NONE;
   // staged leaves of at most 32 descriptors visit only the matching ones
   uint32_t todo = staged && n <= 32 ? lc.match[leaf - 1] : 0u;
   const bool listed = staged && n <= 32;
   for (uint32_t i = 0; listed ? todo != 0u : i < n; ++i) {
      if (listed) {
         i = __ffs(todo) - 1;
         todo &= todo - 1;
      }
      const uint4 raw = src[i];
      const CtrDesc d = *reinterpret_cast<const CtrDesc*>(&raw);
      if (use_mask && !((mask >> d.sym) & 1u)) continue;
      const uint16_t po = staged ? lc.poff[lc.beg[leaf - 1] + i] : LC_NOPAY;
      if (po != LC_NOPAY) {  // array copied into shared memory with the item's leaves
         const uint16_t* sp = po < LC_PAY ? reinterpret_cast<const uint16_t*>(lc.pay4) + po : lc.ext + (po - LC_PAY);
         const uint32_t card = d.card_m1 + 1u;
         for (uint32_t k = threadIdx.x; k < card; k += blockDim.x) {
            const uint32_t r = static_cast<uint32_t>(sp[k]) - c.row0;
            if (r < c.W) atomicOr(&t[r >> 5], 1u << (r & 31));
         }
      } else {
         or_container(t, d, payload, c.row0, c.W);
      }
   }
}

// A staged leaf of at most 32 descriptors whose matching containers are arrays copied into shared
// memory, LC_OWNER_MAX rows at most: set by the owners of its words (see below), with no CTA
// barrier. Each thread clears the words it owns; each warp then reads every row of the leaf and sets
// those in the words its lanes own (shared-memory atomics: two lanes may hit one word), fenced by
// __syncwarp on both sides. Returns false (nothing done) for any other leaf.
__device__ __forceinline__ bool push_owned(uint4* t4, uint32_t* t, const TileCtx& c, const LeafCache& lc, uint32_t leaf) {
   if (leaf < 1 || leaf > lc.nl) return false;
   const uint32_t k = leaf - 1;
   if (lc.beg[k] == LC_NONE || lc.n[k] > 32 || lc.tot[k] > LC_OWNER_MAX) return false;
   const uint32_t W4 = c.W >> 7, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
   for (uint32_t w4 = threadIdx.x; w4 < W4; w4 += blockDim.x) t4[w4] = make_uint4(0, 0, 0, 0);
   __syncwarp();
   uint32_t todo = lc.match[k];
   while (todo) {
      const uint32_t i = __ffs(todo) - 1;
      todo &= todo - 1;
      const uint32_t j = lc.beg[k] + i;
      const CtrDesc d = *reinterpret_cast<const CtrDesc*>(&lc.desc[j]);
      const uint16_t po = lc.poff[j];
      const uint16_t* sp = po < LC_PAY ? reinterpret_cast<const uint16_t*>(lc.pay4) + po : lc.ext + (po - LC_PAY);
      const uint32_t card = d.card_m1 + 1u;
      for (uint32_t e = lane; e < card; e += 32) {
         const uint32_t r = static_cast<uint32_t>(sp[e]) - c.row0;
         if (r < c.W && (((r >> 7) % FT) >> 5) == warp) atomicOr(&t[r >> 5], 1u << (r & 31));
      }
   }
   __syncwarp();
   return true;
}

// Word-parallel tile operations use one fixed mapping: thread i owns the uint4 words i, i +
// blockDim.x, ... of every tile. Consecutive word-parallel operations therefore need no barrier
// between them; leaves that scatter with shared-memory atomics (or write per warp) are fenced by
// barriers on both sides, except the small staged leaves that only their words' owning warps write
// (push_owned, fenced per warp).
__device__ __forceinline__ uint4 valid4(uint32_t w4, const TileCtx& c) {
   if (c.nvalid == c.W) return make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu);
   return make_uint4(valid_word(4 * w4, c.nvalid), valid_word(4 * w4 + 1, c.nvalid), valid_word(4 * w4 + 2, c.nvalid),
                     valid_word(4 * w4 + 3, c.nvalid));
}
__device__ __forceinline__ uint4 and4(uint4 a, uint4 b) { return make_uint4(a.x & b.x, a.y & b.y, a.z & b.z, a.w & b.w); }
__device__ __forceinline__ uint4 andnot4(uint4 a, uint4 b) {
   return make_uint4(a.x & ~b.x, a.y & ~b.y, a.z & ~b.z, a.w & ~b.w);
}
__device__ __forceinline__ uint4 or4(uint4 a, uint4 b) { return make_uint4(a.x | b.x, a.y | b.y, a.z | b.z, a.w | b.w); }
__device__ __forceinline__ bool any4(uint4 a) { return (a.x | a.y | a.z | a.w) != 0u; }
__device__ __forceinline__ bool ne4(uint4 a, uint4 b) {
   return ((a.x ^ b.x) | (a.y ^ b.y) | (a.z ^ b.z) | (a.w ^ b.w)) != 0u;
}
__device__ __forceinline__ uint32_t get4(const uint4& a, uint32_t i) { return i == 0 ? a.x : i == 1 ? a.y : i == 2 ? a.z : a.w; }

// Rows covered at pos (or not covered when `negate`): all valid rows minus the exceptions whose
// covered region misses pos and the rows with a missing interval over pos, within the tile's
// ranges r of both lists.
__device__ void push_covered(uint32_t* t, const TileCtx& c, const DevSeqCol* __restrict__ col, uint32_t pos, bool negate,
                             uint4 r) {
   const uint32_t W4 = c.W >> 7;
   uint4* t4 = reinterpret_cast<uint4*>(t);
   for (uint32_t w4 = threadIdx.x; w4 < W4; w4 += blockDim.x) t4[w4] = valid4(w4, c);
   __syncthreads();
   constexpr uint32_t U = 4;  // entries per thread in flight
   const uint4* exc = reinterpret_cast<const uint4*>(col->exc);
   for (uint32_t i0 = r.x + threadIdx.x; i0 < r.y; i0 += U * blockDim.x) {
      uint4 e[U];
#pragma unroll
      for (uint32_t u = 0; u < U; ++u) {
         const uint32_t i = i0 + u * blockDim.x;
         e[u] = i < r.y ? __ldg(exc + i) : make_uint4(c.row0, 0, 0xFFFFFFFFu, 0);
      }
#pragma unroll
      for (uint32_t u = 0; u < U; ++u) {
         const uint32_t row = e[u].x - c.row0;
         if (row < c.W && !(e[u].y <= pos && pos < e[u].z)) atomicAnd(&t[row >> 5], ~(1u << (row & 31)));
      }
   }
   const uint32_t q = pos % NBLOCK;
   const uint2* nb = reinterpret_cast<const uint2*>(col->nblk);
   for (uint32_t i0 = r.z + threadIdx.x; i0 < r.w; i0 += U * blockDim.x) {
      uint2 e[U];
#pragma unroll
      for (uint32_t u = 0; u < U; ++u) {
         const uint32_t i = i0 + u * blockDim.x;
         e[u] = i < r.w ? __ldg(nb + i) : make_uint2(0, 0);
      }
#pragma unroll
      for (uint32_t u = 0; u < U; ++u) {
         const uint32_t row = (e[u].x & 0xFFFFu) - c.row0;
         const uint32_t lo = e[u].y & 0xFFFFu, hi = e[u].y >> 16;
         if (row < c.W && lo <= q && q < hi) atomicAnd(&t[row >> 5], ~(1u << (row & 31)));
      }
   }
   __syncthreads();
   if (negate) {
      for (uint32_t w4 = threadIdx.x; w4 < W4; w4 += blockDim.x) t4[w4] = andnot4(valid4(w4, c), t4[w4]);
   }
}

// Rows whose date lies in [lo, hi] (outside it when `invert`); null dates match when `with_nulls`.
// Every comparison of the date predicates and the two-sided DateBetween reduce to this form. The
// bit-sliced index is compared against the clamped bounds from the top bit down (lo <= x keeps
// "greater" and "equal" masks, x <= hi "less" and "equal"); word-parallel in the fixed mapping.
__device__ void push_date(uint4* t4, const TileCtx& c, const DevDateCol* __restrict__ col, int32_t lo, int32_t hi,
                          bool invert, bool with_nulls) {
   const uint32_t W4 = c.W >> 7, nbits = col->nbits;
   const int64_t maxv = (int64_t{1} << nbits) - 1;
   const int64_t l = static_cast<int64_t>(lo) - col->base, h = static_cast<int64_t>(hi) - col->base;
   const bool empty = lo > hi || h < 0 || l > maxv;
   const uint32_t L = static_cast<uint32_t>(l < 0 ? 0 : l), H = static_cast<uint32_t>(h > maxv ? maxv : h);
   const size_t stride4 = static_cast<size_t>(c.tab->nchunks) * (CHUNK_WORDS / 4);
   const size_t base4 = (static_cast<size_t>(c.v) * CHUNK_WORDS + (c.row0 >> 5)) / 4;
   const uint4* planes = reinterpret_cast<const uint4*>(col->planes) + base4;
   const uint4* nulls = reinterpret_cast<const uint4*>(col->nulls) + base4;
   const uint4 ones = make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu);
   for (uint32_t w4 = threadIdx.x; w4 < W4; w4 += blockDim.x) {
      uint4 inside = make_uint4(0, 0, 0, 0);
      if (!empty) {
         uint4 eqL = ones, gtL = inside, eqH = ones, ltH = inside;
#pragma unroll 4
         for (int i = static_cast<int>(nbits) - 1; i >= 0; --i) {
            const uint4 x = __ldg(planes + static_cast<size_t>(i) * stride4 + w4);
            if ((L >> i) & 1u) {
               eqL = and4(eqL, x);
            } else {
               gtL = or4(gtL, and4(eqL, x));
               eqL = andnot4(eqL, x);
            }
            if ((H >> i) & 1u) {
               ltH = or4(ltH, andnot4(eqH, x));
               eqH = and4(eqH, x);
            } else {
               eqH = andnot4(eqH, x);
            }
         }
         inside = and4(or4(gtL, eqL), or4(ltH, eqH));
      }
      const uint4 nul = __ldg(nulls + w4);
      const uint4 m = invert ? andnot4(ones, inside) : inside;
      const uint4 res = with_nulls ? or4(andnot4(m, nul), nul) : andnot4(m, nul);
      t4[w4] = and4(res, valid4(w4, c));
   }
}

// Runs a filter program for one tile. The result is left in stack slot 0, complete for the thread
// that owns each uint4 word (see valid4); a barrier is needed before other threads read it.
// Returns false on a malformed program (the error flag is set).
// With `trace` (trace mode of the single-query kernel, for planner training) every executed
// instruction pc stores trace[2 pc] = its cycles (first thread, between barriers around the
// instruction) and trace[2 pc + 1] = the population count of the top of the stack after it.
__device__ bool run_program(const TileCtx& c, const Instr* __restrict__ code, uint32_t ncode, uint32_t* stk,
                            uint32_t cap, const LeafCache& lc, int* err, uint32_t* trace = nullptr) {
   __shared__ uint32_t tred[FT / 32];
   const uint32_t WW = c.W >> 5, W4 = c.W >> 7;
   uint4* stk4 = reinterpret_cast<uint4*>(stk);
   uint32_t sp = 0;
   uint32_t pc = 0;
   uint32_t steps = 0;
   bool synced = true;  // no word-parallel write since the last barrier
   while (pc < ncode) {
      if (++steps > 4u * MAX_PROGRAM) {  // jumps only go forward; this bounds a corrupted program
         if (threadIdx.x == 0) atomicExch(err, 3);
         return false;
      }
      long long t_start = 0;
      if (trace) {
         __syncthreads();
         t_start = clock64();
      }
      Instr in;
      {
         const uint4 raw = __ldg(reinterpret_cast<const uint4*>(code) + pc);
         in = *reinterpret_cast<const Instr*>(&raw);
      }
      uint32_t next = pc + 1;
      switch (in.op) {
         case OP_PUSH_EMPTY:
         case OP_PUSH_FULL:
         case OP_PUSH_SCAN:
         case OP_PUSH_NULLS:
         case OP_PUSH_DICT:
         case OP_PUSH_COVERED:
         case OP_PUSH_DATE:
         case OP_PUSH_AUX: {
            if (sp >= cap) {
               if (threadIdx.x == 0) atomicExch(err, 1);
               return false;
            }
            uint32_t* t = stk + sp * WW;
            uint4* t4 = stk4 + sp * W4;
            ++sp;
            if (in.op == OP_PUSH_FULL) {
               for (uint32_t w4 = threadIdx.x; w4 < W4; w4 += blockDim.x) t4[w4] = valid4(w4, c);
               synced = false;
            } else if (in.op == OP_PUSH_EMPTY) {
               for (uint32_t w4 = threadIdx.x; w4 < W4; w4 += blockDim.x) t4[w4] = make_uint4(0, 0, 0, 0);
               synced = false;
            } else if (in.op == OP_PUSH_NULLS) {
               const uint4* src = reinterpret_cast<const uint4*>(c.tab->seq[in.col].null_tiles +
                                                                 static_cast<size_t>(c.v) * CHUNK_WORDS + (c.row0 >> 5));
               for (uint32_t w4 = threadIdx.x; w4 < W4; w4 += blockDim.x) t4[w4] = __ldg(src + w4);
               synced = false;
            } else if (in.op == OP_PUSH_AUX) {
               if (c.aux == nullptr) {
                  if (threadIdx.x == 0) atomicExch(err, 5);
                  return false;
               }
               const uint4* src = reinterpret_cast<const uint4*>(
                  c.aux + static_cast<size_t>(in.a) * c.tab->nchunks * CHUNK_WORDS + static_cast<size_t>(c.v) * CHUNK_WORDS +
                  (c.row0 >> 5));
               for (uint32_t w4 = threadIdx.x; w4 < W4; w4 += blockDim.x) t4[w4] = __ldg(src + w4);
               synced = false;
            } else if (in.op == OP_PUSH_COVERED) {
               const DevSeqCol* col = &c.tab->seq[in.col];
               const uint4 r = (in.c >= 1 && in.c <= lc.ncov) ? lc.cov[in.c - 1]
                                                              : cover_ranges(c.tab, col, c.v, c.row0, c.W, in.a);
               push_covered(t, c, col, in.a, in.flags & 1, r);
               synced = !(in.flags & 1);
            } else if (in.op == OP_PUSH_DATE) {
               push_date(t4, c, &c.tab->date[in.col], static_cast<int32_t>(in.a), static_cast<int32_t>(in.b), in.flags & 2,
                         in.flags & 1);
               synced = false;
            } else if (push_owned(t4, t, c, lc, in.c)) {
               synced = false;
            } else {
               for (uint32_t w4 = threadIdx.x; w4 < W4; w4 += blockDim.x) t4[w4] = make_uint4(0, 0, 0, 0);
               __syncthreads();
               if (in.op == OP_PUSH_SCAN) {
                  const DevSeqCol* col = &c.tab->seq[in.col];
                  push_containers(t, c, col->ctrs, col->payload, col->off, static_cast<size_t>(c.v) * col->L + in.a, in.b,
                                  true, lc, in.c);
               } else {
                  const DevDictCol* col = &c.tab->dict[in.col];
                  push_containers(t, c, col->ctrs, col->payload, col->off, static_cast<size_t>(c.v) * col->nkeys + in.a, 0,
                                  false, lc, in.c);
               }
               __syncthreads();
               synced = true;
            }
            break;
         }
         case OP_AND:
         case OP_ANDNOT:
         case OP_OR: {
            if (sp < 2) {
               if (threadIdx.x == 0) atomicExch(err, 2);
               return false;
            }
            uint4* x = stk4 + (sp - 2) * W4;
            const uint4* y = stk4 + (sp - 1) * W4;
            if (in.op == OP_AND) {
               for (uint32_t w4 = threadIdx.x; w4 < W4; w4 += blockDim.x) x[w4] = and4(x[w4], y[w4]);
            } else if (in.op == OP_ANDNOT) {
               for (uint32_t w4 = threadIdx.x; w4 < W4; w4 += blockDim.x) x[w4] = andnot4(x[w4], y[w4]);
            } else {
               for (uint32_t w4 = threadIdx.x; w4 < W4; w4 += blockDim.x) x[w4] = or4(x[w4], y[w4]);
            }
            --sp;
            synced = false;
            break;
         }
         case OP_NOT: {
            if (sp < 1) {
               if (threadIdx.x == 0) atomicExch(err, 2);
               return false;
            }
            uint4* x = stk4 + (sp - 1) * W4;
            for (uint32_t w4 = threadIdx.x; w4 < W4; w4 += blockDim.x) x[w4] = andnot4(valid4(w4, c), x[w4]);
            synced = false;
            break;
         }
         case OP_THR_BEGIN: {
            if (sp + in.a > cap) {
               if (threadIdx.x == 0) atomicExch(err, 1);
               return false;
            }
            for (uint32_t i = 0; i < in.a; ++i)
               for (uint32_t w4 = threadIdx.x; w4 < W4; w4 += blockDim.x) stk4[(sp + i) * W4 + w4] = make_uint4(0, 0, 0, 0);
            sp += in.a;
            synced = false;
            break;
         }
         case OP_THR_ADD: {
            const uint32_t P = in.a;
            if (sp < P + 1) {
               if (threadIdx.x == 0) atomicExch(err, 2);
               return false;
            }
            const uint4* x4 = stk4 + (sp - 1) * W4;
            uint4* planes4 = stk4 + (sp - 1 - P) * W4;
            const bool neg = in.flags & 1;
            // ripple-carry add of one bit per row into the bit-sliced counter, four words at a time
            for (uint32_t w4 = threadIdx.x; w4 < W4; w4 += blockDim.x) {
               uint4 carry = neg ? andnot4(valid4(w4, c), x4[w4]) : x4[w4];
               for (uint32_t i = 0; i < P && (carry.x | carry.y | carry.z | carry.w); ++i) {
                  const uint4 p = planes4[i * W4 + w4];
                  planes4[i * W4 + w4] = make_uint4(p.x ^ carry.x, p.y ^ carry.y, p.z ^ carry.z, p.w ^ carry.w);
                  carry = make_uint4(carry.x & p.x, carry.y & p.y, carry.z & p.z, carry.w & p.w);
               }
               if (carry.x | carry.y | carry.z | carry.w) {  // saturate at 2^P - 1
                  for (uint32_t i = 0; i < P; ++i) {
                     const uint4 p = planes4[i * W4 + w4];
                     planes4[i * W4 + w4] = make_uint4(p.x | carry.x, p.y | carry.y, p.z | carry.z, p.w | carry.w);
                  }
               }
            }
            --sp;
            synced = false;
            break;
         }
         case OP_THR_END: {
            const uint32_t P = in.a, n = in.b;
            if (sp < P) {
               if (threadIdx.x == 0) atomicExch(err, 2);
               return false;
            }
            uint4* planes4 = stk4 + (sp - P) * W4;
            const bool exact = in.flags & 1;
            // compare the counter with n from the top plane down, four words at a time
            for (uint32_t w4 = threadIdx.x; w4 < W4; w4 += blockDim.x) {
               uint4 gt = make_uint4(0, 0, 0, 0), eq = make_uint4(~0u, ~0u, ~0u, ~0u);
               for (int i = static_cast<int>(P) - 1; i >= 0; --i) {
                  const uint4 p = planes4[i * W4 + w4];
                  const uint32_t nb = ((n >> i) & 1u) ? 0xFFFFFFFFu : 0u;
                  gt = make_uint4(gt.x | (eq.x & p.x & ~nb), gt.y | (eq.y & p.y & ~nb), gt.z | (eq.z & p.z & ~nb),
                                  gt.w | (eq.w & p.w & ~nb));
                  eq = make_uint4(eq.x & ~(p.x ^ nb), eq.y & ~(p.y ^ nb), eq.z & ~(p.z ^ nb), eq.w & ~(p.w ^ nb));
               }
               if (n >> P) eq = make_uint4(0, 0, 0, 0);  // n does not fit: the saturated count is below it
               const uint4 vm = valid4(w4, c);
               planes4[w4] = exact ? make_uint4(eq.x & vm.x, eq.y & vm.y, eq.z & vm.z, eq.w & vm.w)
                                   : make_uint4((gt.x | eq.x) & vm.x, (gt.y | eq.y) & vm.y, (gt.z | eq.z) & vm.z,
                                                (gt.w | eq.w) & vm.w);
            }
            sp = sp - P + 1;
            synced = false;
            break;
         }
         case OP_JZ:
         case OP_JFULL: {
            if (sp < 1) {
               if (threadIdx.x == 0) atomicExch(err, 2);
               return false;
            }
            const uint4* x = stk4 + (sp - 1) * W4;
            int differs = 0;
            if (in.op == OP_JZ) {
               for (uint32_t w4 = threadIdx.x; w4 < W4; w4 += blockDim.x) differs |= any4(x[w4]);
            } else {
               for (uint32_t w4 = threadIdx.x; w4 < W4; w4 += blockDim.x) differs |= ne4(x[w4], valid4(w4, c));
            }
            differs = __syncthreads_or(differs);
            synced = true;
            if (!differs) {
               if (in.a <= pc || in.a > ncode) {
                  if (threadIdx.x == 0) atomicExch(err, 4);
                  return false;
               }
               next = in.a;
            }
            break;
         }
         default:
            if (threadIdx.x == 0) atomicExch(err, 5);
            return false;
      }
      if (trace) {
         __syncthreads();
         const long long t_end = clock64();
         uint32_t n = 0;
         if (sp >= 1) {
            const uint4* x = stk4 + (sp - 1) * W4;
            for (uint32_t w4 = threadIdx.x; w4 < W4; w4 += blockDim.x)
               n += __popc(x[w4].x) + __popc(x[w4].y) + __popc(x[w4].z) + __popc(x[w4].w);
         }
         n = __reduce_add_sync(0xFFFFFFFFu, n);
         if ((threadIdx.x & 31) == 0) tred[threadIdx.x >> 5] = n;
         __syncthreads();
         if (threadIdx.x == 0) {
            uint32_t s = 0;
            for (uint32_t w = 0; w < (blockDim.x >> 5); ++w) s += tred[w];
            const long long dt = t_end - t_start;
            trace[2 * pc] = static_cast<uint32_t>(dt < 1 ? 1 : (dt > 0xFFFFFFFFll ? 0xFFFFFFFFll : dt));
            trace[2 * pc + 1] = s;
         }
         __syncthreads();
         synced = true;
      }
      pc = next;
   }
   if (sp != 1) {
      if (threadIdx.x == 0) atomicExch(err, 2);
      return false;
   }
   return true;
}

__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t* red) {
   v = __reduce_add_sync(0xFFFFFFFFu, v);
   const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
   __syncthreads();
   if (lane == 0) red[warp] = v;
   __syncthreads();
   uint32_t s = 0;
   if (threadIdx.x == 0) {
      for (uint32_t i = 0; i < (blockDim.x >> 5); ++i) s += red[i];
   }
   return s;  // valid in thread 0
}

// Popcount of the result tile (slot 0) by the owners of its words, optionally copied to dst.
__device__ __forceinline__ uint32_t result_popc(const uint32_t* smem, uint32_t W, uint32_t* dst) {
   const uint4* r4 = reinterpret_cast<const uint4*>(smem);
   uint4* d4 = reinterpret_cast<uint4*>(dst);
   uint32_t pc = 0;
   for (uint32_t w4 = threadIdx.x; w4 < (W >> 7); w4 += blockDim.x) {
      const uint4 x = r4[w4];
      pc += __popc(x.x) + __popc(x.y) + __popc(x.z) + __popc(x.w);
      if (dst) d4[w4] = x;
   }
   return pc;
}

__global__ void __launch_bounds__(FT) filter_kernel(const DevTable* __restrict__ tab, const Instr* __restrict__ code,
                                                    uint32_t ncode, uint32_t n_leaves, uint32_t tile_bits, uint32_t cap,
                                                    uint32_t* __restrict__ out_tiles, unsigned long long* count, int* err,
                                                    uint32_t* trace, const uint32_t* __restrict__ aux) {
   extern __shared__ __align__(16) uint32_t smem[];
   __shared__ uint32_t red[FT / 32];
   __shared__ LeafCache lc;
   const uint32_t T = CHUNK_ROWS / tile_bits;
   TileCtx c;
   c.tab = tab;
   c.v = blockIdx.x / T;
   c.W = tile_bits;
   c.row0 = (blockIdx.x % T) * tile_bits;
   c.aux = aux;
   const uint32_t csize = __ldg(tab->chunk_sizes + c.v);
   c.nvalid = csize > c.row0 ? min(tile_bits, csize - c.row0) : 0u;
   if (c.nvalid == 0) {
      for (uint32_t w4 = threadIdx.x; w4 < (tile_bits >> 7); w4 += blockDim.x)
         reinterpret_cast<uint4*>(smem)[w4] = make_uint4(0, 0, 0, 0);
   } else {
      init_leaves(lc);
      clear_leaves(lc, min(n_leaves & 0xFFFFu, LC_LEAVES), min(n_leaves >> 16, LC_COV));
      __syncthreads();
      uint32_t phase = 0;
      if (!stage_leaves(lc, c, code, ncode, phase, err)) return;
      if (!run_program(c, code, ncode, smem, cap, lc, err,
                       trace ? trace + static_cast<size_t>(blockIdx.x) * ncode * 2 : nullptr))
         return;
   }
   const uint32_t pc =
      result_popc(smem, tile_bits, out_tiles ? out_tiles + static_cast<size_t>(c.v) * CHUNK_WORDS + (c.row0 >> 5) : nullptr);
   if (count) {
      const uint32_t s = block_sum(pc, red);
      if (threadIdx.x == 0 && s) atomicAdd(count, static_cast<unsigned long long>(s));
   }
}

__global__ void __launch_bounds__(FT) filter_batch_kernel(const DevTable* __restrict__ tab, const Instr* __restrict__ code,
                                                          const QueryDesc* __restrict__ queries,
                                                          const WorkItem* __restrict__ items, uint32_t n_items,
                                                          uint32_t stack_words, uint32_t* __restrict__ out_tiles,
                                                          unsigned long long* counts, uint32_t* next_item, int* err,
                                                          const uint32_t* __restrict__ aux) {
   extern __shared__ __align__(16) uint32_t smem[];
   __shared__ uint32_t red[FT / 32];
   __shared__ uint32_t item_idx;
   __shared__ LeafCache lc;
   const size_t per_query = static_cast<size_t>(tab->nchunks) * CHUNK_WORDS;
   init_leaves(lc);
   uint32_t phase = 0;
   for (;;) {
      if (threadIdx.x == 0) item_idx = atomicAdd(next_item, 1u);
      __syncthreads();
      const uint32_t it = item_idx;
      if (it >= n_items) return;
      const WorkItem wi = items[it];
      const QueryDesc q = queries[wi.query];
      const uint32_t tile_bits = q.tile_bits, T = CHUNK_ROWS / tile_bits;
      const uint32_t cap = stack_words / (tile_bits >> 5);  // stack tiles of this width
      // the program uses q.depth stack tiles; the CTA's other tiles take this item's payloads
      const uint32_t depth = min(max(q.depth, 1u), cap);
      const uint32_t ext_cap = min((cap - depth) * (tile_bits / 16), 65535u - LC_PAY - 16u) & ~7u;
      clear_leaves(lc, min(q.n_leaves & 0xFFFFu, LC_LEAVES), min(q.n_leaves >> 16, LC_COV),
                   reinterpret_cast<uint16_t*>(smem + static_cast<size_t>(depth) * (tile_bits >> 5)), ext_cap);
      __syncthreads();
      TileCtx c;
      c.tab = tab;
      c.v = wi.tile / T;
      c.W = tile_bits;
      c.row0 = (wi.tile % T) * tile_bits;
      c.aux = aux ? aux + static_cast<size_t>(q.aux_base) * per_query : nullptr;
      const uint32_t csize = __ldg(tab->chunk_sizes + c.v);
      c.nvalid = csize > c.row0 ? min(tile_bits, csize - c.row0) : 0u;
      if (c.nvalid == 0) {
         for (uint32_t w4 = threadIdx.x; w4 < (tile_bits >> 7); w4 += blockDim.x)
            reinterpret_cast<uint4*>(smem)[w4] = make_uint4(0, 0, 0, 0);
      } else {
         if (!stage_leaves(lc, c, code + q.code_off, q.code_len, phase, err)) return;
         // the stack may not grow past the program's depth into the staged payloads
         if (!run_program(c, code + q.code_off, q.code_len, smem, depth, lc, err)) return;
      }
      uint32_t* dst = q.out_tiles ? out_tiles + static_cast<size_t>(q.out_tiles - 1) * per_query +
                                       static_cast<size_t>(c.v) * CHUNK_WORDS + (c.row0 >> 5)
                                  : nullptr;
      const uint32_t pc = result_popc(smem, tile_bits, dst);
      const uint32_t s = block_sum(pc, red);
      if (threadIdx.x == 0 && s) atomicAdd(counts + wi.query, static_cast<unsigned long long>(s));
      __syncthreads();
   }
}
}  // namespace

// ------------------------------------------------------------------------------------------------
// launchers

cudaError_t launch_filter(const DevTable* d_table, uint32_t nchunks, const Instr* d_code, uint32_t ncode,
                          uint32_t n_leaves, uint32_t tile_bits, uint32_t stack_tiles, uint32_t* d_out_tiles, unsigned long long* d_count,
                          int* d_err, void* stream, uint32_t* d_trace, const uint32_t* d_aux) {
   const uint32_t T = CHUNK_ROWS / tile_bits;
   const size_t smem = static_cast<size_t>(stack_tiles) * (tile_bits / 8);
   cudaError_t e = cudaFuncSetAttribute(filter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        static_cast<int>(smem > 48 * 1024 ? smem : 48 * 1024));
   if (e != cudaSuccess) return e;
   filter_kernel<<<nchunks * T, FT, smem, static_cast<cudaStream_t>(stream)>>>(
      d_table, d_code, ncode, n_leaves, tile_bits, stack_tiles, d_out_tiles, d_count, d_err, d_trace, d_aux);
   return cudaGetLastError();
}

int filter_batch_blocks_per_sm(size_t smem_bytes) {
   if (cudaFuncSetAttribute(filter_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            static_cast<int>(smem_bytes > 48 * 1024 ? smem_bytes : 48 * 1024)) != cudaSuccess) {
      cudaGetLastError();
      return 1;
   }
   int n = 0;
   if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, filter_batch_kernel, FT, smem_bytes) != cudaSuccess) {
      cudaGetLastError();
      return 1;
   }
   return n > 0 ? n : 1;
}

cudaError_t launch_filter_batch(const DevTable* d_table, uint32_t nchunks, const Instr* d_code, const QueryDesc* d_queries,
                         const WorkItem* d_items, uint32_t n_items, uint32_t stack_bytes, uint32_t* d_out_tiles,
                         unsigned long long* d_counts, uint32_t* d_next, uint32_t grid, int* d_err, void* stream,
                         const uint32_t* d_aux) {
   (void)nchunks;
   const size_t smem = stack_bytes;
   cudaError_t e = cudaFuncSetAttribute(filter_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        static_cast<int>(smem > 48 * 1024 ? smem : 48 * 1024));
   if (e != cudaSuccess) return e;
   filter_batch_kernel<<<grid, FT, smem, static_cast<cudaStream_t>(stream)>>>(
      d_table, d_code, d_queries, d_items, n_items, stack_bytes / 4, d_out_tiles, d_counts, d_next, d_err, d_aux);
   return cudaGetLastError();
}

void set_copy_withholding(bool on) {
   const uint32_t v = on ? 1u : 0u;
   const cudaError_t e = cudaMemcpyToSymbol(g_withhold_leaf_copies, &v, sizeof(v));
   if (e != cudaSuccess) throw std::runtime_error(std::string("set_copy_withholding: ") + cudaGetErrorString(e));
}

}  // namespace rhygpu
