// Batched Mutations: many filters per pass over the vertical index.
//
// The plain path streams every container once per query. Here up to MUT_GROUP (16) filters share
// one pass: their row sets are transposed into one 16-bit query mask per row (transpose_kernel,
// warp ballots over 32 x 16 bit blocks), a CTA stages the masks of one chunk (128 KiB) into shared
// memory with a TMA bulk copy, and every container element yields the membership of all 16 queries
// with a single shared-memory load. The coverage pass reads every missing-interval and coverage
// boundary event once for all queries: the transpose also writes a row-major copy of the masks,
// and one lane per 16-query group gathers its mask of the event's row. Results are bit-identical
// to the single-query kernels.
#include <cuda_runtime.h>

#include "device.h"
#include "mutations_common.cuh"

namespace rhygpu {

constexpr uint32_t MUT_GROUP = 16;

namespace {

constexpr uint32_t BT = 256;
constexpr uint32_t CT = 1024;   // container kernel: one 128 KiB-mask CTA per SM, so make it wide


// Query masks in two layouts, both with bit q of a 16-bit mask set iff the row is in filter 16 g + q:
//   group-major T[g][v * CHUNK_ROWS + row]   one 128 KiB slab per (group, chunk), staged by the
//                                            container kernel;
//   row-major   R[row][c] (u32, c < nqc)     the masks of all groups of one row side by side, 4 nqc
//                                            bytes, gathered by the coverage kernel.
// A CTA covers TR_WORDS filter words (32 TR_WORDS rows); warp w turns word w of 32 filters at a
// time into 32 row masks with ballots and stages them in shared memory for coalesced row stores.
constexpr uint32_t TR_WORDS = BT / 32;
constexpr uint32_t TR_CHUNKS = 32;  // query chunks of 32 staged per round

__global__ void __launch_bounds__(BT) transpose_kernel(const uint32_t* __restrict__ tiles, uint32_t nq, uint32_t nchunks,
                                                       uint16_t* __restrict__ T, uint32_t* __restrict__ R) {
   __shared__ uint32_t stage[TR_WORDS * 32 * (TR_CHUNKS + 1)];
   const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
   const uint32_t words = nchunks * CHUNK_WORDS;
   const uint32_t ngroups = (nq + MUT_GROUP - 1) / MUT_GROUP;
   const uint32_t nqc = (nq + 31) / 32;
   const uint32_t w = blockIdx.x * TR_WORDS + warp;  // words is a multiple of TR_WORDS
   const size_t rows = static_cast<size_t>(words) * 32;
   for (uint32_t c0 = 0; c0 < nqc; c0 += TR_CHUNKS) {
      const uint32_t nc = nqc - c0 < TR_CHUNKS ? nqc - c0 : TR_CHUNKS;
      const uint32_t P = nc | 1u;  // odd stride: the 32 lanes of a warp hit 32 banks
      for (uint32_t c = 0; c < nc; ++c) {
         const uint32_t q = 32 * (c0 + c) + lane;
         const uint32_t x = q < nq ? __ldg(tiles + static_cast<size_t>(q) * words + w) : 0u;
         uint32_t mine = 0;
#pragma unroll
         for (uint32_t b = 0; b < 32; ++b) {
            const uint32_t m = __ballot_sync(0xFFFFFFFFu, (x >> b) & 1u);
            if (lane == b) mine = m;
         }
         const uint32_t g0 = 2 * (c0 + c);
         const size_t row = static_cast<size_t>(w) * 32 + lane;
         T[static_cast<size_t>(g0) * rows + row] = static_cast<uint16_t>(mine);
         if (g0 + 1 < ngroups) T[static_cast<size_t>(g0 + 1) * rows + row] = static_cast<uint16_t>(mine >> 16);
         stage[(warp * 32 + lane) * P + c] = mine;
      }
      __syncthreads();
      const size_t row0 = static_cast<size_t>(blockIdx.x) * TR_WORDS * 32;
      for (uint32_t k = threadIdx.x; k < TR_WORDS * 32 * nc; k += blockDim.x) {
         const uint32_t r = k / nc, c = k % nc;
         R[(row0 + r) * nqc + c0 + c] = stage[r * P + c];
      }
      __syncthreads();
   }
}

__device__ __forceinline__ void bulk_load_smem(void* smem, const void* gmem, uint32_t bytes, uint64_t* bar) {
   // one thread issues TMA bulk copies global -> shared that complete on the mbarrier
   const uint32_t s = static_cast<uint32_t>(__cvta_generic_to_shared(smem));
   const uint32_t b = static_cast<uint32_t>(__cvta_generic_to_shared(bar));
   if (threadIdx.x == 0) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b));
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
   }
   __syncthreads();
   if (threadIdx.x == 0) {
      asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}\n" ::"r"(b), "r"(bytes)
                   : "memory");
      for (uint32_t off = 0; off < bytes; off += 65536u) {
         const uint32_t n = bytes - off < 65536u ? bytes - off : 65536u;
         asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(s + off),
            "l"(static_cast<const char*>(gmem) + off), "r"(n), "r"(b)
            : "memory");
      }
   }
}

// Waits for phase 0 of the mbarrier with a bounded spin. Returns false if it gave up.
__device__ __forceinline__ bool bulk_wait(uint64_t* bar) {
   const uint32_t b = static_cast<uint32_t>(__cvta_generic_to_shared(bar));
   for (uint32_t i = 0; i < (1u << 24); ++i) {
      uint32_t done;
      asm volatile(
         "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
         : "=r"(done)
         : "r"(b)
         : "memory");
      if (done) return true;
   }
   return false;
}

// Per-query counters for 16 queries packed as eight u32 registers of two 16-bit lanes; a table
// maps one byte of a query mask to its four packed increments, so one element costs two table
// loads and eight adds for all 16 queries.
struct PackedLut {
   uint4 e[256];
};

__device__ __forceinline__ void build_lut(PackedLut& lut) {
   for (uint32_t x = threadIdx.x; x < 256; x += blockDim.x) {
      uint4 v;
      v.x = ((x >> 0) & 1u) | (((x >> 1) & 1u) << 16);
      v.y = ((x >> 2) & 1u) | (((x >> 3) & 1u) << 16);
      v.z = ((x >> 4) & 1u) | (((x >> 5) & 1u) << 16);
      v.w = ((x >> 6) & 1u) | (((x >> 7) & 1u) << 16);
      lut.e[x] = v;
   }
}

__device__ __forceinline__ void add_packed(uint32_t (&acc)[8], const PackedLut& lut, uint32_t m) {
   const uint4 a = lut.e[m & 0xFFu];
   const uint4 b = lut.e[(m >> 8) & 0xFFu];
   acc[0] += a.x;
   acc[1] += a.y;
   acc[2] += a.z;
   acc[3] += a.w;
   acc[4] += b.x;
   acc[5] += b.y;
   acc[6] += b.z;
   acc[7] += b.w;
}

__device__ __forceinline__ uint32_t unpack(const uint32_t (&acc)[8], uint32_t q) {
   uint32_t v = acc[0];
#pragma unroll
   for (uint32_t i = 1; i < 8; ++i)
      if ((q >> 1) == i) v = acc[i];
   return (q & 1u) ? (v >> 16) : (v & 0xFFFFu);
}

__global__ void __launch_bounds__(CT) mut_ctr_batch_kernel(const DevTable* __restrict__ tab, uint32_t col,
                                                           const uint16_t* __restrict__ T, uint32_t nq,
                                                           uint32_t* __restrict__ counts, int* err) {
   extern __shared__ __align__(128) uint16_t M[];  // CHUNK_ROWS query masks
   __shared__ __align__(8) uint64_t bar;
   __shared__ PackedLut lut;
   const DevSeqCol* cs = &tab->seq[col];
   const uint32_t L = cs->L;
   const uint32_t nchunks = tab->nchunks;
   const uint32_t v = blockIdx.x % nchunks, g = blockIdx.x / nchunks;
   const size_t per_query = static_cast<size_t>(cs->nsym) * L;
   const uint32_t qbase = g * MUT_GROUP;
   const uint32_t nqg = nq - qbase < MUT_GROUP ? nq - qbase : MUT_GROUP;
   build_lut(lut);
   bulk_load_smem(M, T + (static_cast<size_t>(g) * nchunks + v) * CHUNK_ROWS, CHUNK_ROWS * 2, &bar);
   const bool ok = bulk_wait(&bar);
   if (!__syncthreads_and(ok)) {
      if (threadIdx.x == 0) atomicExch(err, 6);
      return;
   }
   const CtrDesc* __restrict__ ctrs = cs->ctrs;
   const uint16_t* __restrict__ payload = cs->payload;
   const uint4* __restrict__ pw = reinterpret_cast<const uint4*>(payload);
   const uint32_t begin = __ldg(cs->off + static_cast<size_t>(v) * L), end = __ldg(cs->off + static_cast<size_t>(v + 1) * L);
   const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
   uint32_t* cbase = counts + static_cast<size_t>(qbase) * per_query;
   for (uint32_t base = begin + warp * 32; base < end; base += nw * 32) {
      const uint32_t idx = base + lane;
      const bool valid = idx < end;
      uint4 raw = make_uint4(0, 0, 0, 0);
      if (valid) raw = __ldg(reinterpret_cast<const uint4*>(ctrs) + idx);
      const CtrDesc d = *reinterpret_cast<const CtrDesc*>(&raw);
      const bool small = valid && d.type == CT_ARRAY && d.card_m1 < SMALL_ARRAY;
      if (small) {
         uint32_t acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
         const uint32_t s = d.payload, e = s + d.card_m1 + 1u;
         for (uint32_t w = s >> 3; w <= (e - 1) >> 3; ++w) {
            const uint4 x = __ldg(pw + w);
#pragma unroll
            for (uint32_t t = 0; t < 8; ++t) {
               const uint32_t j = 8 * w + t;
               if (j >= s && j < e) add_packed(acc, lut, M[u16_of(x, t)]);
            }
         }
         uint32_t* dst = cbase + static_cast<size_t>(d.sym) * L + d.key;
#pragma unroll
         for (uint32_t q = 0; q < MUT_GROUP; ++q) {
            const uint32_t c = (acc[q >> 1] >> (16 * (q & 1))) & 0xFFFFu;
            if (q < nqg && c) atomicAdd(dst + q * per_query, c);
         }
      }
      uint32_t bigmask = __ballot_sync(0xFFFFFFFFu, valid && !small);
      while (bigmask) {
         const int j = __ffs(bigmask) - 1;
         bigmask &= bigmask - 1;
         const CtrDesc dj = shfl_desc(raw, j);
         uint32_t total[MUT_GROUP];
         if (dj.type == CT_ARRAY) {
            // at most 4096 elements: the packed 16-bit counters cannot overflow
            uint32_t acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            const uint32_t s = dj.payload, e = s + dj.card_m1 + 1u;
            const uint32_t w0 = s >> 3, w1 = (e - 1) >> 3;
#pragma unroll 2
            for (uint32_t w = w0 + lane; w <= w1; w += 32) {
               const uint4 x = __ldg(pw + w);
#pragma unroll
               for (uint32_t t = 0; t < 8; ++t) {
                  const uint32_t jj = 8 * w + t;
                  if (jj >= s && jj < e) add_packed(acc, lut, M[u16_of(x, t)]);
               }
            }
#pragma unroll
            for (uint32_t i = 0; i < 8; ++i) acc[i] = __reduce_add_sync(0xFFFFFFFFu, acc[i]);
#pragma unroll
            for (uint32_t q = 0; q < MUT_GROUP; ++q) total[q] = unpack(acc, q);
         } else {
            // bitsets and runs can hold a whole chunk: count per lane, then reduce in 32 bits
            uint32_t acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            if (dj.type == CT_BITSET) {
               const uint32_t* bits = reinterpret_cast<const uint32_t*>(payload + dj.payload);
               for (uint32_t w = lane; w < CHUNK_WORDS; w += 32) {  // at most 2048 rows per lane
                  uint32_t x = __ldg(bits + w);
                  while (x) {
                     const uint32_t b = __ffs(x) - 1;
                     x &= x - 1;
                     add_packed(acc, lut, M[32 * w + b]);
                  }
               }
#pragma unroll
               for (uint32_t q = 0; q < MUT_GROUP; ++q) total[q] = __reduce_add_sync(0xFFFFFFFFu, unpack(acc, q));
            } else {
#pragma unroll
               for (uint32_t q = 0; q < MUT_GROUP; ++q) total[q] = 0;
               const uint16_t* p = payload + dj.payload;
               for (uint32_t k = lane; k < dj.nruns; k += 32) {
                  const uint32_t s = __ldg(p + 2 * k), e = s + __ldg(p + 2 * k + 1);
                  for (uint32_t r = s; r <= e; ++r) {
                     const uint32_t m = M[r];
#pragma unroll
                     for (uint32_t q = 0; q < MUT_GROUP; ++q) total[q] += (m >> q) & 1u;
                  }
               }
#pragma unroll
               for (uint32_t q = 0; q < MUT_GROUP; ++q) total[q] = __reduce_add_sync(0xFFFFFFFFu, total[q]);
            }
         }
         uint32_t mine = 0;
#pragma unroll
         for (uint32_t q = 0; q < MUT_GROUP; ++q)
            if (lane == q) mine = total[q];
         if (lane < nqg && mine) atomicAdd(cbase + lane * per_query + static_cast<size_t>(dj.sym) * L + dj.key, mine);
      }
   }
}

// Per-lane counters of the 16 queries of one group at the current position. Masks are added two
// events at a time as one 32-bit word w = m1 | m2 << 16 into four words of nibble counters:
// nibble k of nib[j] counts query j + 4 (k % 4). After at most 15 additions the nibbles are
// drained into 32-bit counters.
struct GroupCounter {
   uint32_t nib[4];
   uint32_t nadd;
   uint32_t c[MUT_GROUP];    // counts at the current position
   uint32_t seg[MUT_GROUP];  // counts in the current MUT_SEG segment

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

// One CTA per event item and pass of up to 32 query groups (blockIdx.y). A sub-warp of gsz lanes,
// one lane per query group, streams a contiguous slice of the item's position-sorted events: each
// lane gathers its group's mask of the event's row from the row-major matrix R and counts its 16
// queries; when the position changes it adds the nonzero counts to the query's difference array
// (missing events: +1 start, -1 end) or boundary histogram (coverage events), and once per segment
// to the segment totals. Events are read once for all groups of the pass.
__global__ void __launch_bounds__(BT, 3) mut_cov_batch_kernel(const DevTable* __restrict__ tab, uint32_t col,
                                                           const EvItem* __restrict__ items,
                                                           const uint16_t* __restrict__ R, uint32_t nq,
                                                           uint32_t* __restrict__ scratch) {
   const DevSeqCol* cs = &tab->seq[col];
   const uint32_t L = cs->L, nseg = mut_nseg(L);
   const size_t per_query = mut_scratch_words(L);
   const uint32_t ngroups = (nq + MUT_GROUP - 1) / MUT_GROUP;
   const uint32_t S = 2u * ((nq + 31) / 32);  // u16 masks per row of R
   const uint32_t gpass = blockIdx.y * 32;
   const uint32_t gleft = ngroups - gpass;
   uint32_t gsz = 1;
   while (gsz < gleft && gsz < 32) gsz <<= 1;
   const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
   const uint32_t g = gpass + (lane & (gsz - 1));
   const bool gvalid = g < ngroups;
   const uint32_t spw = 32 / gsz;
   const uint32_t nsub = (blockDim.x >> 5) * spw, sub = warp * spw + lane / gsz;
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
   uint32_t* sc = scratch + static_cast<size_t>(g) * MUT_GROUP * per_query;

   GroupCounter k;
#pragma unroll
   for (uint32_t q = 0; q < MUT_GROUP; ++q) k.c[q] = k.seg[q] = 0;
#pragma unroll
   for (uint32_t j = 0; j < 4; ++j) k.nib[j] = 0;
   k.nadd = 0;
   constexpr uint32_t NONE = 0xFFFFFFFEu, INVALID = 0xFFFFFFFFu;
   uint32_t cur = NONE, curseg = NONE;

   auto flush_seg = [&]() {
      if (curseg == NONE) return;
#pragma unroll
      for (uint32_t q = 0; q < MUT_GROUP; ++q) {
         if (k.seg[q] && MUT_GROUP * g + q < nq)
            atomicAdd(sc + q * per_query + segb + curseg, k.seg[q] * sign);
         k.seg[q] = 0;
      }
   };
   auto flush_pos = [&]() {
      k.drain();
      if (cur != NONE && cur <= L) {
#pragma unroll
         for (uint32_t q = 0; q < MUT_GROUP; ++q) {
            if (k.c[q] && MUT_GROUP * g + q < nq) atomicAdd(sc + q * per_query + hist + cur, k.c[q] * sign);
            k.seg[q] += k.c[q];
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
         m[u] = (pos[u] != INVALID && gvalid) ? __ldg(R + static_cast<size_t>(row[u]) * S + g) : 0u;
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

// grid (ceil(L / MUT_SEG), nq): reference counts of slot blockIdx.y.
__global__ void __launch_bounds__(MUT_SEG) mut_final_batch_kernel(const DevTable* __restrict__ tab, uint32_t col,
                                                                  const unsigned long long* __restrict__ fcounts,
                                                                  const uint32_t* __restrict__ slot_query,
                                                                  uint32_t* __restrict__ counts,
                                                                  const uint32_t* __restrict__ scratch) {
   __shared__ uint32_t red[MUT_SEG / 32];
   const DevSeqCol* cs = &tab->seq[col];
   const uint32_t q = blockIdx.y;
   const uint32_t total = static_cast<uint32_t>(fcounts[slot_query[q]]);
   final_position_counts(cs, total, counts + static_cast<size_t>(q) * cs->nsym * cs->L,
                         scratch + static_cast<size_t>(q) * mut_scratch_words(cs->L), red);
}

}  // namespace

size_t mutations_batch_mask_bytes(uint32_t nq, uint32_t nchunks) {
   const uint32_t ngroups = (nq + MUT_GROUP - 1) / MUT_GROUP;
   const uint32_t nqc = (nq + 31) / 32;
   return static_cast<size_t>(ngroups) * nchunks * CHUNK_ROWS * 2 + static_cast<size_t>(nqc) * nchunks * CHUNK_ROWS * 4;
}

void launch_mutations_batch(const DevTable* d_table, const DevSeqCol& col_host, uint32_t col, uint32_t nchunks,
                            const uint32_t* d_filters, uint32_t nq, const unsigned long long* d_fcounts,
                            const uint32_t* d_slot_query, const EvItem* d_ev, uint32_t n_ev, uint16_t* d_masks,
                            uint32_t* d_counts, uint32_t* d_scratch, int* d_err, void* stream, uint32_t parts) {
   if (nq == 0) return;
   cudaStream_t s = static_cast<cudaStream_t>(stream);
   const uint32_t ngroups = (nq + MUT_GROUP - 1) / MUT_GROUP;
   uint16_t* d_rows = d_masks + static_cast<size_t>(ngroups) * nchunks * CHUNK_ROWS;  // row-major masks
   if (parts & BMUT_PART_TRANSPOSE)
      transpose_kernel<<<nchunks * CHUNK_WORDS / TR_WORDS, BT, 0, s>>>(d_filters, nq, nchunks, d_masks,
                                                                       reinterpret_cast<uint32_t*>(d_rows));
   if (parts & BMUT_PART_CTR) {
      const int smem = CHUNK_ROWS * 2;
      cudaFuncSetAttribute(mut_ctr_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
      mut_ctr_batch_kernel<<<nchunks * ngroups, CT, smem, s>>>(d_table, col, d_masks, nq, d_counts, d_err);
   }
   if ((parts & BMUT_PART_COV) && n_ev > 0)
      mut_cov_batch_kernel<<<dim3(n_ev, (ngroups + 31) / 32), BT, 0, s>>>(d_table, col, d_ev, d_rows, nq, d_scratch);
   if (parts & BMUT_PART_FINAL) {
      dim3 fin((col_host.L + MUT_SEG - 1) / MUT_SEG, nq);
      mut_final_batch_kernel<<<fin, MUT_SEG, 0, s>>>(d_table, col, d_fcounts, d_slot_query, d_counts, d_scratch);
   }
}

}  // namespace rhygpu
