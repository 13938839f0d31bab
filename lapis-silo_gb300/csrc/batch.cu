// Batched Mutations: many filters per pass over the vertical index.
//
// The plain path streams every container once per query. Here up to MUT_GROUP (16) filters share
// one pass: their row sets are transposed into one 16-bit query mask per row (transpose_kernel,
// warp ballots over 32 x 16 bit blocks), a CTA stages the masks of one chunk (128 KiB) into shared
// memory with a TMA bulk copy, and every container element yields the membership of all 16 queries
// with a single shared-memory load. Coverage exceptions and missing intervals are counted per
// query group the same way. Results are bit-identical to the single-query kernels.
#include <cuda_runtime.h>

#include "device.h"
#include "mutations_common.cuh"

namespace rhygpu {

constexpr uint32_t MUT_GROUP = 16;

namespace {

constexpr uint32_t BT = 256;
constexpr uint32_t CT = 1024;   // container kernel: one 128 KiB-mask CTA per SM, so make it wide


// T[g][v * CHUNK_ROWS + row] = bit q set iff row is in filter (16 g + q).
__global__ void __launch_bounds__(BT) transpose_kernel(const uint32_t* __restrict__ tiles, uint32_t nq, uint32_t nchunks,
                                                       uint16_t* __restrict__ T) {
   const uint32_t lane = threadIdx.x & 31;
   const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // global warp id
   const uint32_t words = nchunks * CHUNK_WORDS;
   const uint32_t ngroups = (nq + MUT_GROUP - 1) / MUT_GROUP;
   if (gw >= words * ngroups) return;
   const uint32_t g = gw / words, w = gw % words;
   const uint32_t q = g * MUT_GROUP + lane;
   uint32_t x = 0;
   if (lane < MUT_GROUP && q < nq) x = __ldg(tiles + static_cast<size_t>(q) * words + w);
   uint32_t mine = 0;
#pragma unroll
   for (uint32_t b = 0; b < 32; ++b) {
      const uint32_t m = __ballot_sync(0xFFFFFFFFu, (x >> b) & 1u);
      if (lane == b) mine = m;
   }
   T[static_cast<size_t>(g) * words * 32 + static_cast<size_t>(w) * 32 + lane] = static_cast<uint16_t>(mine);
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

// One CTA per (event item, query group). Missing events: per position, the queries whose filter
// holds the event's row add +1 (start) / -1 (end); coverage events count per query.
__global__ void __launch_bounds__(BT) mut_cov_batch_kernel(const DevTable* __restrict__ tab, uint32_t col,
                                                           const EvItem* __restrict__ items, uint32_t n_items,
                                                           const uint16_t* __restrict__ T, uint32_t nq,
                                                           uint32_t* __restrict__ scratch) {
   __shared__ int cnt[MUT_GROUP][NBLOCK + 1];
   __shared__ PackedLut lut;
   const DevSeqCol* cs = &tab->seq[col];
   const uint32_t L = cs->L, nchunks = tab->nchunks, nseg = mut_nseg(L);
   const uint32_t item = blockIdx.x % n_items, g = blockIdx.x / n_items;
   const uint32_t qbase = g * MUT_GROUP;
   const uint32_t nqg = nq - qbase < MUT_GROUP ? nq - qbase : MUT_GROUP;
   const size_t per_query = mut_scratch_words(L);
   const uint16_t* Tg = T + static_cast<size_t>(g) * nchunks * CHUNK_ROWS;
   const EvItem it = items[item];
   const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
   if (it.list <= EV_MEND) {
      build_lut(lut);
      for (uint32_t i = threadIdx.x; i < MUT_GROUP * (NBLOCK + 1); i += blockDim.x) (&cnt[0][0])[i] = 0;
      __syncthreads();
      const uint32_t* ev = it.list == EV_MSTART ? cs->mstart : cs->mend;
      constexpr uint32_t U = 4;  // events per lane in flight
      for (uint32_t base = it.begin + warp * 32 * U; base < it.end; base += blockDim.x * U) {
         uint32_t e[U], mk[U];
#pragma unroll
         for (uint32_t k = 0; k < U; ++k) {
            const uint32_t i = base + 32 * k + lane;
            e[k] = i < it.end ? __ldg(ev + i) : 0xFFFFFFFFu;
         }
#pragma unroll
         for (uint32_t k = 0; k < U; ++k) mk[k] = e[k] != 0xFFFFFFFFu ? __ldg(Tg + (e[k] >> 8)) : 0u;
#pragma unroll
         for (uint32_t k = 0; k < U; ++k) {
            const bool active = e[k] != 0xFFFFFFFFu;
            const uint32_t pos = e[k] & 0xFFu;
            const uint32_t amask = __ballot_sync(0xFFFFFFFFu, active);
            const uint32_t grp = __match_any_sync(0xFFFFFFFFu, active ? pos : 0xFFFFu);
            if (active) {
               uint32_t acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
               add_packed(acc, lut, mk[k]);
               const uint32_t members = grp & amask;
#pragma unroll
               for (uint32_t j = 0; j < 8; ++j) acc[j] = __reduce_add_sync(members, acc[j]);
               // the lanes of the group share the per-query additions
               const uint32_t gsize = __popc(members);
               const uint32_t grank = __popc(members & ((1u << lane) - 1u));
               for (uint32_t q = grank; q < nqg; q += gsize) {
                  const uint32_t c = unpack(acc, q);
                  if (c) atomicAdd(&cnt[q][pos], static_cast<int>(c));
               }
            }
         }
      }
      __syncthreads();
      const int sign = it.list == EV_MSTART ? 1 : -1;
      for (uint32_t k = threadIdx.x; k < MUT_GROUP * (NBLOCK + 1); k += blockDim.x) {
         const uint32_t q = k / (NBLOCK + 1), o = k % (NBLOCK + 1);
         const int x = cnt[q][o];
         const uint32_t p = it.block * NBLOCK + o;
         if (q < nqg && x != 0 && p <= L) {
            uint32_t* sc = scratch + static_cast<size_t>(qbase + q) * per_query;
            atomicAdd(&sc[2 * (L + 1) + p], static_cast<uint32_t>(sign * x));
            atomicAdd(&sc[3 * (L + 1) + 2 * nseg + p / MUT_SEG], static_cast<uint32_t>(sign * x));
         }
      }
   } else {
      const CovEvent* ev = it.list == EV_CSTART ? cs->cstart : cs->cend;
      const uint32_t hist_off = it.list == EV_CSTART ? 0 : (L + 1);
      const uint32_t seg_off = 3 * (L + 1) + (it.list == EV_CSTART ? 0 : nseg);
      for (uint32_t i = it.begin + threadIdx.x; i < it.end; i += blockDim.x) {
         const uint2 e = __ldg(reinterpret_cast<const uint2*>(ev) + i);
         uint32_t m = __ldg(Tg + e.x);
         while (m) {
            const uint32_t q = __ffs(m) - 1;
            m &= m - 1;
            if (q >= nqg) break;
            uint32_t* sc = scratch + static_cast<size_t>(qbase + q) * per_query;
            atomicAdd(&sc[hist_off + e.y], 1u);
            atomicAdd(&sc[seg_off + e.y / MUT_SEG], 1u);
         }
      }
   }
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
   return static_cast<size_t>(ngroups) * nchunks * CHUNK_ROWS * 2;
}

void launch_mutations_batch(const DevTable* d_table, const DevSeqCol& col_host, uint32_t col, uint32_t nchunks,
                            const uint32_t* d_filters, uint32_t nq, const unsigned long long* d_fcounts,
                            const uint32_t* d_slot_query, const EvItem* d_ev, uint32_t n_ev, uint16_t* d_masks,
                            uint32_t* d_counts, uint32_t* d_scratch, int* d_err, void* stream, uint32_t parts) {
   if (nq == 0) return;
   cudaStream_t s = static_cast<cudaStream_t>(stream);
   const uint32_t ngroups = (nq + MUT_GROUP - 1) / MUT_GROUP;
   const uint64_t warps = static_cast<uint64_t>(nchunks) * CHUNK_WORDS * ngroups;
   if (parts & BMUT_PART_TRANSPOSE)
      transpose_kernel<<<static_cast<uint32_t>((warps * 32 + BT - 1) / BT), BT, 0, s>>>(d_filters, nq, nchunks, d_masks);
   if (parts & BMUT_PART_CTR) {
      const int smem = CHUNK_ROWS * 2;
      cudaFuncSetAttribute(mut_ctr_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
      mut_ctr_batch_kernel<<<nchunks * ngroups, CT, smem, s>>>(d_table, col, d_masks, nq, d_counts, d_err);
   }
   if ((parts & BMUT_PART_COV) && n_ev > 0)
      mut_cov_batch_kernel<<<n_ev * ngroups, BT, 0, s>>>(d_table, col, d_ev, n_ev, d_masks, nq, d_scratch);
   if (parts & BMUT_PART_FINAL) {
      dim3 fin((col_host.L + MUT_SEG - 1) / MUT_SEG, nq);
      mut_final_batch_kernel<<<fin, MUT_SEG, 0, s>>>(d_table, col, d_fcounts, d_slot_query, d_counts, d_scratch);
   }
}

}  // namespace rhygpu
