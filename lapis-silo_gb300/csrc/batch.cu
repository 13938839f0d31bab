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
constexpr uint32_t NSPLIT = 4;  // CTAs per missing-interval block and query group

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

__device__ __forceinline__ void add_mask(uint32_t (&acc)[MUT_GROUP], uint32_t m) {
#pragma unroll
   for (uint32_t q = 0; q < MUT_GROUP; ++q) acc[q] += (m >> q) & 1u;
}

__global__ void __launch_bounds__(CT) mut_ctr_batch_kernel(const DevTable* __restrict__ tab, uint32_t col,
                                                           const uint16_t* __restrict__ T, uint32_t nq,
                                                           uint32_t* __restrict__ counts, int* err) {
   extern __shared__ __align__(128) uint16_t M[];  // CHUNK_ROWS query masks
   __shared__ __align__(8) uint64_t bar;
   const DevSeqCol* cs = &tab->seq[col];
   const uint32_t L = cs->L;
   const uint32_t nchunks = tab->nchunks;
   const uint32_t v = blockIdx.x % nchunks, g = blockIdx.x / nchunks;
   const size_t per_query = static_cast<size_t>(cs->nsym) * L;
   const uint32_t qbase = g * MUT_GROUP;
   const uint32_t nqg = nq - qbase < MUT_GROUP ? nq - qbase : MUT_GROUP;
   bulk_load_smem(M, T + (static_cast<size_t>(g) * nchunks + v) * CHUNK_ROWS, CHUNK_ROWS * 2, &bar);
   const bool ok = bulk_wait(&bar);
   if (!__syncthreads_and(ok)) {
      if (threadIdx.x == 0) atomicExch(err, 6);
      return;
   }
   const CtrDesc* __restrict__ ctrs = cs->ctrs;
   const uint16_t* __restrict__ payload = cs->payload;
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
         uint32_t acc[MUT_GROUP];
#pragma unroll
         for (uint32_t q = 0; q < MUT_GROUP; ++q) acc[q] = 0;
         small_array_for_each(d, payload, [&](uint32_t r) { add_mask(acc, M[r]); });
         uint32_t* dst = cbase + static_cast<size_t>(d.sym) * L + d.key;
#pragma unroll
         for (uint32_t q = 0; q < MUT_GROUP; ++q)
            if (q < nqg && acc[q]) atomicAdd(dst + q * per_query, acc[q]);
      }
      uint32_t bigmask = __ballot_sync(0xFFFFFFFFu, valid && !small);
      while (bigmask) {
         const int j = __ffs(bigmask) - 1;
         bigmask &= bigmask - 1;
         const CtrDesc dj = shfl_desc(raw, j);
         uint32_t acc[MUT_GROUP];
#pragma unroll
         for (uint32_t q = 0; q < MUT_GROUP; ++q) acc[q] = 0;
         if (dj.type == CT_ARRAY) {
            const uint32_t s = dj.payload, e = s + dj.card_m1 + 1u;
            const uint4* pw = reinterpret_cast<const uint4*>(payload);
            const uint32_t w0 = s >> 3, w1 = (e - 1) >> 3;
#pragma unroll 2
            for (uint32_t w = w0 + lane; w <= w1; w += 32) {
               const uint4 x = __ldg(pw + w);
#pragma unroll
               for (uint32_t t = 0; t < 8; ++t) {
                  const uint32_t jj = 8 * w + t;
                  if (jj >= s && jj < e) add_mask(acc, M[u16_of(x, t)]);
               }
            }
         } else if (dj.type == CT_BITSET) {
            const uint32_t* bits = reinterpret_cast<const uint32_t*>(payload + dj.payload);
            for (uint32_t w = lane; w < CHUNK_WORDS; w += 32) {
               uint32_t x = __ldg(bits + w);
               while (x) {
                  const uint32_t b = __ffs(x) - 1;
                  x &= x - 1;
                  add_mask(acc, M[32 * w + b]);
               }
            }
         } else {
            const uint16_t* p = payload + dj.payload;
            for (uint32_t k = lane; k < dj.nruns; k += 32) {
               const uint32_t s = __ldg(p + 2 * k), e = s + __ldg(p + 2 * k + 1);
               for (uint32_t r = s; r <= e; ++r) add_mask(acc, M[r]);
            }
         }
         uint32_t mine = 0;
#pragma unroll
         for (uint32_t q = 0; q < MUT_GROUP; ++q) {
            const uint32_t t = __reduce_add_sync(0xFFFFFFFFu, acc[q]);
            if (lane == q) mine = t;
         }
         if (lane < nqg && mine) atomicAdd(cbase + lane * per_query + static_cast<size_t>(dj.sym) * L + dj.key, mine);
      }
   }
}

// CTAs [0, nblocks * NSPLIT) x groups: missing intervals; the next nchunks x groups: coverage exceptions.
__global__ void __launch_bounds__(BT) mut_cov_batch_kernel(const DevTable* __restrict__ tab, uint32_t col,
                                                           const uint16_t* __restrict__ T, uint32_t nq,
                                                           uint32_t* __restrict__ scratch) {
   const DevSeqCol* cs = &tab->seq[col];
   const uint32_t L = cs->L, nchunks = tab->nchunks, nseg = mut_nseg(L);
   const uint32_t nunits = cs->nblocks * NSPLIT + nchunks;
   const uint32_t unit = blockIdx.x % nunits, g = blockIdx.x / nunits;
   const uint32_t qbase = g * MUT_GROUP;
   const uint32_t nqg = nq - qbase < MUT_GROUP ? nq - qbase : MUT_GROUP;
   const size_t per_query = mut_scratch_words(L);
   const uint16_t* Tg = T + static_cast<size_t>(g) * nchunks * CHUNK_ROWS;
   const uint32_t lane = threadIdx.x & 31;
   if (unit < cs->nblocks * NSPLIT) {
      __shared__ int diff[MUT_GROUP][NBLOCK + 1];
      for (uint32_t i = threadIdx.x; i < MUT_GROUP * (NBLOCK + 1); i += blockDim.x) (&diff[0][0])[i] = 0;
      __syncthreads();
      const uint32_t b = unit / NSPLIT, part = unit % NSPLIT;
      const uint32_t nb = __ldg(cs->nblk_off + static_cast<size_t>(b) * nchunks);
      const uint32_t ne = __ldg(cs->nblk_off + static_cast<size_t>(b + 1) * nchunks);
      const uint32_t per = (ne - nb + NSPLIT - 1) / NSPLIT;
      const uint32_t lo_i = nb + part * per, hi_i = min(ne, lo_i + per);
      // every warp walks its entries in lockstep so the block-edge counts can use ballots
      for (uint32_t i0 = lo_i + (threadIdx.x & ~31u); i0 < hi_i; i0 += blockDim.x) {
         const uint32_t i = i0 + lane;
         uint32_t m = 0, lo = 0, hi = 0;
         if (i < hi_i) {
            const uint2 raw = __ldg(reinterpret_cast<const uint2*>(cs->nblk) + i);
            m = __ldg(Tg + raw.x);
            lo = raw.y & 0xFFFFu;
            hi = raw.y >> 16;
         }
         const uint32_t m_start = lo == 0 ? m : 0, m_end = hi == NBLOCK ? m : 0;
#pragma unroll
         for (uint32_t q = 0; q < MUT_GROUP; ++q) {
            const uint32_t cs0 = __popc(__ballot_sync(0xFFFFFFFFu, (m_start >> q) & 1u));
            const uint32_t ce = __popc(__ballot_sync(0xFFFFFFFFu, (m_end >> q) & 1u));
            if (lane == q) {
               if (cs0) atomicAdd(&diff[q][0], static_cast<int>(cs0));
               if (ce) atomicSub(&diff[q][NBLOCK], static_cast<int>(ce));
            }
         }
         uint32_t mi = lo == 0 ? 0 : m;
         while (mi) {
            const uint32_t q = __ffs(mi) - 1;
            mi &= mi - 1;
            atomicAdd(&diff[q][lo], 1);
         }
         uint32_t mh = hi == NBLOCK ? 0 : m;
         while (mh) {
            const uint32_t q = __ffs(mh) - 1;
            mh &= mh - 1;
            atomicSub(&diff[q][hi], 1);
         }
      }
      __syncthreads();
      for (uint32_t k = threadIdx.x; k < MUT_GROUP * (NBLOCK + 1); k += blockDim.x) {
         const uint32_t q = k / (NBLOCK + 1), o = k % (NBLOCK + 1);
         const int x = diff[q][o];
         const uint32_t p = b * NBLOCK + o;
         if (q < nqg && x != 0 && p <= L) {
            uint32_t* sc = scratch + static_cast<size_t>(qbase + q) * per_query;
            atomicAdd(&sc[2 * (L + 1) + p], static_cast<uint32_t>(x));
            atomicAdd(&sc[3 * (L + 1) + 2 * nseg + p / MUT_SEG], static_cast<uint32_t>(x));
         }
      }
   } else {
      const uint32_t v = unit - cs->nblocks * NSPLIT;
      const uint32_t xb = __ldg(cs->exc_off + v), xe = __ldg(cs->exc_off + v + 1);
      const uint16_t* Tv = Tg + static_cast<size_t>(v) * CHUNK_ROWS;
      for (uint32_t i = xb + threadIdx.x; i < xe; i += blockDim.x) {
         const uint4 raw = __ldg(reinterpret_cast<const uint4*>(cs->exc) + i);
         uint32_t m = __ldg(Tv + raw.x);
         while (m) {
            const uint32_t q = __ffs(m) - 1;
            m &= m - 1;
            if (q >= nqg) break;
            uint32_t* sc = scratch + static_cast<size_t>(qbase + q) * per_query;
            atomicAdd(&sc[raw.y], 1u);
            atomicAdd(&sc[3 * (L + 1) + raw.y / MUT_SEG], 1u);
            atomicAdd(&sc[(L + 1) + raw.z], 1u);
            atomicAdd(&sc[3 * (L + 1) + nseg + raw.z / MUT_SEG], 1u);
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
                            const uint32_t* d_slot_query, uint16_t* d_masks, uint32_t* d_counts, uint32_t* d_scratch,
                            int* d_err, void* stream, uint32_t parts) {
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
   if (parts & BMUT_PART_COV)
      mut_cov_batch_kernel<<<(col_host.nblocks * NSPLIT + nchunks) * ngroups, BT, 0, s>>>(d_table, col, d_masks, nq,
                                                                                          d_scratch);
   if (parts & BMUT_PART_FINAL) {
      dim3 fin((col_host.L + MUT_SEG - 1) / MUT_SEG, nq);
      mut_final_batch_kernel<<<fin, MUT_SEG, 0, s>>>(d_table, col, d_fcounts, d_slot_query, d_counts, d_scratch);
   }
}

}  // namespace rhygpu
