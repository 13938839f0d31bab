// MutationProfile row sets (reference: src/rhydb/query_engine/scalar_expressions/mutation_profile.cpp:198-257).
//
// The reference rewrites a profile into Not(NOf(distance + 1, one SymbolInSet per position)), a
// threshold over up to a genome's length of children. Here every row counts its differences from
// the row index in one pass. A covered row holding the local reference everywhere has `base`
// differences. Each row-index entry then corrects that count on its own:
//   own symbol s at p       + [s is a difference at p] - [the local reference is]
//   covered region from s   + diff[s]                  (positions [0, s) hold the missing symbol)
//   covered region up to e  + diff[L] - diff[e]        (positions [e, L))
//   missing interval [a, z) - diff[a] ... + diff[z]    (one term per event)
// where diff[p] counts, over positions < p, the missing symbol's differences minus the local
// reference's. Null rows match no SymbolInSet, so they count no difference. A row is in the set
// when its count is at most the distance.
//
// One warp per 32 consecutive rows. Their entries are one contiguous range of the row index, read
// in windows of 256: each lane loads 8 consecutive entries as two 16-byte loads (the range is
// widened down to a 16-byte boundary, entries outside it count 0), looks up their terms and sums
// them locally; one warp scan over the lane sums places every entry's exclusive prefix in shared
// memory, where each row reads the prefix at its first entry. A row's count is the prefix at the
// next row's first entry minus the prefix at its own.
//   profile_staged_kernel  genomes up to 32,767 positions: the terms (mask u32, diff i16 per
//                          position, 6 bytes) staged in shared memory, one CTA of 1,024 threads
//                          per SM walking the row words;
//   profile_kernel         longer genomes: 8-byte terms read through L1/L2.
#include <cuda_runtime.h>

#include "device.h"

namespace rhygpu {

namespace {

constexpr uint32_t PT = 256;           // threads of profile_kernel
constexpr uint32_t ST = 1024;          // threads of profile_staged_kernel
constexpr uint32_t PU = 8;             // entries per lane per window
constexpr uint32_t PW = 32 * PU;       // entries per window
constexpr uint32_t STAGE_MAX_L = 32767;  // diff fits 16 bits

__device__ __forceinline__ int32_t event_term(uint32_t code, int32_t d, int32_t diff_L) {
   if (code == ROW_COV_START) return d;
   if (code == ROW_COV_END) return diff_L - d;
   if (code == ROW_MISS_START) return -d;
   return d;  // ROW_MISS_END
}

// Terms read from the interleaved global array.
struct GlobalTerms {
   const uint2* __restrict__ t;
   int32_t diff_L;
   __device__ __forceinline__ int32_t operator()(uint32_t ent) const {
      const uint32_t code = ent & 31u;
      const uint2 v = __ldg(t + (ent >> 5));
      if (code < ROW_COV_START) return static_cast<int32_t>((v.x >> code) & 1u) - static_cast<int32_t>(v.x >> 31);
      return event_term(code, static_cast<int32_t>(v.y), diff_L);
   }
};

// Terms read from shared memory.
struct StagedTerms {
   const uint32_t* mask;
   const int16_t* diff;
   int32_t diff_L;
   __device__ __forceinline__ int32_t operator()(uint32_t ent) const {
      const uint32_t code = ent & 31u, p = ent >> 5;
      if (code < ROW_COV_START) {
         const uint32_t m = mask[p];
         return static_cast<int32_t>((m >> code) & 1u) - static_cast<int32_t>(m >> 31);
      }
      return event_term(code, diff[p], diff_L);
   }
};

// Whole warp: the aux word of rows 32 w .. 32 w + 31. The row index holds 8 entries of readable
// tail past its end.
template <class Terms>
__device__ __forceinline__ void profile_word(const DevTable* __restrict__ tab, const DevSeqCol* __restrict__ cs,
                                             const DevProfile& pr, const Terms& terms, uint32_t w, int32_t* lp,
                                             uint32_t* __restrict__ aux_word) {
   const uint32_t lane = threadIdx.x & 31;
   const uint32_t r = 32 * w + lane;
   const uint32_t b0 = __ldg(cs->hrow_off + 32 * w);
   const uint32_t a0 = b0 & ~3u;  // 16-byte aligned start
   const uint32_t lo = b0 - a0, hi = lo + (__ldg(cs->hrow_off + 32 * w + 32) - b0);  // valid [lo, hi)
   const uint32_t f = lo + (__ldg(cs->hrow_off + r) - b0);  // this row's first entry
   const uint4* __restrict__ src = reinterpret_cast<const uint4*>(cs->hent + a0);
   int32_t S = 0;         // terms of the entries before the window
   int32_t at_first = 0;  // terms of the entries before this row's first
   for (uint32_t j0 = 0; j0 < hi; j0 += PW) {
      const uint32_t j = j0 + PU * lane;
      uint32_t ent[PU];
      if (j < hi) {
         const uint4 x = __ldg(src + j / 4), y = __ldg(src + j / 4 + 1);
         ent[0] = x.x, ent[1] = x.y, ent[2] = x.z, ent[3] = x.w, ent[4] = y.x, ent[5] = y.y, ent[6] = y.z, ent[7] = y.w;
      }
      int32_t c[PU], sum = 0;
#pragma unroll
      for (uint32_t u = 0; u < PU; ++u) {
         c[u] = (j + u >= lo && j + u < hi) ? terms(ent[u]) : 0;
         sum += c[u];
      }
      int32_t incl = sum;
#pragma unroll
      for (uint32_t o = 1; o < 32; o <<= 1) {
         const int32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
         if (lane >= o) incl += v;
      }
      int32_t run = S + incl - sum;
      int32_t ex[PU];
#pragma unroll
      for (uint32_t u = 0; u < PU; ++u) {
         ex[u] = run;
         run += c[u];
      }
      reinterpret_cast<int4*>(lp)[2 * lane] = make_int4(ex[0], ex[1], ex[2], ex[3]);
      reinterpret_cast<int4*>(lp)[2 * lane + 1] = make_int4(ex[4], ex[5], ex[6], ex[7]);
      __syncwarp();
      if (f >= j0 && f < j0 + PW) at_first = lp[f - j0];
      S += __shfl_sync(0xFFFFFFFFu, incl, 31);
      __syncwarp();
   }
   if (f >= hi) at_first = S;  // rows without entries at the end of the range
   const int32_t next = __shfl_down_sync(0xFFFFFFFFu, at_first, 1);
   const int32_t n = static_cast<int32_t>(pr.base) + (lane == 31 ? S : next) - at_first;
   const bool null_row = (__ldg(cs->null_tiles + w) >> lane) & 1u;
   const bool valid = (r & (CHUNK_ROWS - 1)) < __ldg(tab->chunk_sizes + (r >> 16));
   const bool in = valid && (null_row || n <= static_cast<int32_t>(min(pr.distance, 0x7FFFFFFFu)));
   const uint32_t bits = __ballot_sync(0xFFFFFFFFu, in);
   if (lane == 0) *aux_word = bits;
}

// grid (row words / 8, profiles)
__global__ void __launch_bounds__(PT) profile_kernel(const DevTable* __restrict__ tab,
                                                     const DevProfile* __restrict__ profiles,
                                                     uint32_t* __restrict__ aux) {
   __shared__ __align__(16) int32_t prefix[PT / 32][PW];
   const DevProfile pr = profiles[blockIdx.y];
   const DevSeqCol* cs = &tab->seq[pr.col];
   const uint32_t words = tab->nchunks * CHUNK_WORDS;
   const uint32_t w = (blockIdx.x * PT + threadIdx.x) >> 5;
   if (w >= words) return;  // the whole warp leaves
   const GlobalTerms terms{pr.terms, static_cast<int32_t>(__ldg(pr.terms + cs->L).y)};
   profile_word(tab, cs, pr, terms, w, prefix[threadIdx.x >> 5], aux + static_cast<size_t>(blockIdx.y) * words + w);
}

// grid (SMs, profiles), one CTA per SM; dynamic shared memory: the prefix windows, then mask[L],
// then diff[L + 1] as int16.
__global__ void __launch_bounds__(ST, 1) profile_staged_kernel(const DevTable* __restrict__ tab,
                                                               const DevProfile* __restrict__ profiles,
                                                               uint32_t* __restrict__ aux) {
   extern __shared__ __align__(16) int32_t sm_prefix[];
   const DevProfile pr = profiles[blockIdx.y];
   const DevSeqCol* cs = &tab->seq[pr.col];
   const uint32_t L = cs->L;
   uint32_t* mask = reinterpret_cast<uint32_t*>(sm_prefix + (ST / 32) * PW);
   int16_t* diff = reinterpret_cast<int16_t*>(mask + L);
   for (uint32_t p = threadIdx.x; p <= L; p += ST) {
      const uint2 v = __ldg(pr.terms + p);
      if (p < L) mask[p] = v.x;
      diff[p] = static_cast<int16_t>(static_cast<int32_t>(v.y));
   }
   __syncthreads();
   const StagedTerms terms{mask, diff, diff[L]};
   const uint32_t words = tab->nchunks * CHUNK_WORDS;
   int32_t* lp = sm_prefix + (threadIdx.x >> 5) * PW;
   uint32_t* out = aux + static_cast<size_t>(blockIdx.y) * words;
   for (uint32_t w = blockIdx.x * (ST / 32) + (threadIdx.x >> 5); w < words; w += gridDim.x * (ST / 32))
      profile_word(tab, cs, pr, terms, w, lp, out + w);
}

}  // namespace

void launch_profiles(const DevTable* d_table, uint32_t nchunks, const DevProfile* d_profiles, uint32_t n, uint32_t max_L,
                     uint32_t* d_aux, void* stream) {
   const uint32_t words = nchunks * CHUNK_WORDS;
   const cudaStream_t s = static_cast<cudaStream_t>(stream);
   const size_t smem = (ST / 32) * PW * 4 + static_cast<size_t>(max_L) * 4 + (static_cast<size_t>(max_L) + 1) * 2;
   int dev = 0, sms = 0, optin = 0;
   bool staged = max_L <= STAGE_MAX_L && cudaGetDevice(&dev) == cudaSuccess &&
                 cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
                 cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) == cudaSuccess &&
                 smem <= static_cast<size_t>(optin) &&
                 cudaFuncSetAttribute(profile_staged_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(smem)) == cudaSuccess;
   for (uint32_t k = 0; k < n; k += 65535) {  // grid.y is at most 65535
      const uint32_t m = n - k < 65535 ? n - k : 65535;
      if (staged)
         profile_staged_kernel<<<dim3(sms, m), ST, smem, s>>>(d_table, d_profiles + k, d_aux + static_cast<size_t>(k) * words);
      else
         profile_kernel<<<dim3((words + PT / 32 - 1) / (PT / 32), m), PT, 0, s>>>(d_table, d_profiles + k,
                                                                                 d_aux + static_cast<size_t>(k) * words);
   }
}

}  // namespace rhygpu
