// Ingestion of the sequence columns on the GPU (see ingest.h).
//
// Per sequence column (reference: SequenceColumn::appendChunk + finalize,
// src/rhydb/storage/column/sequence_column.cpp:100-212, and extractCoverageAndMutationsFromSequence,
// src/rhydb/common/aligned_sequence.cpp:19-122):
//   1. rows_kernel (two passes: count, then emit), one thread per row: the row's covered region
//      (first to last position that is not missing), its missing intervals inside it (maximal
//      stretches of missing positions, reference-missing positions included), and one key
//      (row, position, symbol) per position whose symbol differs from the reference;
//   2. per position the covered rows (difference array) and per (position, symbol) the keys: the
//      local reference flips where another symbol strictly exceeds it (symbols in alphabet order);
//   3. flip_kernel: per chunk and flipped position the rows that now hold the old reference
//      (covered, no key there), as a bitmap; the keys of the new reference symbol are dropped;
//   4. the keys are counted per (chunk, position, symbol) bucket, scattered into their buckets and
//      each bucket is sorted (a warp sort for small buckets, a shared-memory bitmap for larger ones);
//   5. every bucket becomes a container by the host's rules (array <= 4096 rows, bitset, or runs
//      when smaller) laid out as the host lays it out: per chunk the arrays back to back in
//      descriptor order, then the bitsets (16-byte aligned) and runs in descriptor order.
// The host then finishes the column from the per-chunk row records and the containers, with the
// same code as host ingestion (finish_seq_column). The image equals the host-built one.
#include "ingest.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <stdexcept>
#include <string>
#include <vector>

#include "alphabet.h"
#include "engine.h"
#include "table_build.h"
#include "util.h"

namespace rhygpu {

namespace {

constexpr uint32_t SCAN_BLOCK = 256, SCAN_ITEMS = 8, SCAN_TILE = SCAN_BLOCK * SCAN_ITEMS;

// ---------------------------------------------------------------------------------------------
// Exclusive prefix sums (three launches: tile sums, a scan of the tile sums, tile scans).

template <typename T>
__device__ T block_scan_excl(T x, T* wsum, T* total) {
   const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
   T incl = x;
#pragma unroll
   for (uint32_t o = 1; o < 32; o <<= 1) {
      const T y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
      if (lane >= o) incl += y;
   }
   if (lane == 31) wsum[warp] = incl;
   __syncthreads();
   T before = 0, all = 0;
   for (uint32_t w = 0; w < nw; ++w) {
      const T v = wsum[w];
      before += w < warp ? v : T(0);
      all += v;
   }
   __syncthreads();
   *total = all;
   return before + incl - x;
}

template <typename T>
__global__ void __launch_bounds__(SCAN_BLOCK) tile_sums_kernel(const T* in, size_t n, T* sums) {
   __shared__ T wsum[SCAN_BLOCK / 32];
   const size_t base = static_cast<size_t>(blockIdx.x) * SCAN_TILE;
   T s = 0;
   for (uint32_t i = 0; i < SCAN_ITEMS; ++i) {
      const size_t k = base + static_cast<size_t>(i) * SCAN_BLOCK + threadIdx.x;
      if (k < n) s += in[k];
   }
   T total;
   block_scan_excl<T>(s, wsum, &total);
   if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// One block: exclusive scan of the tile sums in place, *grand receives the total.
template <typename T>
__global__ void __launch_bounds__(SCAN_BLOCK) scan_sums_kernel(T* sums, size_t n, T* grand) {
   __shared__ T wsum[SCAN_BLOCK / 32];
   T carry = 0;
   for (size_t base = 0; base < n; base += SCAN_BLOCK) {
      const size_t k = base + threadIdx.x;
      const T x = k < n ? sums[k] : T(0);
      T total;
      const T ex = block_scan_excl<T>(x, wsum, &total);
      if (k < n) sums[k] = carry + ex;
      carry += total;
   }
   if (threadIdx.x == 0) *grand = carry;
}

template <typename T>
__global__ void __launch_bounds__(SCAN_BLOCK) tile_scan_kernel(const T* in, size_t n, const T* sums, T* out) {
   __shared__ T wsum[SCAN_BLOCK / 32];
   const size_t base = static_cast<size_t>(blockIdx.x) * SCAN_TILE + static_cast<size_t>(threadIdx.x) * SCAN_ITEMS;
   T v[SCAN_ITEMS];
   T s = 0;
   for (uint32_t i = 0; i < SCAN_ITEMS; ++i) {
      const size_t k = base + i;
      v[i] = k < n ? in[k] : T(0);
      s += v[i];
   }
   T total;
   T run = sums[blockIdx.x] + block_scan_excl<T>(s, wsum, &total);
   for (uint32_t i = 0; i < SCAN_ITEMS; ++i) {
      const size_t k = base + i;
      if (k < n) out[k] = run;
      run += v[i];
   }
}

// Device buffers of one column build, freed together.
struct Arena {
   std::vector<void*> ptrs;
   template <typename T>
   T* get(size_t n) {
      void* p = nullptr;
      cuda_check(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)), "cudaMalloc (ingestion)");
      ptrs.push_back(p);
      return static_cast<T*>(p);
   }
   ~Arena() {
      for (void* p : ptrs) cudaFree(p);
   }
};

template <typename T>
T exclusive_scan(Arena& a, const T* in, T* out, size_t n, cudaStream_t s) {
   const size_t tiles = std::max<size_t>(1, (n + SCAN_TILE - 1) / SCAN_TILE);
   T* sums = a.get<T>(tiles);
   T* grand = a.get<T>(1);
   tile_sums_kernel<T><<<static_cast<uint32_t>(tiles), SCAN_BLOCK, 0, s>>>(in, n, sums);
   scan_sums_kernel<T><<<1, SCAN_BLOCK, 0, s>>>(sums, tiles, grand);
   tile_scan_kernel<T><<<static_cast<uint32_t>(tiles), SCAN_BLOCK, 0, s>>>(in, n, sums, out);
   cuda_check(cudaGetLastError(), "scan launch");
   T total = 0;
   cuda_check(cudaMemcpyAsync(&total, grand, sizeof(T), cudaMemcpyDeviceToHost, s), "scan total");
   cuda_check(cudaStreamSynchronize(s), "scan");
   return total;
}

// ---------------------------------------------------------------------------------------------
// 1. Rows

struct RowInput {
   const uint64_t* row_off;   // n_rows + 1
   const uint32_t* run_pos;
   const uint32_t* run_len;
   const uint8_t* run_char;
   const uint8_t* is_null;    // n_rows
   const int8_t* c2s;         // 256: symbol of a character, -1 = illegal
   const uint8_t* ref_sym;    // L: global reference symbols
   const uint32_t* next_ok;   // L + 1: smallest q >= p whose reference symbol is not missing (L: none)
   const uint32_t* prev_ok;   // L + 1: 1 + the largest q < p whose reference symbol is not missing (0: none)
   const uint2* ref_miss;     // maximal intervals [x, y) where the reference symbol is missing, sorted
   uint32_t n_ref_miss;
   uint32_t L, missing, n_rows;
};

struct RowOutput {
   uint64_t* nkeys;    // pass 0: keys per row; pass 1: their offsets
   uint32_t* nint;     // missing intervals per row / offsets
   uint32_t* nexc;     // 1 if the row is a coverage exception / offsets
   uint64_t* keys;     // pass 1: (global row << 32) | (position << 5) | symbol
   uint2* ints;        // pass 1: [start, end) of each missing interval
   CovExc* exc;        // pass 1: {row in chunk, start, end}
   int* diff;          // pass 1: L + 1 covered-row difference array (full rows go to *full)
   unsigned long long* full;
   unsigned long long* err;  // smallest (row << 32 | run index) of an illegal character
};

template <int PASS>
__global__ void __launch_bounds__(256) rows_kernel(RowInput in, RowOutput out) {
   const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
   bool full_row = false;
   if (g < in.n_rows) {
      const uint32_t L = in.L, M = in.missing, r = g & 0xFFFFu;
      uint64_t nk = 0;
      uint32_t ni = 0, ne = 0;
      uint64_t ko = 0;
      uint32_t io = 0, eo = 0;
      if (PASS == 1) {
         ko = out.nkeys[g];
         io = out.nint[g];
         eo = out.nexc[g];
      }
      if (in.is_null[g]) {
         ne = 1;
         if (PASS == 1) out.exc[eo] = CovExc{r, 0, 0, 0};
      } else {
         const uint64_t b = in.row_off[g], e = in.row_off[g + 1];
         // covered region: the first and one past the last position that is not missing
         uint32_t start = L, cursor = 0;
         bool bad = false;
         for (uint64_t k = b; k < e && start == L; ++k) {
            const uint32_t p0 = in.run_pos[k];
            const int s = in.c2s[in.run_char[k]];
            const uint32_t q = in.next_ok[cursor];
            if (q < p0) {
               start = q;
               break;
            }
            if (s >= 0 && static_cast<uint32_t>(s) != M) start = p0;
            cursor = p0 + in.run_len[k];
         }
         if (start == L) start = in.next_ok[cursor] < L ? in.next_ok[cursor] : L;
         uint32_t end = 0;
         bool found = false;
         uint32_t cend = L;
         for (uint64_t k = e; k > b; --k) {
            const uint32_t p0 = in.run_pos[k - 1], len = in.run_len[k - 1];
            const int s = in.c2s[in.run_char[k - 1]];
            const uint32_t t = in.prev_ok[cend];
            if (t > p0 + len) {
               end = t;
               found = true;
               break;
            }
            if (s >= 0 && static_cast<uint32_t>(s) != M) {
               end = p0 + len;
               found = true;
               break;
            }
            cend = p0;
         }
         if (!found) end = in.prev_ok[cend];
         for (uint64_t k = b; k < e; ++k)
            if (in.c2s[in.run_char[k]] < 0) {
               bad = true;
               atomicMin(out.err, (static_cast<unsigned long long>(g) << 32) | static_cast<unsigned long long>(k - b));
               break;
            }
         if (bad || start >= end) {
            ne = 1;  // fully missing (or rejected): empty covered region, nothing recorded
            if (PASS == 1) out.exc[eo] = CovExc{r, 0, 0, 0};
         } else {
            if (start != 0 || end != L) {
               ne = 1;
               if (PASS == 1) {
                  out.exc[eo] = CovExc{r, start, end, 0};
                  atomicAdd(&out.diff[start], 1);
                  atomicAdd(&out.diff[end], -1);
               }
            } else {
               full_row = true;
            }
            // keys and missing intervals, in position order
            uint32_t cs = 0, ce = 0;  // the open missing interval [cs, ce), empty when cs == ce
            auto segment = [&](uint32_t a, uint32_t z) {  // a missing stretch [a, z)
               if (a < start || a >= end) return;     // leading / trailing: outside coverage
               if (cs != ce && ce == a) {
                  ce = z;
                  return;
               }
               if (cs != ce) {
                  if (PASS == 1) {
                     out.ints[io + ni] = make_uint2(cs, ce);
                     atomicAdd(&out.diff[cs], -1);
                     atomicAdd(&out.diff[ce], 1);
                  }
                  ++ni;
               }
               cs = a;
               ce = z;
            };
            auto ref_gaps = [&](uint32_t a, uint32_t z) {  // reference-missing stretches in [a, z)
               if (in.n_ref_miss == 0 || a >= z) return;
               uint32_t lo = 0, hi = in.n_ref_miss;  // first interval ending after a
               while (lo < hi) {
                  const uint32_t mid = (lo + hi) / 2;
                  if (in.ref_miss[mid].y <= a) lo = mid + 1;
                  else hi = mid;
               }
               for (uint32_t t = lo; t < in.n_ref_miss && in.ref_miss[t].x < z; ++t)
                  segment(max(a, in.ref_miss[t].x), min(z, in.ref_miss[t].y));
            };
            cursor = 0;
            for (uint64_t k = b; k < e; ++k) {
               const uint32_t p0 = in.run_pos[k], len = in.run_len[k];
               const uint32_t s = static_cast<uint32_t>(in.c2s[in.run_char[k]]);
               ref_gaps(cursor, p0);
               if (s == M) {
                  segment(p0, p0 + len);
               } else {
                  for (uint32_t p = p0; p < p0 + len; ++p) {
                     if (s != in.ref_sym[p]) {
                        if (PASS == 1)
                           out.keys[ko + nk] = (static_cast<uint64_t>(g) << 32) | (static_cast<uint64_t>(p) << 5) | s;
                        ++nk;
                     }
                  }
               }
               cursor = p0 + len;
            }
            ref_gaps(cursor, L);
            if (cs != ce) {
               if (PASS == 1) {
                  out.ints[io + ni] = make_uint2(cs, ce);
                  atomicAdd(&out.diff[cs], -1);
                  atomicAdd(&out.diff[ce], 1);
               }
               ++ni;
            }
         }
      }
      if (PASS == 0) {
         out.nkeys[g] = nk;
         out.nint[g] = ni;
         out.nexc[g] = ne;
      }
   }
   if (PASS == 1) {  // full rows, counted per warp
      const uint32_t n = __popc(__ballot_sync(0xFFFFFFFFu, full_row));
      if ((threadIdx.x & 31) == 0 && n) atomicAdd(out.full, static_cast<unsigned long long>(n));
   }
}

// ---------------------------------------------------------------------------------------------
// 2. Counts, coverage and the local-reference flips

// Keys per (chunk, position, symbol) bucket and per (position, symbol).
__global__ void count_keys_kernel(const uint64_t* keys, uint64_t n, uint32_t L, uint32_t nsym, uint32_t* hist,
                                  uint32_t* ps) {
   for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
        i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
      const uint64_t k = keys[i];
      const uint32_t v = static_cast<uint32_t>(k >> 48), ps_ = static_cast<uint32_t>(k);
      const uint32_t p = ps_ >> 5, s = ps_ & 31u;
      atomicAdd(&hist[(static_cast<size_t>(v) * L + p) * nsym + s], 1u);
      atomicAdd(&ps[static_cast<size_t>(p) * nsym + s], 1u);
   }
}

// Per position: the symbol that becomes the local reference (flip[p] = new symbol, or 0xFF).
// Reference: VerticalSequenceIndex::getSymbolWithHighestCount, vertical_sequence_index.cpp:79-116
// (the current reference keeps its place unless another symbol has strictly more rows).
__global__ void flips_kernel(const int* cover, const uint32_t* ps, const uint8_t* ref, uint32_t L, uint32_t nsym,
                             uint8_t* flip) {
   const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
   if (p >= L) return;
   const uint32_t r = ref[p];
   uint32_t ref_count = static_cast<uint32_t>(cover[p]);
   for (uint32_t s = 0; s < nsym; ++s) ref_count -= ps[static_cast<size_t>(p) * nsym + s];
   uint32_t best = r, best_count = ref_count;
   for (uint32_t s = 0; s < nsym; ++s) {
      if (s == r) continue;
      const uint32_t c = ps[static_cast<size_t>(p) * nsym + s];
      if (c > best_count) {
         best = s;
         best_count = c;
      }
   }
   flip[p] = best != r ? static_cast<uint8_t>(best) : 0xFFu;
}

// 3. One CTA per (chunk, group of up to FLIP_GROUP flipped positions): the rows of the chunk that
// hold the old reference symbol at each position (covered, not in a missing interval there, and
// without a key there), as 8 KiB bitmaps, and their counts.
constexpr uint32_t FLIP_GROUP = 16;
__global__ void __launch_bounds__(256) flip_rows_kernel(const uint32_t* flip_pos, uint32_t n_flip, uint32_t n_rows,
                                                        const uint8_t* is_null, const uint64_t* key_off,
                                                        const uint64_t* keys, const uint32_t* int_off,
                                                        const uint2* ints, const uint32_t* exc_off, const CovExc* exc,
                                                        uint32_t* bits_out, uint32_t* counts_out) {
   extern __shared__ uint32_t bm[];  // FLIP_GROUP * CHUNK_WORDS
   const uint32_t v = blockIdx.x, f0 = blockIdx.y * FLIP_GROUP;
   const uint32_t nf = min(FLIP_GROUP, n_flip - f0);
   const uint32_t g0 = v * CHUNK_ROWS, g1 = min(n_rows, g0 + CHUNK_ROWS), size = g1 - g0;
   for (uint32_t j = 0; j < nf; ++j)
      for (uint32_t w = threadIdx.x; w < CHUNK_WORDS; w += blockDim.x) {
         const uint32_t lo = 32 * w;
         bm[j * CHUNK_WORDS + w] = lo + 32 <= size ? 0xFFFFFFFFu : (lo < size ? (1u << (size - lo)) - 1u : 0u);
      }
   __syncthreads();
   // coverage exceptions (null and fully missing rows included): rows not covering the position
   for (uint32_t i = exc_off[g0] + threadIdx.x; i < exc_off[g1]; i += blockDim.x) {
      const CovExc x = exc[i];
      for (uint32_t j = 0; j < nf; ++j) {
         const uint32_t f = flip_pos[f0 + j];
         if (!(x.start <= f && f < x.end)) atomicAnd(&bm[j * CHUNK_WORDS + (x.row >> 5)], ~(1u << (x.row & 31)));
      }
   }
   // missing intervals and keys at the position
   for (uint32_t g = g0 + threadIdx.x; g < g1; g += blockDim.x) {
      const uint32_t r = g - g0;
      if (is_null[g]) continue;
      for (uint32_t q = int_off[g]; q < int_off[g + 1]; ++q) {
         const uint2 iv = ints[q];
         for (uint32_t j = 0; j < nf; ++j) {
            const uint32_t f = flip_pos[f0 + j];
            if (iv.x <= f && f < iv.y) atomicAnd(&bm[j * CHUNK_WORDS + (r >> 5)], ~(1u << (r & 31)));
         }
      }
      for (uint64_t q = key_off[g]; q < key_off[g + 1]; ++q) {
         const uint32_t p = static_cast<uint32_t>(keys[q]) >> 5;
         for (uint32_t j = 0; j < nf; ++j)
            if (p == flip_pos[f0 + j]) atomicAnd(&bm[j * CHUNK_WORDS + (r >> 5)], ~(1u << (r & 31)));
      }
   }
   __syncthreads();
   for (uint32_t j = 0; j < nf; ++j) {
      uint32_t c = 0;
      uint32_t* dst = bits_out + (static_cast<size_t>(f0 + j) * gridDim.x + v) * CHUNK_WORDS;
      for (uint32_t w = threadIdx.x; w < CHUNK_WORDS; w += blockDim.x) {
         const uint32_t x = bm[j * CHUNK_WORDS + w];
         dst[w] = x;
         c += __popc(x);
      }
      c = __reduce_add_sync(0xFFFFFFFFu, c);
      if ((threadIdx.x & 31) == 0 && c) atomicAdd(&counts_out[(f0 + j) * gridDim.x + v], c);
   }
}

// ---------------------------------------------------------------------------------------------
// 4. Buckets

// The bucket counts with the flips applied: the new reference symbol's keys are dropped, the old
// one's bucket holds the flip rows.
__global__ void flip_hist_kernel(const uint32_t* flip_pos, const uint8_t* flip_new, const uint8_t* old_ref,
                                 uint32_t n_flip, uint32_t nchunks, uint32_t L, uint32_t nsym, const uint32_t* flip_counts,
                                 uint32_t* hist) {
   const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n_flip * nchunks) return;
   const uint32_t j = i / nchunks, v = i % nchunks, f = flip_pos[j];
   const size_t base = (static_cast<size_t>(v) * L + f) * nsym;
   hist[base + flip_new[f]] = 0;
   hist[base + old_ref[f]] = flip_counts[i];
}

__global__ void scatter_keys_kernel(const uint64_t* keys, uint64_t n, uint32_t L, uint32_t nsym, const uint8_t* flip,
                                    uint32_t* cursor, uint16_t* rows) {
   for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
        i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
      const uint64_t k = keys[i];
      const uint32_t g = static_cast<uint32_t>(k >> 32), ps_ = static_cast<uint32_t>(k);
      const uint32_t p = ps_ >> 5, s = ps_ & 31u, v = g >> 16;
      if (flip[p] == s) continue;  // the new local reference is not stored
      const uint32_t at = atomicAdd(&cursor[(static_cast<size_t>(v) * L + p) * nsym + s], 1u);
      rows[at] = static_cast<uint16_t>(g & 0xFFFFu);
   }
}

// The flip rows of (flip j, chunk v), in row order, into the old reference's bucket.
__global__ void __launch_bounds__(256) flip_scatter_kernel(const uint32_t* flip_pos, const uint8_t* old_ref,
                                                           uint32_t nchunks, uint32_t L, uint32_t nsym,
                                                           const uint32_t* bits, const uint32_t* boff, uint16_t* rows) {
   __shared__ uint32_t wsum[8];
   const uint32_t j = blockIdx.y, v = blockIdx.x, f = flip_pos[j];
   const uint32_t* bm = bits + (static_cast<size_t>(j) * nchunks + v) * CHUNK_WORDS;
   uint32_t at = boff[(static_cast<size_t>(v) * L + f) * nsym + old_ref[f]];
   for (uint32_t w0 = 0; w0 < CHUNK_WORDS; w0 += blockDim.x) {
      const uint32_t w = w0 + threadIdx.x;
      const uint32_t x = bm[w];
      uint32_t total;
      const uint32_t ex = block_scan_excl<uint32_t>(__popc(x), wsum, &total);
      uint32_t o = at + ex;
      for (uint32_t y = x; y; y &= y - 1) rows[o++] = static_cast<uint16_t>(32 * w + __ffs(y) - 1);
      at += total;
   }
}

// 5. Per non-empty bucket, one warp: sort its rows (in place), count its runs and choose its
// container: array (<= 4096 rows), bitset, or runs when 4 * runs + 2 bytes are fewer than the
// array's 2 * rows + 2 or the bitset's 8 KiB (reference: RoaringContainer::runOptimize,
// roaring_container.cpp:7-62, by the public Roaring size rules).
constexpr uint32_t SORT_WARPS = 4;  // 8 KiB bitmap per warp: 32 KiB of static shared memory
__global__ void __launch_bounds__(SORT_WARPS * 32) sort_buckets_kernel(const uint32_t* list, uint32_t n_list,
                                                                       const uint32_t* hist, const uint32_t* boff,
                                                                       uint16_t* rows, uint32_t* nruns_out,
                                                                       uint8_t* type_out) {
   __shared__ uint32_t bm[SORT_WARPS][CHUNK_WORDS];
   const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
   for (uint32_t li = blockIdx.x * SORT_WARPS + warp; li < n_list; li += gridDim.x * SORT_WARPS) {
      const uint32_t b = list[li], card = hist[b];
      uint16_t* seg = rows + boff[b];
      if (card <= 32) {  // bitonic sort of up to 32 rows in the lanes, padded with 0xFFFF
         uint32_t x = lane < card ? seg[lane] : 0xFFFFu;
         for (uint32_t k = 2; k <= 32; k <<= 1) {
            for (uint32_t j = k >> 1; j > 0; j >>= 1) {
               const uint32_t y = __shfl_xor_sync(0xFFFFFFFFu, x, j);
               const bool up = (lane & k) == 0, lower = (lane & j) == 0;
               x = (lower == up) ? min(x, y) : max(x, y);
            }
         }
         if (lane < card) seg[lane] = static_cast<uint16_t>(x);
         const uint32_t prev = __shfl_up_sync(0xFFFFFFFFu, x, 1);
         const bool starts = lane < card && (lane == 0 || x != prev + 1);
         const uint32_t nr = __popc(__ballot_sync(0xFFFFFFFFu, starts));
         if (lane == 0) {
            nruns_out[li] = nr;
            type_out[li] = (2 + 4 * nr < 2 + 2 * card) ? CT_RUN : CT_ARRAY;
         }
         continue;
      }
      // larger buckets: a bitmap of the chunk's rows in shared memory, then the rows in order
      uint32_t* m = bm[warp];
      for (uint32_t w = lane; w < CHUNK_WORDS; w += 32) m[w] = 0;
      __syncwarp();
      for (uint32_t i = lane; i < card; i += 32) {
         const uint32_t r = seg[i];
         atomicOr(&m[r >> 5], 1u << (r & 31));
      }
      __syncwarp();
      // lane l owns words 64 l .. 64 l + 63: its rows are written after the rows of lanes < l
      uint32_t c = 0, starts = 0;
      for (uint32_t t = 0; t < 64; ++t) {
         const uint32_t w = 64 * lane + t, x = m[w];
         const uint32_t carry = w > 0 ? (m[w - 1] >> 31) : 0u;  // the previous row is set
         c += __popc(x);
         starts += __popc(x & ~((x << 1) | carry));
      }
      uint32_t incl = c;
#pragma unroll
      for (uint32_t o = 1; o < 32; o <<= 1) {
         const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
         if (lane >= o) incl += y;
      }
      uint32_t at = incl - c;
      for (uint32_t t = 0; t < 64; ++t) {
         const uint32_t w = 64 * lane + t;
         for (uint32_t x = m[w]; x; x &= x - 1) seg[at++] = static_cast<uint16_t>(32 * w + __ffs(x) - 1);
      }
      const uint32_t nr = __reduce_add_sync(0xFFFFFFFFu, starts);
      if (lane == 0) {
         nruns_out[li] = nr;
         const uint32_t base_bytes = card <= 4096 ? 2 + 2 * card : 8192;
         type_out[li] = (2 + 4 * nr < base_bytes) ? CT_RUN : (card <= 4096 ? CT_ARRAY : CT_BITSET);
      }
      __syncwarp();
   }
}

// Payload of each container at its offset: the sorted rows (array), the bitmap (bitset) or
// (start, length - 1) pairs (runs). One warp per container.
__global__ void __launch_bounds__(256) write_payload_kernel(const uint32_t* list, uint32_t n_list, const uint32_t* hist,
                                                            const uint32_t* boff, const uint16_t* rows,
                                                            const uint8_t* type, const uint32_t* poff, uint16_t* payload) {
   const uint32_t lane = threadIdx.x & 31;
   for (uint32_t li = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; li < n_list; li += (gridDim.x * blockDim.x) >> 5) {
      const uint32_t b = list[li], card = hist[b];
      const uint16_t* seg = rows + boff[b];
      uint16_t* dst = payload + poff[li];
      if (type[li] == CT_ARRAY) {
         for (uint32_t i = lane; i < card; i += 32) dst[i] = seg[i];
      } else if (type[li] == CT_BITSET) {
         uint32_t* d32 = reinterpret_cast<uint32_t*>(dst);  // 16-byte aligned
         for (uint32_t w = lane; w < CHUNK_WORDS; w += 32) d32[w] = 0;
         __syncwarp();
         for (uint32_t i = lane; i < card; i += 32) atomicOr(&d32[seg[i] >> 5], 1u << (seg[i] & 31));
      } else if (lane == 0) {  // runs: sequential, a run container has few runs
         uint32_t k = 0, o = 0;
         while (k < card) {
            uint32_t e = k;
            while (e + 1 < card && seg[e + 1] == seg[e] + 1) ++e;
            dst[o++] = seg[k];
            dst[o++] = static_cast<uint16_t>(e - k);
            k = e + 1;
         }
      }
   }
}

__global__ void list_buckets_kernel(const uint32_t* hist, const uint32_t* lofs, size_t n, uint32_t* list) {
   for (size_t b = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; b < n;
        b += static_cast<size_t>(gridDim.x) * blockDim.x)
      if (hist[b]) list[lofs[b]] = static_cast<uint32_t>(b);
}

__global__ void nonzero_kernel(const uint32_t* hist, size_t n, uint32_t* flag) {
   for (size_t b = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; b < n;
        b += static_cast<size_t>(gridDim.x) * blockDim.x)
      flag[b] = hist[b] ? 1u : 0u;
}

uint32_t grid_for(size_t n, uint32_t block) {  // at least one block: a launch of none is an error
   return static_cast<uint32_t>(std::max<size_t>(1, std::min<size_t>((n + block - 1) / block, 1u << 20)));
}

template <typename T>
T* to_device(Arena& a, const std::vector<T>& v, cudaStream_t s) {
   T* p = a.get<T>(v.size());
   if (!v.empty()) cuda_check(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s), "H2D");
   return p;
}

template <typename T>
std::vector<T> to_host(const T* p, size_t n, cudaStream_t s) {
   std::vector<T> v(n);
   if (n) cuda_check(cudaMemcpyAsync(v.data(), p, n * sizeof(T), cudaMemcpyDeviceToHost, s), "D2H");
   cuda_check(cudaStreamSynchronize(s), "D2H");
   return v;
}

// One sequence column on the GPU.
SeqColumnImage build_seq_column_gpu(const RawSeqColumn& raw, const std::vector<uint32_t>& chunk_sizes, uint32_t threads,
                                    cudaStream_t st) {
   SeqColumnImage col;
   init_seq_column(raw, col);
   const Alphabet& A = alphabet(raw.kind);
   const uint32_t L = col.L, nsym = A.count, M = A.missing;
   const uint32_t nchunks = static_cast<uint32_t>(chunk_sizes.size());
   const uint32_t n_rows = static_cast<uint32_t>(raw.is_null.size());
   Arena a;

   // inputs
   std::vector<int8_t> c2s(256);
   for (int c = 0; c < 256; ++c) c2s[c] = A.char_to_sym[c];
   std::vector<uint32_t> next_ok(L + 1), prev_ok(L + 1);
   next_ok[L] = L;
   for (uint32_t p = L; p-- > 0;) next_ok[p] = col.global_ref[p] != M ? p : next_ok[p + 1];
   prev_ok[0] = 0;
   for (uint32_t p = 1; p <= L; ++p) prev_ok[p] = col.global_ref[p - 1] != M ? p : prev_ok[p - 1];
   std::vector<uint2> ref_miss;
   for (uint32_t p = 0; p < L; ++p) {
      if (col.global_ref[p] != M) continue;
      if (!ref_miss.empty() && ref_miss.back().y == p) ref_miss.back().y = p + 1;
      else ref_miss.push_back(make_uint2(p, p + 1));
   }
   RowInput in{};
   in.row_off = to_device(a, raw.row_off, st);
   in.run_pos = to_device(a, raw.run_pos, st);
   in.run_len = to_device(a, raw.run_len, st);
   {
      uint8_t* rc = a.get<uint8_t>(raw.run_char.size());
      if (!raw.run_char.empty())
         cuda_check(cudaMemcpyAsync(rc, raw.run_char.data(), raw.run_char.size(), cudaMemcpyHostToDevice, st), "H2D");
      in.run_char = rc;
   }
   in.is_null = to_device(a, raw.is_null, st);
   in.c2s = to_device(a, c2s, st);
   in.ref_sym = to_device(a, col.global_ref, st);
   in.next_ok = to_device(a, next_ok, st);
   in.prev_ok = to_device(a, prev_ok, st);
   in.ref_miss = to_device(a, ref_miss, st);
   in.n_ref_miss = static_cast<uint32_t>(ref_miss.size());
   in.L = L;
   in.missing = M;
   in.n_rows = n_rows;

   // 1. rows: count, scan, emit
   RowOutput out{};
   uint64_t* nk = a.get<uint64_t>(n_rows + 1);
   uint32_t* ni = a.get<uint32_t>(n_rows + 1);
   uint32_t* ne = a.get<uint32_t>(n_rows + 1);
   uint64_t* ko = a.get<uint64_t>(n_rows + 1);
   uint32_t* io = a.get<uint32_t>(n_rows + 1);
   uint32_t* eo = a.get<uint32_t>(n_rows + 1);
   out.nkeys = nk;
   out.nint = ni;
   out.nexc = ne;
   out.err = a.get<unsigned long long>(1);
   const unsigned long long no_err = ~0ull;
   cuda_check(cudaMemcpyAsync(out.err, &no_err, sizeof(no_err), cudaMemcpyHostToDevice, st), "H2D");
   cuda_check(cudaMemsetAsync(nk + n_rows, 0, sizeof(uint64_t), st), "memset");
   cuda_check(cudaMemsetAsync(ni + n_rows, 0, sizeof(uint32_t), st), "memset");
   cuda_check(cudaMemsetAsync(ne + n_rows, 0, sizeof(uint32_t), st), "memset");
   rows_kernel<0><<<(n_rows + 255) / 256, 256, 0, st>>>(in, out);
   cuda_check(cudaGetLastError(), "rows kernel");
   unsigned long long err = 0;
   cuda_check(cudaMemcpyAsync(&err, out.err, sizeof(err), cudaMemcpyDeviceToHost, st), "D2H");
   cuda_check(cudaStreamSynchronize(st), "rows kernel");
   if (err != ~0ull) {
      const uint32_t row = static_cast<uint32_t>(err >> 32);
      const uint64_t k = raw.row_off[row] + (err & 0xFFFFFFFFull);
      throw std::invalid_argument(std::string("illegal character '") + raw.run_char[k] + "' at position " +
                                  std::to_string(raw.run_pos[k]) + " in the input sequence (column " + raw.name +
                                  ", row " + std::to_string(row) + ")");
   }
   const uint64_t total_keys = exclusive_scan<uint64_t>(a, nk, ko, n_rows + 1, st);
   if (total_keys > 0xFFFFFFFFull) throw std::invalid_argument("column " + raw.name + ": more than 2^32 stored symbols");
   const uint32_t total_ints = exclusive_scan<uint32_t>(a, ni, io, n_rows + 1, st);
   const uint32_t total_exc = exclusive_scan<uint32_t>(a, ne, eo, n_rows + 1, st);
   out.nkeys = ko;
   out.nint = io;
   out.nexc = eo;
   out.keys = a.get<uint64_t>(total_keys);
   out.ints = a.get<uint2>(total_ints);
   out.exc = a.get<CovExc>(total_exc);
   out.diff = a.get<int>(L + 1);
   out.full = a.get<unsigned long long>(1);
   cuda_check(cudaMemsetAsync(out.diff, 0, (L + 1) * sizeof(int), st), "memset");
   cuda_check(cudaMemsetAsync(out.full, 0, sizeof(unsigned long long), st), "memset");
   rows_kernel<1><<<(n_rows + 255) / 256, 256, 0, st>>>(in, out);
   cuda_check(cudaGetLastError(), "rows kernel");

   // 2. counts, coverage, flips
   const size_t nb = static_cast<size_t>(nchunks) * L * nsym;  // buckets (chunk, position, symbol)
   uint32_t* hist = a.get<uint32_t>(nb);
   uint32_t* ps = a.get<uint32_t>(static_cast<size_t>(L) * nsym);
   cuda_check(cudaMemsetAsync(hist, 0, nb * sizeof(uint32_t), st), "memset");
   cuda_check(cudaMemsetAsync(ps, 0, static_cast<size_t>(L) * nsym * sizeof(uint32_t), st), "memset");
   // keys carry the chunk in bits 48..63 of the global row: (row << 32) >> 48 = row >> 16
   count_keys_kernel<<<grid_for(total_keys, 256), 256, 0, st>>>(out.keys, total_keys, L, nsym, hist, ps);
   unsigned long long full = 0;
   cuda_check(cudaMemcpyAsync(&full, out.full, sizeof(full), cudaMemcpyDeviceToHost, st), "D2H");
   std::vector<int> diff = to_host(out.diff, L + 1, st);
   std::vector<int> cover(L);
   {
      long long run = static_cast<long long>(full);
      for (uint32_t p = 0; p < L; ++p) {
         run += diff[p];
         cover[p] = static_cast<int>(run);
      }
   }
   int* d_cover = to_device(a, cover, st);
   uint8_t* d_flip = a.get<uint8_t>(L);
   flips_kernel<<<(L + 255) / 256, 256, 0, st>>>(d_cover, ps, in.ref_sym, L, nsym, d_flip);
   std::vector<uint8_t> flip = to_host(d_flip, L, st);
   std::vector<uint32_t> flip_pos;
   for (uint32_t p = 0; p < L; ++p)
      if (flip[p] != 0xFFu) flip_pos.push_back(p);
   const uint32_t n_flip = static_cast<uint32_t>(flip_pos.size());
   col.flipped_positions = n_flip;

   // 3. flip rows
   uint32_t* d_flip_pos = to_device(a, flip_pos, st);
   uint32_t* flip_bits = nullptr;
   if (n_flip) {
      flip_bits = a.get<uint32_t>(static_cast<size_t>(n_flip) * nchunks * CHUNK_WORDS);
      uint32_t* flip_counts = a.get<uint32_t>(static_cast<size_t>(n_flip) * nchunks);
      cuda_check(cudaMemsetAsync(flip_counts, 0, static_cast<size_t>(n_flip) * nchunks * sizeof(uint32_t), st), "memset");
      const size_t smem = FLIP_GROUP * CHUNK_WORDS * sizeof(uint32_t);
      cuda_check(cudaFuncSetAttribute(flip_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)),
                 "flip kernel shared memory");
      flip_rows_kernel<<<dim3(nchunks, (n_flip + FLIP_GROUP - 1) / FLIP_GROUP), 256, smem, st>>>(
         d_flip_pos, n_flip, n_rows, in.is_null, ko, out.keys, io, out.ints, eo, out.exc, flip_bits, flip_counts);
      cuda_check(cudaGetLastError(), "flip kernel");
      flip_hist_kernel<<<(n_flip * nchunks + 255) / 256, 256, 0, st>>>(d_flip_pos, d_flip, in.ref_sym, n_flip, nchunks, L,
                                                                      nsym, flip_counts, hist);
      cuda_check(cudaGetLastError(), "flip counts");
   }

   // 4. buckets: offsets, scatter, sort
   uint32_t* boff = a.get<uint32_t>(nb);
   const uint32_t n_stored = exclusive_scan<uint32_t>(a, hist, boff, nb, st);
   uint32_t* cursor = a.get<uint32_t>(nb);
   cuda_check(cudaMemcpyAsync(cursor, boff, nb * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st), "copy");
   uint16_t* rows = a.get<uint16_t>(n_stored);
   scatter_keys_kernel<<<grid_for(total_keys, 256), 256, 0, st>>>(out.keys, total_keys, L, nsym, d_flip, cursor, rows);
   if (n_flip)
      flip_scatter_kernel<<<dim3(nchunks, n_flip), 256, 0, st>>>(d_flip_pos, in.ref_sym, nchunks, L, nsym, flip_bits, boff,
                                                              rows);
   cuda_check(cudaGetLastError(), "scatter");
   uint32_t* flag = a.get<uint32_t>(nb);
   uint32_t* lofs = a.get<uint32_t>(nb);
   nonzero_kernel<<<grid_for(nb, 256), 256, 0, st>>>(hist, nb, flag);
   const uint32_t n_ctr = exclusive_scan<uint32_t>(a, flag, lofs, nb, st);
   uint32_t* list = a.get<uint32_t>(n_ctr);
   list_buckets_kernel<<<grid_for(nb, 256), 256, 0, st>>>(hist, lofs, nb, list);
   uint32_t* nruns = a.get<uint32_t>(n_ctr);
   uint8_t* type = a.get<uint8_t>(n_ctr);
   if (n_ctr)
      sort_buckets_kernel<<<grid_for(n_ctr, SORT_WARPS), SORT_WARPS * 32, 0, st>>>(list, n_ctr, hist, boff, rows, nruns,
                                                                                 type);
   cuda_check(cudaGetLastError(), "sort");

   // 5. containers: descriptors and payload offsets in the host's layout
   const std::vector<uint32_t> h_list = to_host(list, n_ctr, st);
   const std::vector<uint32_t> h_hist_b = [&] {
      std::vector<uint32_t> c(n_ctr);
      // cardinality of each listed bucket
      std::vector<uint32_t> all = to_host(hist, nb, st);
      for (uint32_t i = 0; i < n_ctr; ++i) c[i] = all[h_list[i]];
      return c;
   }();
   const std::vector<uint32_t> h_nruns = to_host(nruns, n_ctr, st);
   const std::vector<uint8_t> h_type = to_host(type, n_ctr, st);
   ContainerSet& cs = col.vertical;
   cs.nkeys = L;
   cs.ctrs.resize(n_ctr);
   std::vector<uint32_t> poff(n_ctr);
   {
      size_t at = 0;   // global payload size so far
      uint32_t i = 0;
      for (uint32_t v = 0; v < nchunks; ++v) {
         while (at % 8) ++at;
         const size_t chunk_base = at;
         size_t arrays = 0;
         uint32_t j = i;
         const size_t vend = (static_cast<size_t>(v) + 1) * L * nsym;
         while (j < n_ctr && h_list[j] < vend) {
            if (h_type[j] == CT_ARRAY) arrays += h_hist_b[j];
            ++j;
         }
         size_t a_at = chunk_base, o_at = chunk_base + ((arrays + 7) / 8) * 8;
         for (uint32_t k = i; k < j; ++k) {
            const uint32_t b = h_list[k];
            CtrDesc d{};
            d.key = (b / nsym) % L;
            d.v = static_cast<uint16_t>(v);
            d.sym = static_cast<uint8_t>(b % nsym);
            d.type = h_type[k];
            d.card_m1 = static_cast<uint16_t>(h_hist_b[k] - 1);
            if (d.type == CT_ARRAY) {
               d.payload = static_cast<uint32_t>(a_at);
               a_at += h_hist_b[k];
            } else if (d.type == CT_BITSET) {
               while (o_at % 8) ++o_at;
               d.payload = static_cast<uint32_t>(o_at);
               o_at += 4096;
            } else {
               d.nruns = static_cast<uint16_t>(h_nruns[k]);
               d.payload = static_cast<uint32_t>(o_at);
               o_at += 2ull * h_nruns[k];
            }
            cs.ctrs[k] = d;
            poff[k] = d.payload;
         }
         at = o_at;
         i = j;
      }
      while (at % 8) ++at;
      at += 8;  // the spare 16 bytes read past a container's last element
      if (at > 0xFFFFFFFFull) throw std::runtime_error("payload arena exceeds 2^32 entries");
      uint32_t* d_poff = to_device(a, poff, st);
      uint16_t* d_payload = a.get<uint16_t>(at);
      cuda_check(cudaMemsetAsync(d_payload, 0, at * sizeof(uint16_t), st), "memset");
      if (n_ctr)
         write_payload_kernel<<<grid_for(static_cast<size_t>(n_ctr) * 32, 256), 256, 0, st>>>(list, n_ctr, hist, boff, rows,
                                                                                               type, d_poff, d_payload);
      cuda_check(cudaGetLastError(), "payload");
      cs.payload = to_host(d_payload, at, st);
   }
   finish_container_set(cs, nchunks);
   for (uint32_t p : flip_pos) col.local_ref[p] = flip[p];

   // per-chunk row records for the host's finishing passes
   const std::vector<uint32_t> h_io = to_host(io, n_rows + 1, st);
   const std::vector<uint32_t> h_eo = to_host(eo, n_rows + 1, st);
   const std::vector<uint2> h_ints = to_host(out.ints, total_ints, st);
   const std::vector<CovExc> h_exc = to_host(out.exc, total_exc, st);
   std::vector<ChunkRows> chunks(nchunks);
   parallel_for(nchunks, threads, [&](uint32_t v) {
      ChunkRows& c = chunks[v];
      const uint32_t g0 = v * CHUNK_ROWS, g1 = g0 + chunk_sizes[v];
      c.exc.assign(h_exc.begin() + h_eo[g0], h_exc.begin() + h_eo[g1]);
      c.nr_off.resize(chunk_sizes[v] + 1);
      for (uint32_t r = 0; r <= chunk_sizes[v]; ++r) c.nr_off[r] = h_io[g0 + r] - h_io[g0];
      c.nr_s.resize(h_io[g1] - h_io[g0]);
      c.nr_e.resize(h_io[g1] - h_io[g0]);
      for (uint32_t q = h_io[g0]; q < h_io[g1]; ++q) {
         c.nr_s[q - h_io[g0]] = h_ints[q].x;
         c.nr_e[q - h_io[g0]] = h_ints[q].y;
      }
      for (uint32_t g = g0; g < g1; ++g)
         if (raw.is_null[g]) c.nulls.push_back(g);
   });
   finish_seq_column(col, chunks, chunk_sizes, threads);
   return col;
}

}  // namespace

TableImage build_table_gpu(const RawTable& raw, int device, uint32_t threads) {
   cuda_check(cudaSetDevice(device), "cudaSetDevice");
   TableImage t;
   build_table_frame(raw, t);
   cudaStream_t st = nullptr;
   cuda_check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream");
   try {
      for (const auto& c : raw.seq) t.seq.push_back(build_seq_column_gpu(c, t.chunk_sizes, threads, st));
   } catch (...) {
      cudaStreamSynchronize(st);
      cudaStreamDestroy(st);
      throw;
   }
   cudaStreamDestroy(st);
   build_metadata_columns(raw, t, threads);
   return t;
}

}  // namespace rhygpu
