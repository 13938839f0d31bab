// sm_103a kernels of the filter / count / mutations hot path.
//
//  filter_kernel        one CTA per (chunk, tile of W rows): runs the postorder filter program over a
//                       stack of W-bit tiles in shared memory; leaves expand array / bitset / run
//                       containers straight into shared memory; writes the row-set tile and/or adds
//                       its popcount (Count action, reference: copy_on_write_bitmap.cpp:108-118).
//  filter_batch_kernel  persistent variant: CTAs pull (query, tile) work items from a counter.
//  mut_ctr_kernel       Mutations: every vertical container once, popcount against the filter tile of
//                       its chunk staged in shared memory, integer counts per (symbol, position)
//                       (reference: mutations_node.cpp:139-189).
//  mut_cov_kernel       Mutations: rows of the filter outside coverage and inside missing intervals,
//                       by position block (reference: mutations_node.cpp:51-136).
//  mut_final_kernel     Mutations: local-reference counts (reference: mutations_node.cpp:192-203).
// All arithmetic is integer; results are bit-exact with the CPU operators.
#include <cuda_runtime.h>

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
};

__device__ __forceinline__ void tile_zero(uint32_t* t, uint32_t WW) {
   for (uint32_t w = threadIdx.x; w < WW; w += blockDim.x) t[w] = 0u;
}

// Scan of one (key) slot of a container set: OR of the containers whose symbol is in `mask`.
__device__ void push_containers(uint32_t* t, const TileCtx& c, const CtrDesc* __restrict__ ctrs,
                                const uint16_t* __restrict__ payload, const uint32_t* __restrict__ off, size_t slot,
                                uint32_t mask, bool use_mask) {
   const uint32_t b = __ldg(off + slot), e = __ldg(off + slot + 1);
   for (uint32_t i = b; i < e; ++i) {
      CtrDesc d;
      const uint4 raw = __ldg(reinterpret_cast<const uint4*>(ctrs) + i);
      d = *reinterpret_cast<const CtrDesc*>(&raw);
      if (use_mask && !((mask >> d.sym) & 1u)) continue;
      or_container(t, d, payload, c.row0, c.W);
   }
}

__device__ void push_covered(uint32_t* t, const TileCtx& c, const DevSeqCol* __restrict__ col, uint32_t pos, bool negate) {
   const uint32_t WW = c.W >> 5;
   for (uint32_t w = threadIdx.x; w < WW; w += blockDim.x) t[w] = valid_word(w, c.nvalid);
   __syncthreads();
   // rows whose covered region does not contain pos
   const uint32_t xb = __ldg(col->exc_off + c.v), xe = __ldg(col->exc_off + c.v + 1);
   for (uint32_t i = xb + threadIdx.x; i < xe; i += blockDim.x) {
      const uint4 raw = __ldg(reinterpret_cast<const uint4*>(col->exc) + i);
      const uint32_t r = raw.x - c.row0;
      if (r < c.W && !(raw.y <= pos && pos < raw.z)) atomicAnd(&t[r >> 5], ~(1u << (r & 31)));
   }
   // rows with a missing interval over pos
   const uint32_t blk = pos / NBLOCK, q = pos % NBLOCK;
   const uint32_t* boff = col->nblk_off + static_cast<size_t>(blk) * c.tab->nchunks + c.v;
   const uint32_t nb = __ldg(boff), ne = __ldg(boff + 1);
   for (uint32_t i = nb + threadIdx.x; i < ne; i += blockDim.x) {
      const uint2 raw = __ldg(reinterpret_cast<const uint2*>(col->nblk) + i);
      const uint32_t r = (raw.x & 0xFFFFu) - c.row0;
      const uint32_t lo = raw.y & 0xFFFFu, hi = raw.y >> 16;
      if (r < c.W && lo <= q && q < hi) atomicAnd(&t[r >> 5], ~(1u << (r & 31)));
   }
   if (negate) {
      __syncthreads();
      for (uint32_t w = threadIdx.x; w < WW; w += blockDim.x) t[w] = valid_word(w, c.nvalid) & ~t[w];
   }
}

// Rows whose date lies in [lo, hi] (outside it when `invert`); null dates match when `with_nulls`.
// Every comparison of the date predicates and the two-sided DateBetween reduce to this form.
__device__ void push_date(uint32_t* t, const TileCtx& c, const DevDateCol* __restrict__ col, int32_t lo, int32_t hi,
                          bool invert, bool with_nulls) {
   const uint32_t WW = c.W >> 5;
   const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
   const int32_t* days = col->days + static_cast<size_t>(c.v) * CHUNK_ROWS + c.row0;
   constexpr uint32_t U = 4;  // words per warp in flight
   for (uint32_t w0 = warp * U; w0 < WW; w0 += nw * U) {
      int32_t d[U];
#pragma unroll
      for (uint32_t k = 0; k < U; ++k) {
         const uint32_t r = 32 * (w0 + k) + lane;
         d[k] = (w0 + k < WW && r < c.nvalid) ? __ldg(days + r) : INT32_MIN;
      }
#pragma unroll
      for (uint32_t k = 0; k < U; ++k) {
         const uint32_t r = 32 * (w0 + k) + lane;
         const bool inside = d[k] >= lo && d[k] <= hi;
         const bool m = r < c.nvalid && (d[k] == INT32_MIN ? with_nulls : (inside != invert));
         const uint32_t bits = __ballot_sync(0xFFFFFFFFu, m);
         if (lane == 0 && w0 + k < WW) t[w0 + k] = bits;
      }
   }
}

// Runs a filter program for one tile. The result is left in stack slot 0. Returns false on a
// malformed program (the error flag is set).
__device__ bool run_program(const TileCtx& c, const Instr* __restrict__ code, uint32_t ncode, uint32_t* stk,
                            uint32_t cap, int* err) {
   const uint32_t WW = c.W >> 5;
   uint32_t sp = 0;
   uint32_t pc = 0;
   uint32_t steps = 0;
   while (pc < ncode) {
      if (++steps > 4u * MAX_PROGRAM) {  // jumps only go forward; this bounds a corrupted program
         if (threadIdx.x == 0) atomicExch(err, 3);
         return false;
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
         case OP_PUSH_DATE: {
            if (sp >= cap) {
               if (threadIdx.x == 0) atomicExch(err, 1);
               return false;
            }
            uint32_t* t = stk + sp * WW;
            ++sp;
            if (in.op == OP_PUSH_FULL) {
               for (uint32_t w = threadIdx.x; w < WW; w += blockDim.x) t[w] = valid_word(w, c.nvalid);
            } else if (in.op == OP_PUSH_COVERED) {
               push_covered(t, c, &c.tab->seq[in.col], in.a, in.flags & 1);
            } else if (in.op == OP_PUSH_DATE) {
               push_date(t, c, &c.tab->date[in.col], static_cast<int32_t>(in.a), static_cast<int32_t>(in.b), in.flags & 2,
                         in.flags & 1);
            } else if (in.op == OP_PUSH_NULLS) {
               const uint32_t* src = c.tab->seq[in.col].null_tiles + static_cast<size_t>(c.v) * CHUNK_WORDS + (c.row0 >> 5);
               for (uint32_t w = threadIdx.x; w < WW; w += blockDim.x) t[w] = __ldg(src + w);
            } else {
               tile_zero(t, WW);
               if (in.op == OP_PUSH_SCAN) {
                  __syncthreads();
                  const DevSeqCol* col = &c.tab->seq[in.col];
                  push_containers(t, c, col->ctrs, col->payload, col->off, static_cast<size_t>(c.v) * col->L + in.a, in.b,
                                  true);
               } else if (in.op == OP_PUSH_DICT) {
                  __syncthreads();
                  const DevDictCol* col = &c.tab->dict[in.col];
                  push_containers(t, c, col->ctrs, col->payload, col->off, static_cast<size_t>(c.v) * col->nkeys + in.a, 0,
                                  false);
               }
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
            uint32_t* x = stk + (sp - 2) * WW;
            const uint32_t* y = stk + (sp - 1) * WW;
            if (in.op == OP_AND) {
               for (uint32_t w = threadIdx.x; w < WW; w += blockDim.x) x[w] &= y[w];
            } else if (in.op == OP_ANDNOT) {
               for (uint32_t w = threadIdx.x; w < WW; w += blockDim.x) x[w] &= ~y[w];
            } else {
               for (uint32_t w = threadIdx.x; w < WW; w += blockDim.x) x[w] |= y[w];
            }
            --sp;
            break;
         }
         case OP_NOT: {
            if (sp < 1) {
               if (threadIdx.x == 0) atomicExch(err, 2);
               return false;
            }
            uint32_t* x = stk + (sp - 1) * WW;
            for (uint32_t w = threadIdx.x; w < WW; w += blockDim.x) x[w] = valid_word(w, c.nvalid) & ~x[w];
            break;
         }
         case OP_THR_BEGIN: {
            if (sp + in.a > cap) {
               if (threadIdx.x == 0) atomicExch(err, 1);
               return false;
            }
            for (uint32_t i = 0; i < in.a; ++i) tile_zero(stk + (sp + i) * WW, WW);
            sp += in.a;
            break;
         }
         case OP_THR_ADD: {
            const uint32_t P = in.a;
            if (sp < P + 1) {
               if (threadIdx.x == 0) atomicExch(err, 2);
               return false;
            }
            const uint32_t* x = stk + (sp - 1) * WW;
            uint32_t* planes = stk + (sp - 1 - P) * WW;
            const bool neg = in.flags & 1;
            for (uint32_t w = threadIdx.x; w < WW; w += blockDim.x) {
               uint32_t carry = neg ? (valid_word(w, c.nvalid) & ~x[w]) : x[w];
               for (uint32_t i = 0; i < P && carry; ++i) {
                  const uint32_t p = planes[i * WW + w];
                  planes[i * WW + w] = p ^ carry;
                  carry &= p;
               }
               if (carry) {  // saturate at 2^P - 1
                  for (uint32_t i = 0; i < P; ++i) planes[i * WW + w] |= carry;
               }
            }
            --sp;
            break;
         }
         case OP_THR_END: {
            const uint32_t P = in.a, n = in.b;
            if (sp < P) {
               if (threadIdx.x == 0) atomicExch(err, 2);
               return false;
            }
            uint32_t* planes = stk + (sp - P) * WW;
            const bool exact = in.flags & 1;
            for (uint32_t w = threadIdx.x; w < WW; w += blockDim.x) {
               uint32_t gt = 0, eq = 0xFFFFFFFFu;
               for (int i = static_cast<int>(P) - 1; i >= 0; --i) {
                  const uint32_t p = planes[i * WW + w];
                  const uint32_t nb = ((n >> i) & 1u) ? 0xFFFFFFFFu : 0u;
                  gt |= eq & p & ~nb;
                  eq &= ~(p ^ nb);
               }
               if (n >> P) eq = 0;  // n does not fit: the saturated count can only be below it
               planes[w] = (exact ? eq : (gt | eq)) & valid_word(w, c.nvalid);
            }
            sp = sp - P + 1;
            break;
         }
         case OP_JZ:
         case OP_JFULL: {
            if (sp < 1) {
               if (threadIdx.x == 0) atomicExch(err, 2);
               return false;
            }
            const uint32_t* x = stk + (sp - 1) * WW;
            int differs = 0;
            if (in.op == OP_JZ) {
               for (uint32_t w = threadIdx.x; w < WW; w += blockDim.x) differs |= (x[w] != 0u);
            } else {
               for (uint32_t w = threadIdx.x; w < WW; w += blockDim.x) differs |= (x[w] != valid_word(w, c.nvalid));
            }
            differs = __syncthreads_or(differs);
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
      __syncthreads();
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

__global__ void __launch_bounds__(FT) filter_kernel(const DevTable* __restrict__ tab, const Instr* __restrict__ code,
                                                    uint32_t ncode, uint32_t tile_bits, uint32_t cap,
                                                    uint32_t* __restrict__ out_tiles, unsigned long long* count, int* err) {
   extern __shared__ __align__(16) uint32_t smem[];
   __shared__ uint32_t red[FT / 32];
   const uint32_t T = CHUNK_ROWS / tile_bits;
   TileCtx c;
   c.tab = tab;
   c.v = blockIdx.x / T;
   c.W = tile_bits;
   c.row0 = (blockIdx.x % T) * tile_bits;
   const uint32_t csize = __ldg(tab->chunk_sizes + c.v);
   c.nvalid = csize > c.row0 ? min(tile_bits, csize - c.row0) : 0u;
   const uint32_t WW = tile_bits >> 5;
   uint32_t* result = smem;
   if (c.nvalid == 0) {
      tile_zero(result, WW);
      __syncthreads();
   } else if (!run_program(c, code, ncode, smem, cap, err)) {
      return;
   }
   uint32_t pc = 0;
   for (uint32_t w = threadIdx.x; w < WW; w += blockDim.x) {
      const uint32_t x = result[w];
      pc += __popc(x);
      if (out_tiles) out_tiles[static_cast<size_t>(c.v) * CHUNK_WORDS + (c.row0 >> 5) + w] = x;
   }
   if (count) {
      const uint32_t s = block_sum(pc, red);
      if (threadIdx.x == 0 && s) atomicAdd(count, static_cast<unsigned long long>(s));
   }
}

__global__ void __launch_bounds__(FT) filter_batch_kernel(const DevTable* __restrict__ tab, const Instr* __restrict__ code,
                                                          const QueryDesc* __restrict__ queries,
                                                          const WorkItem* __restrict__ items, uint32_t n_items,
                                                          uint32_t tile_bits, uint32_t cap, uint32_t* __restrict__ out_tiles,
                                                          unsigned long long* counts, uint32_t* next_item, int* err) {
   extern __shared__ __align__(16) uint32_t smem[];
   __shared__ uint32_t red[FT / 32];
   __shared__ uint32_t item_idx;
   const uint32_t T = CHUNK_ROWS / tile_bits;
   const uint32_t WW = tile_bits >> 5;
   const size_t per_query = static_cast<size_t>(tab->nchunks) * CHUNK_WORDS;
   for (;;) {
      if (threadIdx.x == 0) item_idx = atomicAdd(next_item, 1u);
      __syncthreads();
      const uint32_t it = item_idx;
      __syncthreads();
      if (it >= n_items) return;
      const WorkItem wi = items[it];
      const QueryDesc q = queries[wi.query];
      TileCtx c;
      c.tab = tab;
      c.v = wi.tile / T;
      c.W = tile_bits;
      c.row0 = (wi.tile % T) * tile_bits;
      const uint32_t csize = __ldg(tab->chunk_sizes + c.v);
      c.nvalid = csize > c.row0 ? min(tile_bits, csize - c.row0) : 0u;
      if (c.nvalid == 0) {
         tile_zero(smem, WW);
         __syncthreads();
      } else if (!run_program(c, code + q.code_off, q.code_len, smem, cap, err)) {
         return;
      }
      uint32_t pc = 0;
      uint32_t* dst = q.out_tiles ? out_tiles + static_cast<size_t>(q.out_tiles - 1) * per_query +
                                       static_cast<size_t>(c.v) * CHUNK_WORDS + (c.row0 >> 5)
                                  : nullptr;
      for (uint32_t w = threadIdx.x; w < WW; w += blockDim.x) {
         const uint32_t x = smem[w];
         pc += __popc(x);
         if (dst) dst[w] = x;
      }
      const uint32_t s = block_sum(pc, red);
      if (threadIdx.x == 0 && s) atomicAdd(counts + wi.query, static_cast<unsigned long long>(s));
      __syncthreads();
   }
}
}  // namespace

// ------------------------------------------------------------------------------------------------
// launchers

cudaError_t launch_filter(const DevTable* d_table, uint32_t nchunks, const Instr* d_code, uint32_t ncode,
                          uint32_t tile_bits, uint32_t stack_tiles, uint32_t* d_out_tiles, unsigned long long* d_count,
                          int* d_err, void* stream) {
   const uint32_t T = CHUNK_ROWS / tile_bits;
   const size_t smem = static_cast<size_t>(stack_tiles) * (tile_bits / 8);
   cudaError_t e = cudaFuncSetAttribute(filter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        static_cast<int>(smem > 48 * 1024 ? smem : 48 * 1024));
   if (e != cudaSuccess) return e;
   filter_kernel<<<nchunks * T, FT, smem, static_cast<cudaStream_t>(stream)>>>(d_table, d_code, ncode, tile_bits,
                                                                                stack_tiles, d_out_tiles, d_count, d_err);
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
                         const WorkItem* d_items, uint32_t n_items, uint32_t tile_bits, uint32_t stack_tiles,
                         uint32_t* d_out_tiles, unsigned long long* d_counts, uint32_t* d_next, uint32_t grid, int* d_err,
                         void* stream) {
   (void)nchunks;
   const size_t smem = static_cast<size_t>(stack_tiles) * (tile_bits / 8);
   cudaError_t e = cudaFuncSetAttribute(filter_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        static_cast<int>(smem > 48 * 1024 ? smem : 48 * 1024));
   if (e != cudaSuccess) return e;
   filter_batch_kernel<<<grid, FT, smem, static_cast<cudaStream_t>(stream)>>>(
      d_table, d_code, d_queries, d_items, n_items, tile_bits, stack_tiles, d_out_tiles, d_counts, d_next, d_err);
   return cudaGetLastError();
}

}  // namespace rhygpu
