// The planner's network on the GPU: 24 -> 64 -> 64 -> 2 with ReLU, BF16 weights, FP32 arithmetic.
//
//   mlp_forward_kernel   one thread per sample; the BF16 weights are widened once per CTA into
//                        shared memory; the second hidden layer is folded into the output as it
//                        is produced, so only the first hidden layer lives in registers.
//   mlp_grad_kernel      forward + backward of the mean squared error for 128 samples per CTA, the
//                        hidden layers' products on the tensor cores (tcgen05.mma, accumulators in
//                        tensor memory), FP32 operands entering as split BF16 parts.
//   mlp_adam_kernel      Adam on the FP32 master weights; writes the BF16 copy the other kernels use.
// The gradient is taken with respect to the BF16 weights the forward pass used and applied to the
// master weights.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>

#include "mlp.h"

namespace rhygpu {

namespace {

constexpr uint32_t FWD_T = 128;

__device__ __forceinline__ void load_weights(const __nv_bfloat16* __restrict__ w, float* sw) {
   for (uint32_t i = threadIdx.x; i < MLP_NPARAM; i += blockDim.x) sw[i] = __bfloat162float(w[i]);
   __syncthreads();
}

__global__ void __launch_bounds__(FWD_T) mlp_forward_kernel(const __nv_bfloat16* __restrict__ w,
                                                            const float* __restrict__ X, uint32_t n,
                                                            float* __restrict__ Y) {
   extern __shared__ float sw[];
   load_weights(w, sw);
   const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
   if (s >= n) return;
   const float* W1 = sw + MLP_W1;
   const float* B1 = sw + MLP_B1;
   const float* W2 = sw + MLP_W2;
   const float* B2 = sw + MLP_B2;
   const float* W3 = sw + MLP_W3;
   const float* B3 = sw + MLP_B3;
   float x[MLP_IN];
#pragma unroll
   for (uint32_t i = 0; i < MLP_IN; ++i) x[i] = X[static_cast<size_t>(s) * MLP_IN + i];
   float h1[MLP_H];
#pragma unroll
   for (uint32_t j = 0; j < MLP_H; ++j) {
      float a = B1[j];
#pragma unroll
      for (uint32_t i = 0; i < MLP_IN; ++i) a = fmaf(W1[j * MLP_IN + i], x[i], a);
      h1[j] = fmaxf(a, 0.0f);
   }
   float y0 = B3[0], y1 = B3[1];
   for (uint32_t j = 0; j < MLP_H; ++j) {
      float a = B2[j];
#pragma unroll
      for (uint32_t i = 0; i < MLP_H; ++i) a = fmaf(W2[j * MLP_H + i], h1[i], a);
      a = fmaxf(a, 0.0f);
      y0 = fmaf(W3[j], a, y0);
      y1 = fmaf(W3[MLP_H + j], a, y1);
   }
   Y[2 * static_cast<size_t>(s)] = y0;
   Y[2 * static_cast<size_t>(s) + 1] = y1;
}

// ---- gradient on the tensor cores ----
//
// One CTA of 128 threads per 128 samples (the MMA's M); thread t owns sample t, which is row t of
// every accumulator in tensor memory (TMEM lane t). The products run as tcgen05.mma (kind::f16,
// BF16 operands, FP32 accumulation) issued by one thread, operands in shared memory in the
// no-swizzle K-major layout (8 x 16-byte core matrices), accumulators in TMEM:
//   phase 0  Z1 = X W1^T                     (M 128, N 64, K 32: the 24 features and zeros)
//   phase 1  Z2 = H1 W2^T                    (N 64, K 64)
//   phase 2  G1 = D2 W2                      (N 64, K 64)
//            [D2_hi^T; D2_lo^T] [H1^T; 1]^T  (N 80, K 128 samples): dW2 and, from the ones row, db2
//   phase 3  [D1_hi^T; D1_lo^T] [X^T; 1]^T   (N 32, K 128 samples): dW1 and db1
// The network keeps FP32 arithmetic: an FP32 operand v enters as two BF16 parts, hi = bf16(v) and
// lo = bf16(v - hi), and the products add the parts' MMAs (the weights are BF16 already, so a
// forward product takes two MMAs; a weight gradient takes all four combinations, the lo rows of
// its A operand giving the second half of the accumulator rows, which the threads add when they
// write the gradient out). That leaves a relative error near 2^-16 per product. The output layer,
// dW3 and db3 (two outputs) stay on the CUDA cores with warp reductions.
constexpr uint32_t TC_S = 128;
// byte offset of element (r, k) in a K-major operand of kc 16-byte chunks along K
__device__ __forceinline__ uint32_t cm_off(uint32_t r, uint32_t k, uint32_t kc) {
   return ((((r >> 3) * kc) + (k >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1);
}
// shared memory of the gradient kernel (bytes)
constexpr uint32_t SO_XA_HI = 0;           // X [128 x 32], hi / lo
constexpr uint32_t SO_XA_LO = 8192;
constexpr uint32_t SO_XB_HI = 16384;       // [X^T; 1; 0] [32 x 128], hi / lo
constexpr uint32_t SO_XB_LO = 24576;
constexpr uint32_t SO_W1 = 32768;          // W1 [64 x 32]
constexpr uint32_t SO_W2 = 36864;          // W2 [64 x 64]
constexpr uint32_t SO_W2T = 45056;         // W2^T [64 x 64]
constexpr uint32_t SO_A_HI = 53248;        // H1 [128 x 64] hi / lo; then D2 hi / lo; then [D1_hi^T; D1_lo^T]
constexpr uint32_t SO_A_LO = 69632;
constexpr uint32_t SO_H1B_HI = 86016;      // [H1^T; 1; 0] [80 x 128], hi / lo
constexpr uint32_t SO_H1B_LO = 106496;
constexpr uint32_t SO_D2T = 126976;        // [D2_hi^T; D2_lo^T] [128 x 128]
constexpr uint32_t SO_F32 = 159744;        // W3 (128), b1 (64), b2 (64), b3 (2) as floats
constexpr uint32_t SO_BAR = SO_F32 + 1040;
constexpr uint32_t SO_TMEM = SO_BAR + 8;
constexpr uint32_t SO_END = SO_TMEM + 8;
// TMEM columns of the accumulators
constexpr uint32_t TM_Z1 = 0, TM_Z2 = 64, TM_G1 = 128, TM_DW2 = 192, TM_DW1 = 272, TM_COLS = 512;

// a device error of the gradient kernel (a bounded wait for its MMAs that gave up); read and cleared
// by mlp_take_error
__device__ int g_mlp_err = 0;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

// shared-memory matrix descriptor: no swizzle, start address, leading byte offset (next 16-byte
// chunk along K), stride byte offset (next 8-row group), descriptor version 1 (bits 46-47)
__device__ __forceinline__ uint64_t mma_sdesc(uint32_t addr, uint32_t sbo) {
   return static_cast<uint64_t>((addr >> 4) & 0x3FFFu) | (static_cast<uint64_t>(128u >> 4) << 16) |
          (static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, M = 128
__host__ __device__ constexpr uint32_t mma_idesc(uint32_t n) {
   return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((128u >> 4) << 24);
}
// D[tmem] (+)= A B^T over K = 16 * ksteps: A [128 x K] and B [N x K] K-major with kc chunks along K
__device__ __forceinline__ void mma_k(uint32_t d, uint32_t a, uint32_t b, uint32_t kc, uint32_t ksteps,
                                      uint32_t idesc, bool accumulate) {
   for (uint32_t k = 0; k < ksteps; ++k) {
      const uint64_t ad = mma_sdesc(a + 256 * k, kc * 128), bd = mma_sdesc(b + 256 * k, kc * 128);
      const uint32_t acc = (accumulate || k > 0) ? 1u : 0u;
      asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
                   "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                   : "memory");
   }
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
   asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// operands written by the threads become visible to the tensor cores; then one thread issues
__device__ __forceinline__ void operands_ready() {
   asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
   asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
   __syncthreads();
   asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// waits (bounded: 2 s on the global timer) for the MMAs committed as phase `parity`; the whole CTA
// agrees on the outcome
__device__ __forceinline__ bool mma_wait(uint64_t* bar, uint32_t parity) {
   const uint32_t b = smem_u32(bar);
   uint64_t t0 = 0;
   bool done = false;
   for (uint32_t i = 0; i < (1u << 24) && !done; ++i) {
      uint32_t d;
      asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
                   : "=r"(d)
                   : "r"(b), "r"(parity), "r"(1000u)
                   : "memory");
      done = d != 0;
      if (!done) {
         uint64_t now;
         asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
         if (t0 == 0) t0 = now;
         else if (now - t0 > 2000000000ull) break;
      }
   }
   done = __syncthreads_and(done) != 0;
   asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
   return done;
}
// 16 consecutive FP32 accumulator columns of this thread's row (its warp's 32 TMEM lanes)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
   uint32_t r[16];
   asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
                  "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                : "r"(taddr));
   asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
   for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}
__device__ __forceinline__ void put_bf16(uint8_t* base, uint32_t off, __nv_bfloat16 v) {
   *reinterpret_cast<__nv_bfloat16*>(base + off) = v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
   for (uint32_t o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
   return v;
}

__global__ void __launch_bounds__(TC_S, 1) mlp_grad_kernel(const __nv_bfloat16* __restrict__ w,
                                                           const float* __restrict__ X, const float* __restrict__ T,
                                                           uint32_t n, float inv_total, float* __restrict__ grad,
                                                           float* __restrict__ loss) {
   extern __shared__ __align__(1024) uint8_t sm[];
   const uint32_t t = threadIdx.x, warp = t >> 5, lane = t & 31;
   const uint32_t s = blockIdx.x * TC_S + t;
   const bool live = s < n;
   uint64_t* bar = reinterpret_cast<uint64_t*>(sm + SO_BAR);
   uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + SO_TMEM);
   float* W3f = reinterpret_cast<float*>(sm + SO_F32);
   float* b1f = W3f + 2 * MLP_H;
   float* b2f = b1f + MLP_H;
   float* b3f = b2f + MLP_H;
   if (t == 0) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)));
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
   }
   if (warp == 0) {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                   "r"(TM_COLS)
                   : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
   }
   // weights: W1 [64 x 32] (zeros past the 24 inputs), W2 and W2^T [64 x 64]; the rest as floats
   for (uint32_t i = t; i < MLP_H * 32; i += TC_S) {
      const uint32_t j = i / 32, k = i % 32;
      put_bf16(sm + SO_W1, cm_off(j, k, 4), k < MLP_IN ? w[MLP_W1 + j * MLP_IN + k] : __float2bfloat16_rn(0.0f));
   }
   for (uint32_t i = t; i < MLP_H * MLP_H; i += TC_S) {
      const uint32_t j = i / MLP_H, k = i % MLP_H;
      const __nv_bfloat16 v = w[MLP_W2 + i];
      put_bf16(sm + SO_W2, cm_off(j, k, 8), v);
      put_bf16(sm + SO_W2T, cm_off(k, j, 8), v);
   }
   for (uint32_t i = t; i < 2 * MLP_H; i += TC_S) W3f[i] = __bfloat162float(w[MLP_W3 + i]);
   if (t < MLP_H) {
      b1f[t] = __bfloat162float(w[MLP_B1 + t]);
      b2f[t] = __bfloat162float(w[MLP_B2 + t]);
   }
   if (t < MLP_OUT) b3f[t] = __bfloat162float(w[MLP_B3 + t]);
   // this sample's features: row t of X (hi, lo) and column t of [X^T; 1; 0]
   for (uint32_t k = 0; k < 32; ++k) {
      const float v = (live && k < MLP_IN) ? X[static_cast<size_t>(s) * MLP_IN + k] : 0.0f;
      const __nv_bfloat16 hi = __float2bfloat16_rn(v), lo = __float2bfloat16_rn(v - __bfloat162float(hi));
      put_bf16(sm + SO_XA_HI, cm_off(t, k, 4), hi);
      put_bf16(sm + SO_XA_LO, cm_off(t, k, 4), lo);
      put_bf16(sm + SO_XB_HI, cm_off(k, t, 16), k == MLP_IN ? __float2bfloat16_rn(1.0f) : hi);
      put_bf16(sm + SO_XB_LO, cm_off(k, t, 16), lo);
   }
   operands_ready();
   const uint32_t tmem = *tmem_slot;
   const uint32_t base = smem_u32(sm);
   const uint32_t lane_addr = tmem + ((32u * warp) << 16);
   bool ok = true;
   uint32_t committed = 0;  // MMA phases committed to the barrier (the same in every thread)
   // ---- phase 0: Z1 = X W1^T
   if (t == 0) {
      mma_k(tmem + TM_Z1, base + SO_XA_HI, base + SO_W1, 4, 2, mma_idesc(64), false);
      mma_k(tmem + TM_Z1, base + SO_XA_LO, base + SO_W1, 4, 2, mma_idesc(64), true);
      mma_commit(bar);
   }
   ++committed;
   ok = mma_wait(bar, 0);
   uint32_t mask1[2] = {0, 0}, mask2[2] = {0, 0};
   if (ok) {
      // h1 = relu(z1 + b1): row t of H1 (hi, lo) and column t of [H1^T; 1; 0]
      for (uint32_t c0 = 0; c0 < MLP_H; c0 += 16) {
         float z[16];
         tmem_ld16(lane_addr + TM_Z1 + c0, z);
#pragma unroll
         for (uint32_t j = 0; j < 16; ++j) {
            const float a = z[j] + b1f[c0 + j];
            const float h = fmaxf(a, 0.0f);
            if (a > 0.0f) mask1[(c0 + j) >> 5] |= 1u << ((c0 + j) & 31);
            const __nv_bfloat16 hi = __float2bfloat16_rn(h), lo = __float2bfloat16_rn(h - __bfloat162float(hi));
            put_bf16(sm + SO_A_HI, cm_off(t, c0 + j, 8), hi);
            put_bf16(sm + SO_A_LO, cm_off(t, c0 + j, 8), lo);
            put_bf16(sm + SO_H1B_HI, cm_off(c0 + j, t, 16), hi);
            put_bf16(sm + SO_H1B_LO, cm_off(c0 + j, t, 16), lo);
         }
      }
      for (uint32_t i = MLP_H; i < 80; ++i) {
         put_bf16(sm + SO_H1B_HI, cm_off(i, t, 16), __float2bfloat16_rn(i == MLP_H ? 1.0f : 0.0f));
         put_bf16(sm + SO_H1B_LO, cm_off(i, t, 16), __float2bfloat16_rn(0.0f));
      }
   }
   operands_ready();
   // ---- phase 1: Z2 = H1 W2^T
   if (ok && t == 0) {
      mma_k(tmem + TM_Z2, base + SO_A_HI, base + SO_W2, 8, 4, mma_idesc(64), false);
      mma_k(tmem + TM_Z2, base + SO_A_LO, base + SO_W2, 8, 4, mma_idesc(64), true);
      mma_commit(bar);
   }
   if (ok) {
      ++committed;
      ok = mma_wait(bar, 1);
   }
   if (ok) {
      // output layer and its error
      float y0 = b3f[0], y1 = b3f[1];
      for (uint32_t c0 = 0; c0 < MLP_H; c0 += 16) {
         float z[16];
         tmem_ld16(lane_addr + TM_Z2 + c0, z);
#pragma unroll
         for (uint32_t j = 0; j < 16; ++j) {
            const float a = z[j] + b2f[c0 + j];
            const float h = fmaxf(a, 0.0f);
            if (a > 0.0f) mask2[(c0 + j) >> 5] |= 1u << ((c0 + j) & 31);
            y0 = fmaf(W3f[c0 + j], h, y0);
            y1 = fmaf(W3f[MLP_H + c0 + j], h, y1);
         }
      }
      const float r0 = live ? y0 - T[static_cast<size_t>(s) * MLP_OUT] : 0.0f;
      const float r1 = live ? y1 - T[static_cast<size_t>(s) * MLP_OUT + 1] : 0.0f;
      const float d30 = 2.0f * r0 * inv_total, d31 = 2.0f * r1 * inv_total;
      const float e2 = warp_sum(fmaf(r0, r0, r1 * r1));
      const float g30 = warp_sum(d30), g31 = warp_sum(d31);
      if (lane == 0) {
         atomicAdd(loss, e2 * inv_total);
         atomicAdd(grad + MLP_B3, g30);
         atomicAdd(grad + MLP_B3 + 1, g31);
      }
      // delta2 = (W3^T d3) * relu'(z2): row t of D2 (hi, lo), column t of [D2_hi^T; D2_lo^T];
      // dW3 = sum over the samples of d3 h2^T (warp sums, then one atomic per warp)
      for (uint32_t c0 = 0; c0 < MLP_H; c0 += 16) {
         float z[16];
         tmem_ld16(lane_addr + TM_Z2 + c0, z);
#pragma unroll
         for (uint32_t j = 0; j < 16; ++j) {
            const uint32_t u = c0 + j;
            const float h = fmaxf(z[j] + b2f[u], 0.0f);
            const bool on = (mask2[u >> 5] >> (u & 31)) & 1u;
            const float d2 = on ? fmaf(W3f[u], d30, W3f[MLP_H + u] * d31) : 0.0f;
            const __nv_bfloat16 hi = __float2bfloat16_rn(d2), lo = __float2bfloat16_rn(d2 - __bfloat162float(hi));
            put_bf16(sm + SO_A_HI, cm_off(t, u, 8), hi);
            put_bf16(sm + SO_A_LO, cm_off(t, u, 8), lo);
            put_bf16(sm + SO_D2T, cm_off(u, t, 16), hi);
            put_bf16(sm + SO_D2T, cm_off(MLP_H + u, t, 16), lo);
            const float g0 = warp_sum(d30 * h), g1 = warp_sum(d31 * h);
            if (lane == 0) {
               atomicAdd(grad + MLP_W3 + u, g0);
               atomicAdd(grad + MLP_W3 + MLP_H + u, g1);
            }
         }
      }
   }
   operands_ready();
   // ---- phase 2: G1 = D2 W2; [D2_hi^T; D2_lo^T] [H1^T; 1]^T
   if (ok && t == 0) {
      mma_k(tmem + TM_G1, base + SO_A_HI, base + SO_W2T, 8, 4, mma_idesc(64), false);
      mma_k(tmem + TM_G1, base + SO_A_LO, base + SO_W2T, 8, 4, mma_idesc(64), true);
      mma_k(tmem + TM_DW2, base + SO_D2T, base + SO_H1B_HI, 16, 8, mma_idesc(80), false);
      mma_k(tmem + TM_DW2, base + SO_D2T, base + SO_H1B_LO, 16, 8, mma_idesc(80), true);
      mma_commit(bar);
   }
   if (ok) {
      ++committed;
      ok = mma_wait(bar, 0);
   }
   if (ok) {
      // delta1 = G1 * relu'(z1) into column t of [D1_hi^T; D1_lo^T] (over D2, which phase 2 has read)
      for (uint32_t c0 = 0; c0 < MLP_H; c0 += 16) {
         float g[16];
         tmem_ld16(lane_addr + TM_G1 + c0, g);
#pragma unroll
         for (uint32_t j = 0; j < 16; ++j) {
            const uint32_t u = c0 + j;
            const float d1 = ((mask1[u >> 5] >> (u & 31)) & 1u) ? g[j] : 0.0f;
            const __nv_bfloat16 hi = __float2bfloat16_rn(d1), lo = __float2bfloat16_rn(d1 - __bfloat162float(hi));
            put_bf16(sm + SO_A_HI, cm_off(u, t, 16), hi);
            put_bf16(sm + SO_A_HI, cm_off(MLP_H + u, t, 16), lo);
         }
      }
      // dW2 and db2: accumulator row t holds unit t & 63 (hi part for t < 64, lo part above)
      const uint32_t j = t & (MLP_H - 1);
      for (uint32_t c0 = 0; c0 < 80; c0 += 16) {
         float v[16];
         tmem_ld16(lane_addr + TM_DW2 + c0, v);
#pragma unroll
         for (uint32_t q = 0; q < 16; ++q) {
            const uint32_t i = c0 + q;
            if (i < MLP_H) atomicAdd(grad + MLP_W2 + j * MLP_H + i, v[q]);
            else if (i == MLP_H) atomicAdd(grad + MLP_B2 + j, v[q]);
         }
      }
   }
   operands_ready();
   // ---- phase 3: [D1_hi^T; D1_lo^T] [X^T; 1]^T
   if (ok && t == 0) {
      mma_k(tmem + TM_DW1, base + SO_A_HI, base + SO_XB_HI, 16, 8, mma_idesc(32), false);
      mma_k(tmem + TM_DW1, base + SO_A_HI, base + SO_XB_LO, 16, 8, mma_idesc(32), true);
      mma_commit(bar);
   }
   if (ok) {
      ++committed;
      ok = mma_wait(bar, 1);
   }
   if (ok) {
      const uint32_t j = t & (MLP_H - 1);
      for (uint32_t c0 = 0; c0 < 32; c0 += 16) {
         float v[16];
         tmem_ld16(lane_addr + TM_DW1 + c0, v);
#pragma unroll
         for (uint32_t q = 0; q < 16; ++q) {
            const uint32_t i = c0 + q;
            if (i < MLP_IN) atomicAdd(grad + MLP_W1 + j * MLP_IN + i, v[q]);
            else if (i == MLP_IN) atomicAdd(grad + MLP_B1 + j, v[q]);
         }
      }
   } else if (t == 0) {
      atomicExch(&g_mlp_err, 1);
   }
   // a wait that gave up leaves MMAs possibly in flight: wait for the phase it gave up on (bounded)
   // before the tensor memory is freed
   if (!ok) mma_wait(bar, (committed - 1) & 1u);
   asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
   __syncthreads();
   if (warp == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TM_COLS) : "memory");
   }
}

__global__ void mlp_adam_kernel(float* __restrict__ master, __nv_bfloat16* __restrict__ w, float* __restrict__ grad,
                                float* __restrict__ m, float* __restrict__ v, float lr, float beta1, float beta2,
                                float eps, float c1, float c2) {
   const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
   if (p >= MLP_NPARAM) return;
   const float g = grad[p];
   const float mm = beta1 * m[p] + (1.0f - beta1) * g;
   const float vv = beta2 * v[p] + (1.0f - beta2) * g * g;
   m[p] = mm;
   v[p] = vv;
   const float x = master[p] - lr * (mm / c1) / (sqrtf(vv / c2) + eps);
   master[p] = x;
   w[p] = __float2bfloat16_rn(x);
   grad[p] = 0.0f;
}

__global__ void mlp_cast_kernel(const float* __restrict__ master, __nv_bfloat16* __restrict__ w) {
   const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
   if (p < MLP_NPARAM) w[p] = __float2bfloat16_rn(master[p]);
}

}  // namespace

cudaError_t mlp_cast(const float* d_master, __nv_bfloat16* d_w, cudaStream_t s) {
   mlp_cast_kernel<<<(MLP_NPARAM + 255) / 256, 256, 0, s>>>(d_master, d_w);
   return cudaGetLastError();
}

cudaError_t mlp_forward(const __nv_bfloat16* d_w, const float* d_X, uint32_t n, float* d_Y, cudaStream_t s) {
   if (n == 0) return cudaSuccess;
   const size_t smem = MLP_NPARAM * sizeof(float);
   mlp_forward_kernel<<<(n + FWD_T - 1) / FWD_T, FWD_T, smem, s>>>(d_w, d_X, n, d_Y);
   return cudaGetLastError();
}

cudaError_t mlp_gradient(const __nv_bfloat16* d_w, const float* d_X, const float* d_T, uint32_t n, float* d_grad,
                         float* d_loss, cudaStream_t s) {
   if (n == 0) return cudaSuccess;
   cudaError_t e = cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(SO_END));
   if (e != cudaSuccess) return e;
   mlp_grad_kernel<<<(n + TC_S - 1) / TC_S, TC_S, SO_END, s>>>(d_w, d_X, d_T, n, 1.0f / static_cast<float>(n), d_grad, d_loss);
   return cudaGetLastError();
}

int mlp_take_error() {
   int v = 0;
   const int zero = 0;
   if (cudaMemcpyFromSymbol(&v, g_mlp_err, sizeof(int)) != cudaSuccess) return -1;
   if (v != 0 && cudaMemcpyToSymbol(g_mlp_err, &zero, sizeof(int)) != cudaSuccess) return -1;
   return v;
}

cudaError_t mlp_adam(float* d_master, __nv_bfloat16* d_w, float* d_grad, float* d_m, float* d_v, float lr, uint32_t step,
                     cudaStream_t s) {
   const float beta1 = 0.9f, beta2 = 0.999f;
   const float c1 = 1.0f - static_cast<float>(std::pow(beta1, static_cast<double>(step)));
   const float c2 = 1.0f - static_cast<float>(std::pow(beta2, static_cast<double>(step)));
   mlp_adam_kernel<<<(MLP_NPARAM + 255) / 256, 256, 0, s>>>(d_master, d_w, d_grad, d_m, d_v, lr, beta1, beta2, 1e-8f, c1,
                                                            c2);
   return cudaGetLastError();
}

}  // namespace rhygpu
