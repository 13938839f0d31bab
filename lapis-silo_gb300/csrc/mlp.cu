// The planner's network on the GPU: 24 -> 64 -> 64 -> 2 with ReLU, BF16 weights, FP32 arithmetic.
//
//   mlp_forward_kernel   one thread per sample; the BF16 weights are widened once per CTA into
//                        shared memory; the second hidden layer is folded into the output as it
//                        is produced, so only the first hidden layer lives in registers.
//   mlp_grad_kernel      forward + backward of the mean squared error for 64 samples per CTA: the
//                        activations and deltas of the CTA's samples are kept in shared memory,
//                        then every thread reduces the gradient of its share of the parameters over
//                        the 64 samples and adds it to the global gradient.
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
constexpr uint32_t GRAD_S = 64;  // samples (= threads) per gradient CTA

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

// Shared memory of the gradient kernel (floats): weights, then per sample x, h1, h2, d1, d2, d3.
constexpr uint32_t G_X = MLP_NPARAM;
constexpr uint32_t G_H1 = G_X + GRAD_S * MLP_IN;
constexpr uint32_t G_H2 = G_H1 + GRAD_S * MLP_H;
constexpr uint32_t G_D1 = G_H2 + GRAD_S * MLP_H;
constexpr uint32_t G_D2 = G_D1 + GRAD_S * MLP_H;
constexpr uint32_t G_D3 = G_D2 + GRAD_S * MLP_H;
constexpr uint32_t G_END = G_D3 + GRAD_S * MLP_OUT;

__global__ void __launch_bounds__(GRAD_S) mlp_grad_kernel(const __nv_bfloat16* __restrict__ w,
                                                          const float* __restrict__ X, const float* __restrict__ T,
                                                          uint32_t n, float inv_total, float* __restrict__ grad,
                                                          float* __restrict__ loss) {
   extern __shared__ float sm[];
   load_weights(w, sm);
   const float* W1 = sm + MLP_W1;
   const float* B1 = sm + MLP_B1;
   const float* W2 = sm + MLP_W2;
   const float* B2 = sm + MLP_B2;
   const float* W3 = sm + MLP_W3;
   const float* B3 = sm + MLP_B3;
   float* sx = sm + G_X;
   float* sh1 = sm + G_H1;
   float* sh2 = sm + G_H2;
   float* sd1 = sm + G_D1;
   float* sd2 = sm + G_D2;
   float* sd3 = sm + G_D3;
   const uint32_t t = threadIdx.x;
   const uint32_t s = blockIdx.x * GRAD_S + t;
   const bool live = s < n;
   // ---- forward (one sample per thread); rows of absent samples stay zero
   float* x = sx + t * MLP_IN;
   float* h1 = sh1 + t * MLP_H;
   float* h2 = sh2 + t * MLP_H;
   for (uint32_t i = 0; i < MLP_IN; ++i) x[i] = live ? X[static_cast<size_t>(s) * MLP_IN + i] : 0.0f;
   for (uint32_t j = 0; j < MLP_H; ++j) {
      float a = B1[j];
      for (uint32_t i = 0; i < MLP_IN; ++i) a = fmaf(W1[j * MLP_IN + i], x[i], a);
      h1[j] = live ? fmaxf(a, 0.0f) : 0.0f;
   }
   for (uint32_t j = 0; j < MLP_H; ++j) {
      float a = B2[j];
      for (uint32_t i = 0; i < MLP_H; ++i) a = fmaf(W2[j * MLP_H + i], h1[i], a);
      h2[j] = live ? fmaxf(a, 0.0f) : 0.0f;
   }
   float e2 = 0.0f;
   for (uint32_t k = 0; k < MLP_OUT; ++k) {
      float y = B3[k];
      for (uint32_t j = 0; j < MLP_H; ++j) y = fmaf(W3[k * MLP_H + j], h2[j], y);
      const float r = live ? y - T[static_cast<size_t>(s) * MLP_OUT + k] : 0.0f;
      e2 = fmaf(r, r, e2);
      sd3[t * MLP_OUT + k] = 2.0f * r * inv_total;  // d(mean squared error)/dy
   }
   // ---- backward through the hidden layers
   float* d2 = sd2 + t * MLP_H;
   float* d1 = sd1 + t * MLP_H;
   for (uint32_t j = 0; j < MLP_H; ++j) {
      float a = 0.0f;
      for (uint32_t k = 0; k < MLP_OUT; ++k) a = fmaf(W3[k * MLP_H + j], sd3[t * MLP_OUT + k], a);
      d2[j] = h2[j] > 0.0f ? a : 0.0f;
   }
   for (uint32_t i = 0; i < MLP_H; ++i) {
      float a = 0.0f;
      for (uint32_t j = 0; j < MLP_H; ++j) a = fmaf(W2[j * MLP_H + i], d2[j], a);
      d1[i] = h1[i] > 0.0f ? a : 0.0f;
   }
   // loss of the CTA's samples (per warp)
#pragma unroll
   for (uint32_t o = 16; o > 0; o >>= 1) e2 += __shfl_xor_sync(0xFFFFFFFFu, e2, o);
   __syncthreads();
   // ---- parameter gradients: thread t reduces parameters t, t + 64, ... over the 64 samples
   for (uint32_t p = t; p < MLP_NPARAM; p += GRAD_S) {
      float g = 0.0f;
      if (p < MLP_B1) {
         const uint32_t j = p / MLP_IN, i = p % MLP_IN;
         for (uint32_t q = 0; q < GRAD_S; ++q) g = fmaf(sd1[q * MLP_H + j], sx[q * MLP_IN + i], g);
      } else if (p < MLP_W2) {
         const uint32_t j = p - MLP_B1;
         for (uint32_t q = 0; q < GRAD_S; ++q) g += sd1[q * MLP_H + j];
      } else if (p < MLP_B2) {
         const uint32_t j = (p - MLP_W2) / MLP_H, i = (p - MLP_W2) % MLP_H;
         for (uint32_t q = 0; q < GRAD_S; ++q) g = fmaf(sd2[q * MLP_H + j], sh1[q * MLP_H + i], g);
      } else if (p < MLP_W3) {
         const uint32_t j = p - MLP_B2;
         for (uint32_t q = 0; q < GRAD_S; ++q) g += sd2[q * MLP_H + j];
      } else if (p < MLP_B3) {
         const uint32_t k = (p - MLP_W3) / MLP_H, j = (p - MLP_W3) % MLP_H;
         for (uint32_t q = 0; q < GRAD_S; ++q) g = fmaf(sd3[q * MLP_OUT + k], sh2[q * MLP_H + j], g);
      } else {
         const uint32_t k = p - MLP_B3;
         for (uint32_t q = 0; q < GRAD_S; ++q) g += sd3[q * MLP_OUT + k];
      }
      atomicAdd(grad + p, g);
   }
   if ((t & 31) == 0) atomicAdd(loss, e2 * inv_total);
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
   const size_t smem = G_END * sizeof(float);
   cudaError_t e = cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
   if (e != cudaSuccess) return e;
   mlp_grad_kernel<<<(n + GRAD_S - 1) / GRAD_S, GRAD_S, smem, s>>>(d_w, d_X, d_T, n, 1.0f / static_cast<float>(n), d_grad,
                                                                   d_loss);
   return cudaGetLastError();
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
