// The planner's network: 24 -> 64 -> 64 -> 2 multilayer perceptron with ReLU, BF16 weights and FP32
// arithmetic, trained and evaluated by the kernels in mlp.cu.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace rhygpu {

constexpr uint32_t MLP_IN = 24, MLP_H = 64, MLP_OUT = 2;
// Flat parameter layout (row-major weights [out][in]).
constexpr uint32_t MLP_W1 = 0;
constexpr uint32_t MLP_B1 = MLP_W1 + MLP_H * MLP_IN;
constexpr uint32_t MLP_W2 = MLP_B1 + MLP_H;
constexpr uint32_t MLP_B2 = MLP_W2 + MLP_H * MLP_H;
constexpr uint32_t MLP_W3 = MLP_B2 + MLP_H;
constexpr uint32_t MLP_B3 = MLP_W3 + MLP_OUT * MLP_H;
constexpr uint32_t MLP_NPARAM = MLP_B3 + MLP_OUT;

// BF16 copy of the FP32 master weights (round to nearest even).
cudaError_t mlp_cast(const float* d_master, __nv_bfloat16* d_w, cudaStream_t s);
// Y[n][2] = net(X[n][24]).
cudaError_t mlp_forward(const __nv_bfloat16* d_w, const float* d_X, uint32_t n, float* d_Y, cudaStream_t s);
// Adds the gradient of mean_n sum_k (net(X)_k - T_k)^2 with respect to the BF16 weights to d_grad
// and the loss to *d_loss.
cudaError_t mlp_gradient(const __nv_bfloat16* d_w, const float* d_X, const float* d_T, uint32_t n, float* d_grad,
                         float* d_loss, cudaStream_t s);
// A device error of the gradient kernel since the last call (1: a bounded wait for its tensor-core
// products gave up; -1: the flag could not be read), cleared on reading; 0 if none.
int mlp_take_error();
// One Adam step (beta 0.9 / 0.999, eps 1e-8, bias-corrected at `step` >= 1) on the master weights;
// refreshes the BF16 copy and clears the gradient.
cudaError_t mlp_adam(float* d_master, __nv_bfloat16* d_w, float* d_grad, float* d_m, float* d_v, float lr, uint32_t step,
                     cudaStream_t s);

}  // namespace rhygpu
