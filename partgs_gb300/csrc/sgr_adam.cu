// Adam update of the surfel parameters (torch.optim.Adam as the reference
// configures it, scene/gaussian_model.py:266: betas (0.9, 0.999), eps 1e-15,
// one learning rate per parameter group) for up to SGR_ADAM_MAX_TENSORS
// tensors in one launch.
//
// Per element, with t the step count after this step:
//   m <- b1 m + (1 - b1) g,  v <- b2 v + (1 - b2) g^2,
//   p <- p - (lr / (1 - b1^t)) m / (sqrt(v) / sqrt(1 - b2^t) + eps),
// the update of torch's Adam (torch/optim/adam.py, _single_tensor_adam).
// The step count lives on the device (incremented by k_adam_tick before the
// update), so the call never reads back to the host.  With zero_grad set the
// gradient is cleared after use, replacing a separate zero fill before the
// next backward accumulates into it.
//
// Work layout: blockIdx.y picks the tensor; a grid-stride loop over its
// float4s, then a scalar tail.  The update is HBM-bound: 28 bytes per
// element (read p, g, m, v; write p, m, v) plus 4 when the gradient is
// cleared.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "../../include/sgr.h"

namespace sgr {
void count_launches(int n);   // sgr_api.cu
}  // namespace sgr

namespace sgradam {

__global__ void k_adam_tick(float* step) {
  if (threadIdx.x == 0 && blockIdx.x == 0) step[0] += 1.0f;
}

struct Coeffs {
  float b1, b2, c1, c2, eps;
};

// torch's order of operations: exp_avg.lerp_(g, 1 - b1) (weight below 0.5:
// m + w (g - m)), exp_avg_sq.mul_(b2).addcmul_(g, g, 1 - b2), then
// p.addcdiv_(m, sqrt(v) / sqrt(bc2) + eps, -lr / bc1).
__device__ __forceinline__ void adam_one(float& p, float g, float& m, float& v, float lr_t, float bc2_sqrt,
                                         const Coeffs& k) {
  m = m + k.c1 * (g - m);
  v = k.b2 * v + k.c2 * (g * g);
  const float denom = sqrtf(v) / bc2_sqrt + k.eps;
  p = p + (-lr_t) * (m / denom);
}

__global__ void __launch_bounds__(256) k_adam(sgr_adam_args a, const float* __restrict__ step) {
  const sgr_adam_tensor T = a.tensors[blockIdx.y];
  const float t = step[0];
  const float bc1 = 1.0f - powf(a.beta1, t);
  const float bc2 = 1.0f - powf(a.beta2, t);
  const float lr_t = T.lr / bc1;
  const float bc2_sqrt = sqrtf(bc2);
  const Coeffs k{a.beta1, a.beta2, 1.0f - a.beta1, 1.0f - a.beta2, a.eps};
  const long long n = T.numel;
  const bool vec = ((reinterpret_cast<uintptr_t>(T.param) | reinterpret_cast<uintptr_t>(T.grad) |
                     reinterpret_cast<uintptr_t>(T.exp_avg) | reinterpret_cast<uintptr_t>(T.exp_avg_sq)) & 15) == 0;
  const long long n4 = vec ? n / 4 : 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  float4* p4 = reinterpret_cast<float4*>(T.param);
  float4* g4 = reinterpret_cast<float4*>(T.grad);
  float4* m4 = reinterpret_cast<float4*>(T.exp_avg);
  float4* v4 = reinterpret_cast<float4*>(T.exp_avg_sq);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride) {
    float4 p = p4[i], m = m4[i], v = v4[i];
    const float4 g = g4[i];
    adam_one(p.x, g.x, m.x, v.x, lr_t, bc2_sqrt, k);
    adam_one(p.y, g.y, m.y, v.y, lr_t, bc2_sqrt, k);
    adam_one(p.z, g.z, m.z, v.z, lr_t, bc2_sqrt, k);
    adam_one(p.w, g.w, m.w, v.w, lr_t, bc2_sqrt, k);
    p4[i] = p;
    m4[i] = m;
    v4[i] = v;
    if (a.zero_grad) g4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  for (long long i = 4 * n4 + (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    float p = T.param[i], m = T.exp_avg[i], v = T.exp_avg_sq[i];
    adam_one(p, T.grad[i], m, v, lr_t, bc2_sqrt, k);
    T.param[i] = p;
    T.exp_avg[i] = m;
    T.exp_avg_sq[i] = v;
    if (a.zero_grad) T.grad[i] = 0.f;
  }
}

}  // namespace sgradam

using namespace sgradam;

extern "C" {

int sgr_adam_step(const sgr_adam_args* a, float* step, void* stream) {
  if (!a || !step || a->count < 0 || a->count > SGR_ADAM_MAX_TENSORS) return SGR_ERR_INVALID_ARGUMENT;
  if (!(a->beta1 >= 0.f && a->beta1 < 1.f && a->beta2 >= 0.f && a->beta2 < 1.f && a->eps >= 0.f))
    return SGR_ERR_INVALID_ARGUMENT;
  long long most = 0;
  for (int i = 0; i < a->count; ++i) {
    const sgr_adam_tensor& t = a->tensors[i];
    if (t.numel < 0) return SGR_ERR_INVALID_ARGUMENT;
    if (t.numel > 0 && (!t.param || !t.grad || !t.exp_avg || !t.exp_avg_sq)) return SGR_ERR_INVALID_ARGUMENT;
    most = std::max(most, (long long)t.numel);
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_adam_tick<<<1, 32, 0, st>>>(step);
  sgr::count_launches(1);
  if (a->count > 0 && most > 0) {
    const long long want = (most / 4 + 255) / 256;
    const unsigned gx = (unsigned)std::max(1LL, std::min(want, 152LL * 8));
    k_adam<<<dim3(gx, (unsigned)a->count), 256, 0, st>>>(*a, step);
    sgr::count_launches(1);
  }
  return cudaGetLastError() == cudaSuccess ? SGR_OK : SGR_ERR_CUDA;
}

}  // extern "C"
