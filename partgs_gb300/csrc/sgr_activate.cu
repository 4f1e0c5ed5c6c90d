// Point-level parameter activations and their backward in one kernel each
// (scene/gaussian_model.py:198-218, the getters the training step calls):
//
//   scales    = exp(log_scaling)                     [P,2]
//   rotations = rotation / max(|rotation|, 1e-12)      (F.normalize)   [P,4]
//   opacities = sigmoid(opacity_logit)               [P,1]
//   shs       = cat(features_dc [P,1,3], features_rest [P,M-1,3])      [P,M,3]
//
// One launch each way.  Its first CTAs take one surfel per thread for the
// small parameters; the rest copy the SH coefficients as one flat array of
// P * M * 3 floats, a float per thread, so that consecutive threads touch
// consecutive addresses (a thread per surfel would put a warp's SH accesses
// 192 bytes apart).  The whole transform is one pass over the parameters
// (HBM-bound: about 440 bytes per surfel forward and backward at SH degree 3).
#include <cuda_runtime.h>

#include <cmath>

#include "../../include/sgr.h"

namespace sgr {
void count_launches(int n);   // sgr_api.cu
}  // namespace sgr

namespace sgract {

constexpr int kThreads = 256;

// CTAs [0, surfel_ctas) take the per-surfel parameters, the rest the SH copy.
__host__ __device__ inline long long surfel_ctas(long long P) { return (P + kThreads - 1) / kThreads; }

__global__ void __launch_bounds__(kThreads) k_activate(sgr_activate_args a) {
  const long long nb = surfel_ctas(a.P);
  if (blockIdx.x >= nb) {   // shs[p, k] = k < 3 ? features_dc[p, k] : features_rest[p, k - 3]
    const int row = a.sh_coeffs * 3;
    const long long e = (long long)(blockIdx.x - nb) * kThreads + threadIdx.x;
    if (e >= a.P * row) return;
    const long long p = e / row;
    const int k = (int)(e - p * row);
    a.shs[e] = k < 3 ? a.features_dc[p * 3 + k] : a.features_rest[p * (row - 3) + (k - 3)];
    return;
  }
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.P) return;
  const float2 ls = reinterpret_cast<const float2*>(a.log_scaling)[i];
  reinterpret_cast<float2*>(a.scales)[i] = make_float2(expf(ls.x), expf(ls.y));
  const float4 q = reinterpret_cast<const float4*>(a.rotation)[i];
  const float n = fmaxf(sqrtf(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w), 1e-12f);
  reinterpret_cast<float4*>(a.rotations)[i] = make_float4(q.x / n, q.y / n, q.z / n, q.w / n);
  a.opacities[i] = 1.0f / (1.0f + expf(-a.opacity_logit[i]));
}

// Adjoints: d log_scaling = d scales * scales; d rotation = (d - r (r.d)) / n
// (the normalisation's Jacobian; below the 1e-12 clamp, d / 1e-12, as
// F.normalize's autograd gives); d logit = d opacities * s (1 - s); the SH
// gradient split back into its two parameter tensors.
__global__ void __launch_bounds__(kThreads) k_activate_bwd(sgr_activate_args a, const float* __restrict__ d_scales,
                                                           const float* __restrict__ d_rotations,
                                                           const float* __restrict__ d_opacities,
                                                           const float* __restrict__ d_shs) {
  const long long nb = surfel_ctas(a.P);
  if (blockIdx.x >= nb) {   // the SH gradient split back into its two tensors
    const int row = a.sh_coeffs * 3;
    const long long e = (long long)(blockIdx.x - nb) * kThreads + threadIdx.x;
    if (e >= a.P * row) return;
    const long long p = e / row;
    const int k = (int)(e - p * row);
    const float d = d_shs ? d_shs[e] : 0.0f;
    if (k < 3) a.d_features_dc[p * 3 + k] = d;
    else a.d_features_rest[p * (row - 3) + (k - 3)] = d;
    return;
  }
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.P) return;
  const float2 ls = reinterpret_cast<const float2*>(a.log_scaling)[i];
  const float2 ds = d_scales ? reinterpret_cast<const float2*>(d_scales)[i] : make_float2(0.f, 0.f);
  reinterpret_cast<float2*>(a.d_log_scaling)[i] = make_float2(ds.x * expf(ls.x), ds.y * expf(ls.y));
  const float4 q = reinterpret_cast<const float4*>(a.rotation)[i];
  const float len = sqrtf(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
  float4 dq = make_float4(0.f, 0.f, 0.f, 0.f);
  if (d_rotations) {
    const float4 d = reinterpret_cast<const float4*>(d_rotations)[i];
    if (len > 1e-12f) {
      const float4 r = make_float4(q.x / len, q.y / len, q.z / len, q.w / len);
      const float rd = r.x * d.x + r.y * d.y + r.z * d.z + r.w * d.w;
      dq = make_float4((d.x - r.x * rd) / len, (d.y - r.y * rd) / len, (d.z - r.z * rd) / len,
                       (d.w - r.w * rd) / len);
    } else {
      dq = make_float4(d.x / 1e-12f, d.y / 1e-12f, d.z / 1e-12f, d.w / 1e-12f);
    }
  }
  reinterpret_cast<float4*>(a.d_rotation)[i] = dq;
  const float s = 1.0f / (1.0f + expf(-a.opacity_logit[i]));
  a.d_opacity_logit[i] = d_opacities ? d_opacities[i] * s * (1.0f - s) : 0.0f;
}

int check(const sgr_activate_args* a) {
  if (!a || a->P < 0 || a->sh_coeffs < 1 || a->sh_coeffs > 16) return SGR_ERR_INVALID_ARGUMENT;
  return SGR_OK;
}

}  // namespace sgract

using namespace sgract;

extern "C" {

int sgr_activate_forward(const sgr_activate_args* a, void* stream) {
  int rc = check(a);
  if (rc) return rc;
  if (a->P == 0) return SGR_OK;
  if (!a->log_scaling || !a->rotation || !a->opacity_logit || !a->features_dc || !a->scales || !a->rotations ||
      !a->opacities || !a->shs || (a->sh_coeffs > 1 && !a->features_rest))
    return SGR_ERR_INVALID_ARGUMENT;
  const long long ctas = surfel_ctas(a->P) + (a->P * a->sh_coeffs * 3 + kThreads - 1) / kThreads;
  k_activate<<<(unsigned)ctas, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(*a);
  sgr::count_launches(1);
  return cudaGetLastError() == cudaSuccess ? SGR_OK : SGR_ERR_CUDA;
}

int sgr_activate_backward(const sgr_activate_args* a, const float* d_scales, const float* d_rotations,
                          const float* d_opacities, const float* d_shs, void* stream) {
  int rc = check(a);
  if (rc) return rc;
  if (a->P == 0) return SGR_OK;
  if (!a->log_scaling || !a->rotation || !a->opacity_logit || !a->d_log_scaling || !a->d_rotation ||
      !a->d_opacity_logit || !a->d_features_dc || (a->sh_coeffs > 1 && !a->d_features_rest))
    return SGR_ERR_INVALID_ARGUMENT;
  const long long ctas = surfel_ctas(a->P) + (a->P * a->sh_coeffs * 3 + kThreads - 1) / kThreads;
  k_activate_bwd<<<(unsigned)ctas, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(*a, d_scales, d_rotations,
                                                                                     d_opacities, d_shs);
  sgr::count_launches(1);
  return cudaGetLastError() == cudaSuccess ? SGR_OK : SGR_ERR_CUDA;
}

}  // extern "C"
