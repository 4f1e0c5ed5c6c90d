// Densification statistics of one training step (train.py:293-297,
// scene/gaussian_model.py:515-517): for every surfel and every view of the
// batch where the surfel is visible (radius > 0),
//   max_radii2D = max(max_radii2D, radius)
//   grad_accum += |dL/dmeans2D[:2]|,  denom += 1
// in view order, which is what as many single-view iterations accumulate.
// One thread per surfel walks its scene's views; no atomics, so the result
// is deterministic.  Records of view v of a scene sit at
// view.record_offset + (surfel - scene.surfel_offset).
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/sgr.h"

namespace sgr {
void count_launches(int n);   // sgr_api.cu
}  // namespace sgr

namespace sgrdens {

__global__ void k_densify_stats(const sgr_scene_desc* __restrict__ scenes, int num_scenes,
                                const sgr_view_desc* __restrict__ views, int num_surfels,
                                const int32_t* __restrict__ radii, const float* __restrict__ dmeans2D,
                                float grad_scale, float* __restrict__ max_radii2D, float* __restrict__ grad_accum,
                                float* __restrict__ denom) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= num_surfels) return;
  int lo = 0, hi = num_scenes - 1;   // last scene whose first surfel is <= i
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (scenes[mid].surfel_offset <= i) lo = mid; else hi = mid - 1;
  }
  const sgr_scene_desc sc = scenes[lo];
  const int local = i - sc.surfel_offset;
  float mr = max_radii2D[i], acc = grad_accum[i], den = denom[i];
  for (int v = sc.view_begin; v < sc.view_begin + sc.view_count; ++v) {
    const long long r = (long long)views[v].record_offset + local;
    const int rad = radii[r];
    if (rad > 0) {
      mr = fmaxf(mr, (float)rad);
      const float gx = dmeans2D[3 * r], gy = dmeans2D[3 * r + 1];
      acc += __fmul_rn(sqrtf(__fadd_rn(__fmul_rn(gx, gx), __fmul_rn(gy, gy))), grad_scale);
      den += 1.0f;
    }
  }
  max_radii2D[i] = mr;
  grad_accum[i] = acc;
  denom[i] = den;
}

}  // namespace sgrdens

extern "C" int sgr_densify_stats(const sgr_scene_desc* scenes, int32_t num_scenes, const sgr_view_desc* views,
                                 int32_t num_surfels, const int32_t* radii, const float* dmeans2D, float grad_scale,
                                 float* max_radii2D, float* grad_accum, float* denom, void* stream) {
  if (num_surfels < 0 || num_scenes < 1 || !scenes || !views) return SGR_ERR_INVALID_ARGUMENT;
  if (num_surfels == 0) return SGR_OK;
  if (!radii || !dmeans2D || !max_radii2D || !grad_accum || !denom) return SGR_ERR_INVALID_ARGUMENT;
  sgrdens::k_densify_stats<<<(num_surfels + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      scenes, num_scenes, views, num_surfels, radii, dmeans2D, grad_scale, max_radii2D, grad_accum, denom);
  sgr::count_launches(1);
  return cudaGetLastError() == cudaSuccess ? SGR_OK : SGR_ERR_CUDA;
}
