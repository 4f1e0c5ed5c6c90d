// Block-stage superquadric losses, forward and backward, fused
// (games/block_mesh_splatting/scene/block_gaussian_model.py:522-582, the
// regularisers of summarize_losses at :584-648; the SDF of
// games/block_mesh_splatting/utils/superquadric.py:25-46 with as_sdf=2; the
// ray samples of scene/cameras.py:79-96).
//
// The reference evaluates the SDF of every ray sample (2048 rays x 128
// samples per view) against every block as a chain of materialised
// [blocks, samples] tensors, then reduces per ray.  Here one warp owns a ray:
// its lanes walk the samples, evaluate every block from shared memory and
// keep only what the losses read -- the minimum SDF with its (block, sample)
// index and the occupancy maximum with its block.  The backward needs the SDF
// gradient at one point per ray (min and max pass their gradient to a single
// element), so it is a thread per ray.  The overlap term is dense (every
// random point against every block) and runs as a thread per point in the
// same launches.
//
// Reductions are deterministic: per-CTA tree sums into partials, summed in
// CTA order by one more launch; no floating-point atomics.
#include <cuda_runtime.h>

#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>

#include "../../include/sgr.h"

namespace sgr {
void count_launches(int n);   // sgr_api.cu
}  // namespace sgr

namespace sgrsq {

constexpr int kThreads = 256;
constexpr int kRaysPerCta = kThreads / 32;   // forward: a warp per ray
constexpr int kG = 18;                       // gradient slots per block: S3 R9 T3 eps1 eps2 occ_logit
constexpr float kClampEps = 1e-6f;           // safe_pow's clamp (utils/pytorch.py SQRT_EPS)

struct Blk {
  float R[9], T[3], S[3], D[3];   // D = S * ratio
  float e1, e2, ie1, ie2, r21, h1;
  float alpha;                    // sigmoid(occ_logit)
  float alpha_n;                  // sigmoid(occ_logit + noise), the overlap term's
  float ratio;
};

__device__ __forceinline__ float sigmoidf(float x) { return 1.0f / (1.0f + expf(-x)); }

__device__ void load_block(const sgr_sq_loss_args& a, int b, Blk& B) {
  for (int k = 0; k < 9; ++k) B.R[k] = a.R[9 * b + k];
  for (int k = 0; k < 3; ++k) {
    B.T[k] = a.T[3 * b + k];
    B.S[k] = a.S[3 * b + k];
    B.D[k] = B.S[k] * a.ratio;
  }
  B.ratio = a.ratio;
  B.e1 = a.eps1[b];
  B.e2 = a.eps2[b];
  B.ie1 = 1.0f / B.e1;
  B.ie2 = 1.0f / B.e2;
  B.r21 = B.e2 / B.e1;
  B.h1 = B.e1 * 0.5f;
  const float occ = a.occ_logit ? a.occ_logit[b] : 0.f;
  B.alpha = sigmoidf(occ);
  B.alpha_n = sigmoidf(occ + (a.overlap_noise ? a.overlap_noise[b] : 0.f));
}

// The intermediate values of one SDF evaluation (implicit_sq, safe, as_sdf=2):
//   u = ((p - T) R^T) / (S ratio), clamped to [-5, 5];  a = u^2
//   X = max(a_x, e)^(1/eps2), Y = max(a_y, e)^(1/eps1), Z = max(a_z, e)^(1/eps2)
//   res = max(X + Z, e)^(eps2/eps1) + Y;  sdf = max(res, e)^(eps1/2) - 1
struct Sdf {
  float d[3], q[3], u[3], a[3], X, Y, Z, W, P, res, out;
};

__device__ __forceinline__ float sdf_eval(const Blk& B, float px, float py, float pz, Sdf& t) {
  t.d[0] = px - B.T[0];
  t.d[1] = py - B.T[1];
  t.d[2] = pz - B.T[2];
  float uc[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    t.q[j] = t.d[0] * B.R[3 * j] + t.d[1] * B.R[3 * j + 1] + t.d[2] * B.R[3 * j + 2];
    t.u[j] = t.q[j] / B.D[j];
    uc[j] = fminf(fmaxf(t.u[j], -5.f), 5.f);
    t.a[j] = uc[j] * uc[j];
  }
  t.X = powf(fmaxf(t.a[0], kClampEps), B.ie2);
  t.Y = powf(fmaxf(t.a[1], kClampEps), B.ie1);
  t.Z = powf(fmaxf(t.a[2], kClampEps), B.ie2);
  t.W = t.X + t.Z;
  t.P = powf(fmaxf(t.W, kClampEps), B.r21);
  t.res = t.P + t.Y;
  t.out = powf(fmaxf(t.res, kClampEps), B.h1);
  return t.out - 1.f;
}

// d sdf / d (S, R, T, eps1, eps2) times g, into gr[0..16] (autograd's chain
// through pow, clamp and the division; clamps pass the gradient where the
// input lies inside their bounds, ends included).
__device__ void sdf_backward(const Blk& B, const Sdf& t, float g, float* gr) {
  const float rc = fmaxf(t.res, kClampEps);
  const float d_rc = g * (B.h1 * powf(rc, B.h1 - 1.f));
  float d_e1 = g * (t.out * logf(rc)) * 0.5f;
  float d_e2 = 0.f;
  const float d_res = t.res >= kClampEps ? d_rc : 0.f;
  // res = Wc^r21 + Y
  const float Wc = fmaxf(t.W, kClampEps);
  const float d_Wc = d_res * (B.r21 * powf(Wc, B.r21 - 1.f));
  const float d_r21 = d_res * (t.P * logf(Wc));
  d_e2 += d_r21 / B.e1;
  d_e1 += -d_r21 * (B.r21 / B.e1);
  const float d_W = t.W >= kClampEps ? d_Wc : 0.f;
  // X, Z = max(a, e)^ie2 ; Y = max(a, e)^ie1
  const float dXYZ[3] = {d_W, d_res, d_W};
  const float val[3] = {t.X, t.Y, t.Z};
  float d_ie1 = 0.f, d_ie2 = 0.f, d_u[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const float ie = j == 1 ? B.ie1 : B.ie2;
    const float ac = fmaxf(t.a[j], kClampEps);
    const float d_ac = dXYZ[j] * (ie * powf(ac, ie - 1.f));
    const float d_ie = dXYZ[j] * (val[j] * logf(ac));
    if (j == 1) d_ie1 += d_ie; else d_ie2 += d_ie;
    const float d_a = t.a[j] >= kClampEps ? d_ac : 0.f;
    const float uc = fminf(fmaxf(t.u[j], -5.f), 5.f);
    const float d_uc = d_a * 2.f * uc;
    d_u[j] = (t.u[j] >= -5.f && t.u[j] <= 5.f) ? d_uc : 0.f;
  }
  d_e1 += -d_ie1 * (B.ie1 * B.ie1);
  d_e2 += -d_ie2 * (B.ie2 * B.ie2);
  float d_d[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const float d_q = d_u[j] / B.D[j];
    const float d_D = -d_u[j] * ((t.q[j] / B.D[j]) / B.D[j]);
    gr[j] += d_D * B.ratio;   // D = S ratio
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      gr[3 + 3 * j + k] += d_q * t.d[k];
      d_d[k] += d_q * B.R[3 * j + k];
    }
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) gr[12 + k] -= d_d[k];
  gr[15] += d_e1;
  gr[16] += d_e2;
}

// The reference's ray sample c of ray r: depth = ((jitter + c) / C) (far - near) + near
__device__ __forceinline__ void ray_point(const sgr_sq_loss_args& a, int r, int c, float& x, float& y, float& z) {
  const float t = __fadd_rn(__fmul_rn(__fdiv_rn(__fadd_rn(a.ray_jitter[(long long)r * a.n_samples + c], (float)c),
                                                (float)a.n_samples),
                                      a.far - a.near),
                            a.near);
  x = __fadd_rn(a.ray_origin[3 * r], __fmul_rn(a.ray_dir[3 * r], t));
  y = __fadd_rn(a.ray_origin[3 * r + 1], __fmul_rn(a.ray_dir[3 * r + 1], t));
  z = __fadd_rn(a.ray_origin[3 * r + 2], __fmul_rn(a.ray_dir[3 * r + 2], t));
}

// The overlap term's point i: a unit-cube sample u of block src = i / P,
// placed by that block: w = (u ratio S) R + T
__device__ __forceinline__ void overlap_point(const sgr_sq_loss_args& a, const Blk& B, long long i, float& x, float& y,
                                              float& z) {
  float v[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) v[k] = (a.overlap_unit[3 * i + k] * a.ratio) * B.S[k];
  x = v[0] * B.R[0] + v[1] * B.R[3] + v[2] * B.R[6] + B.T[0];
  y = v[0] * B.R[1] + v[1] * B.R[4] + v[2] * B.R[7] + B.T[1];
  z = v[0] * B.R[2] + v[1] * B.R[5] + v[2] * B.R[8] + B.T[2];
}

struct Layout {
  size_t min_sdf, argmin, occ_max, occ_idx, stats, ovl_partial, grad_partial, end;
  int ray_ctas_fwd, ovl_ctas, ray_ctas_bwd;
};

Layout layout(const sgr_sq_loss_args& a) {
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  Layout L;
  const long long R = a.n_rays > 0 ? a.n_rays : 0;
  const long long M = a.n_overlap > 0 ? (long long)a.n_overlap * a.n_blocks : 0;
  L.ray_ctas_fwd = (int)((R + kRaysPerCta - 1) / kRaysPerCta);
  L.ray_ctas_bwd = (int)((R + kThreads - 1) / kThreads);
  L.ovl_ctas = (int)((M + kThreads - 1) / kThreads);
  size_t o = 0;
  L.min_sdf = o; o = al(o + 4 * R);
  L.argmin = o; o = al(o + 4 * R);
  L.occ_max = o; o = al(o + 4 * R);
  L.occ_idx = o; o = al(o + 4 * R);
  L.stats = o; o = al(o + 4 * 4);
  L.ovl_partial = o; o = al(o + 4 * (size_t)L.ovl_ctas);
  L.grad_partial = o; o = al(o + 4 * (size_t)(L.ray_ctas_bwd + L.ovl_ctas) * a.n_blocks * kG);
  L.end = o;
  return L;
}

// Deterministic CTA sum of one value per thread (fixed tree order); every
// thread gets the total.
__device__ float cta_sum(float v, float* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  float s = 0.f;
  for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[k];
  return s;
}

__device__ __forceinline__ bool lt_idx(float v, int i, float bv, int bi) { return v < bv || (v == bv && i < bi); }
__device__ __forceinline__ bool gt_idx(float v, int i, float bv, int bi) { return v > bv || (v == bv && i < bi); }

__global__ void __launch_bounds__(kThreads) k_sq_forward(sgr_sq_loss_args a, Layout L, char* __restrict__ scratch) {
  __shared__ Blk s_blk[SGR_SQ_MAX_BLOCKS];
  __shared__ float s_red[kThreads / 32];
  const int N = a.n_blocks;
  for (int b = threadIdx.x; b < N; b += blockDim.x) load_block(a, b, s_blk[b]);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  if ((int)blockIdx.x < L.ray_ctas_fwd) {
    const int r = blockIdx.x * kRaysPerCta + (threadIdx.x >> 5);
    if (r >= a.n_rays) return;
    const int C = a.n_samples;
    float best = FLT_MAX, occ = 0.f;
    int bi = INT_MAX, oi = 0;
    for (int c = lane; c < C; c += 32) {
      float x, y, z;
      ray_point(a, r, c, x, y, z);
      for (int b = 0; b < N; ++b) {
        Sdf t;
        const float s = sdf_eval(s_blk[b], x, y, z, t);
        const int idx = b * C + c;
        if (lt_idx(s, idx, best, bi)) {
          best = s;
          bi = idx;
        }
        if (s <= 1e-8f && gt_idx(s_blk[b].alpha, idx, occ, oi)) {
          occ = s_blk[b].alpha;
          oi = idx;
        }
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float vb = __shfl_xor_sync(0xffffffffu, best, o);
      const int ib = __shfl_xor_sync(0xffffffffu, bi, o);
      if (lt_idx(vb, ib, best, bi)) {
        best = vb;
        bi = ib;
      }
      const float vo = __shfl_xor_sync(0xffffffffu, occ, o);
      const int io = __shfl_xor_sync(0xffffffffu, oi, o);
      if (gt_idx(vo, io, occ, oi)) {
        occ = vo;
        oi = io;
      }
    }
    if (lane == 0) {
      reinterpret_cast<float*>(scratch + L.min_sdf)[r] = best;
      reinterpret_cast<int*>(scratch + L.argmin)[r] = bi;
      reinterpret_cast<float*>(scratch + L.occ_max)[r] = occ;
      reinterpret_cast<int*>(scratch + L.occ_idx)[r] = oi;
    }
    return;
  }
  // overlap: a thread per point, clamp(sum_b occupancy_b - max_blocks, 0)
  const int cta = blockIdx.x - L.ray_ctas_fwd;
  const long long M = (long long)a.n_overlap * N;
  const long long i = (long long)cta * kThreads + threadIdx.x;
  float v = 0.f;
  if (i < M) {
    float x, y, z;
    overlap_point(a, s_blk[i / a.n_overlap], i, x, y, z);
    const float inv_t = 1.0f / a.overlap_temperature;
    float sum = 0.f;
    for (int b = 0; b < N; ++b) {
      Sdf t;
      const float s = sdf_eval(s_blk[b], x, y, z, t);
      sum += sigmoidf(-s * inv_t) * s_blk[b].alpha_n;
    }
    v = fmaxf(sum - a.overlap_max_blocks, 0.f);
  }
  const float tot = cta_sum(v, s_red);
  if (threadIdx.x == 0) reinterpret_cast<float*>(scratch + L.ovl_partial)[cta] = tot;
}

// One CTA: the three ray losses and the overlap mean.
__global__ void __launch_bounds__(1024) k_sq_finish(sgr_sq_loss_args a, Layout L, char* __restrict__ scratch) {
  __shared__ double s_red[5][32];
  const float* min_sdf = reinterpret_cast<const float*>(scratch + L.min_sdf);
  const float* occ_max = reinterpret_cast<const float*>(scratch + L.occ_max);
  double v[5] = {0, 0, 0, 0, 0};   // sum in, n in, sum out, n out, bce
  for (int r = threadIdx.x; r < a.n_rays; r += blockDim.x) {
    const float y = a.ray_label[r], m = min_sdf[r];
    if (y > 0.5f) {
      v[0] += fmaxf(m - 1e-3f, 0.f);
      v[1] += 1.0;
    }
    if (y < 0.5f) {
      v[2] += fmaxf(-m - 1e-3f, 0.f);
      v[3] += 1.0;
    }
    const float x = fminf(fmaxf(occ_max[r], 1e-3f), 0.999f);
    v[4] += (double)((y - 1.f) * fmaxf(log1pf(-x), -100.f) - y * fmaxf(logf(x), -100.f));
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    double x = v[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (l == 0) s_red[k][w] = x;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  double t[5] = {0, 0, 0, 0, 0};
  for (int k = 0; k < 5; ++k)
    for (int j = 0; j < (int)(blockDim.x >> 5); ++j) t[k] += s_red[k][j];
  float* stats = reinterpret_cast<float*>(scratch + L.stats);
  stats[0] = (float)t[1];
  stats[1] = (float)t[3];
  if (a.n_rays > 0) {
    a.losses[0] = (float)(t[0] / t[1]);   // mean over rays inside the mask (NaN when none, like torch)
    a.losses[1] = (float)(t[2] / t[3]);   // sum over rays outside / their count
    a.losses[2] = (float)(t[4] / a.n_rays);
  } else {
    a.losses[0] = a.losses[1] = a.losses[2] = 0.f;
  }
  double o = 0;
  const float* part = reinterpret_cast<const float*>(scratch + L.ovl_partial);
  for (int c = 0; c < L.ovl_ctas; ++c) o += part[c];
  a.losses[3] = L.ovl_ctas ? (float)(o / ((double)a.n_overlap * a.n_blocks)) : 0.f;
}

// Adds the CTA's sum of each thread's kG values into out[0..kG) (fixed
// order: warp butterflies, then the warps in order).  Every thread calls it.
__device__ void cta_sum_vec(const float* v, float (*s_vec)[kG], float* out) {
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
  for (int k = 0; k < kG; ++k) {
    float x = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (l == 0) s_vec[w][k] = x;
  }
  __syncthreads();
  if (threadIdx.x < kG) {
    float t = 0.f;
    for (int j = 0; j < (int)(blockDim.x >> 5); ++j) t += s_vec[j][threadIdx.x];
    out[threadIdx.x] = t;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kThreads) k_sq_backward(sgr_sq_loss_args a, Layout L, char* __restrict__ scratch,
                                                          const float* __restrict__ d_losses) {
  __shared__ Blk s_blk[SGR_SQ_MAX_BLOCKS];
  __shared__ float s_vec[kThreads / 32][kG];
  const int N = a.n_blocks;
  for (int b = threadIdx.x; b < N; b += blockDim.x) load_block(a, b, s_blk[b]);
  __syncthreads();
  float* partial = reinterpret_cast<float*>(scratch + L.grad_partial) + (size_t)blockIdx.x * N * kG;
  if ((int)blockIdx.x < L.ray_ctas_bwd) {
    // a thread per ray: the SDF gradient at its minimum's (block, sample), and
    // the occupancy gradient through the alpha of its maximum's block
    const int r = blockIdx.x * kThreads + threadIdx.x;
    float gr[kG];
#pragma unroll
    for (int k = 0; k < kG; ++k) gr[k] = 0.f;
    int gb = -1, ob = -1;
    float oc = 0.f;
    if (r < a.n_rays) {
      const float* stats = reinterpret_cast<const float*>(scratch + L.stats);
      const float y = a.ray_label[r];
      const float m = reinterpret_cast<const float*>(scratch + L.min_sdf)[r];
      const int bi = reinterpret_cast<const int*>(scratch + L.argmin)[r];
      const int C = a.n_samples;
      float g = 0.f;
      if (y > 0.5f && m - 1e-3f >= 0.f) g += d_losses[0] / stats[0];
      if (y < 0.5f && -m - 1e-3f >= 0.f) g -= d_losses[1] / stats[1];
      if (g != 0.f) {
        gb = bi / C;
        float x, yy, z;
        ray_point(a, r, bi % C, x, yy, z);
        Sdf t;
        sdf_eval(s_blk[gb], x, yy, z, t);
        sdf_backward(s_blk[gb], t, g, gr);
      }
      const float om = reinterpret_cast<const float*>(scratch + L.occ_max)[r];
      if (om >= 1e-3f && om <= 0.999f) {   // BCE(clip(max occupancy), y); clip passes inside its bounds
        const float dx = d_losses[2] / (float)a.n_rays * (om - y) / fmaxf((1.f - om) * om, 1e-12f);
        ob = reinterpret_cast<const int*>(scratch + L.occ_idx)[r] / C;
        const float al = s_blk[ob].alpha;
        oc = dx * (al * (1.f - al));
      }
    }
    for (int b = 0; b < N; ++b) {
      if (!__syncthreads_or(gb == b || ob == b)) {
        if (threadIdx.x < kG) partial[b * kG + threadIdx.x] = 0.f;
        continue;
      }
      float v[kG];
#pragma unroll
      for (int k = 0; k < kG; ++k) v[k] = gb == b ? gr[k] : 0.f;
      v[kG - 1] += ob == b ? oc : 0.f;
      cta_sum_vec(v, s_vec, partial + b * kG);
    }
    return;
  }
  // overlap: a thread per point, the gradient of every block's occupancy
  // where the point's clamp(sum - max_blocks, 0) is active
  const int cta = blockIdx.x - L.ray_ctas_bwd;
  const long long M = (long long)a.n_overlap * N;
  const long long i = (long long)cta * kThreads + threadIdx.x;
  bool active = false;
  float x = 0.f, y = 0.f, z = 0.f;
  const float inv_t = 1.0f / a.overlap_temperature;
  if (i < M) {
    overlap_point(a, s_blk[i / a.n_overlap], i, x, y, z);
    float sum = 0.f;
    for (int b = 0; b < N; ++b) {
      Sdf t;
      const float s = sdf_eval(s_blk[b], x, y, z, t);
      sum += sigmoidf(-s * inv_t) * s_blk[b].alpha_n;
    }
    active = sum - a.overlap_max_blocks >= 0.f;
  }
  const bool any = __syncthreads_or(active);
  const float g = active ? d_losses[3] / (float)((double)a.n_overlap * N) : 0.f;
  for (int b = 0; b < N; ++b) {
    if (!any) {
      if (threadIdx.x < kG) partial[b * kG + threadIdx.x] = 0.f;
      continue;
    }
    float gr[kG];
#pragma unroll
    for (int k = 0; k < kG; ++k) gr[k] = 0.f;
    if (active) {
      const Blk& B = s_blk[b];
      Sdf t;
      const float s = sdf_eval(B, x, y, z, t);
      const float sg = sigmoidf(-s * inv_t);
      const float d_x = g * B.alpha_n * (sg * (1.f - sg));   // through sigmoid(-sdf / temperature)
      sdf_backward(B, t, -(d_x * inv_t), gr);
      gr[kG - 1] = g * sg * (B.alpha_n * (1.f - B.alpha_n));   // through sigmoid(occ_logit + noise)
    }
    cta_sum_vec(gr, s_vec, partial + b * kG);
  }
}

__global__ void k_sq_grad_reduce(sgr_sq_loss_args a, Layout L, const char* __restrict__ scratch) {
  const int N = a.n_blocks;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= N * kG) return;
  const float* part = reinterpret_cast<const float*>(scratch + L.grad_partial);
  const int ctas = L.ray_ctas_bwd + L.ovl_ctas;
  float s = 0.f;
  for (int c = 0; c < ctas; ++c) s += part[(size_t)c * N * kG + e];
  const int b = e / kG, k = e % kG;
  if (k < 3) a.d_S[3 * b + k] = s;
  else if (k < 12) a.d_R[9 * b + (k - 3)] = s;
  else if (k < 15) a.d_T[3 * b + (k - 12)] = s;
  else if (k == 15) a.d_eps1[b] = s;
  else if (k == 16) a.d_eps2[b] = s;
  else if (a.d_occ_logit) a.d_occ_logit[b] = s;
}

__global__ void k_sq_sdf(sgr_sq_loss_args a, const float* __restrict__ pts, long long M, float* __restrict__ out) {
  __shared__ Blk s_blk[SGR_SQ_MAX_BLOCKS];
  for (int b = threadIdx.x; b < a.n_blocks; b += blockDim.x) load_block(a, b, s_blk[b]);
  __syncthreads();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M) return;
  const float x = pts[3 * i], y = pts[3 * i + 1], z = pts[3 * i + 2];
  for (int b = 0; b < a.n_blocks; ++b) {
    Sdf t;
    out[(long long)b * M + i] = sdf_eval(s_blk[b], x, y, z, t);
  }
}

int check(const sgr_sq_loss_args* a) {
  if (!a || a->n_blocks < 1 || a->n_blocks > SGR_SQ_MAX_BLOCKS || !a->S || !a->R || !a->T || !a->eps1 || !a->eps2 ||
      !(a->ratio > 0.f))
    return SGR_ERR_INVALID_ARGUMENT;
  if (a->n_rays < 0 || a->n_overlap < 0) return SGR_ERR_INVALID_ARGUMENT;
  if (a->n_rays > 0 && (a->n_samples < 1 || a->n_samples > (1 << 20) / a->n_blocks || !a->ray_origin ||
                        !a->ray_dir || !a->ray_jitter || !a->ray_label))
    return SGR_ERR_INVALID_ARGUMENT;
  if (a->n_overlap > 0 && (!a->overlap_unit || !(a->overlap_temperature > 0.f))) return SGR_ERR_INVALID_ARGUMENT;
  if ((long long)a->n_overlap * a->n_blocks > (1LL << 30)) return SGR_ERR_UNSUPPORTED;
  return SGR_OK;
}

}  // namespace sgrsq

using namespace sgrsq;

extern "C" {

size_t sgr_sq_scratch_bytes(const sgr_sq_loss_args* a) {
  if (check(a) != SGR_OK) return 0;
  return layout(*a).end;
}

int sgr_sq_losses_forward(const sgr_sq_loss_args* a, void* stream) {
  int rc = check(a);
  if (rc) return rc;
  if (!a->losses) return SGR_ERR_INVALID_ARGUMENT;
  const Layout L = layout(*a);
  if (!a->scratch || a->scratch_bytes < L.end) return SGR_ERR_WORKSPACE;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* sp = static_cast<char*>(a->scratch);
  const int ctas = L.ray_ctas_fwd + L.ovl_ctas;
  if (ctas > 0) {
    k_sq_forward<<<ctas, kThreads, 0, st>>>(*a, L, sp);
    sgr::count_launches(1);
  }
  k_sq_finish<<<1, 1024, 0, st>>>(*a, L, sp);
  sgr::count_launches(1);
  return cudaGetLastError() == cudaSuccess ? SGR_OK : SGR_ERR_CUDA;
}

int sgr_sq_losses_backward(const sgr_sq_loss_args* a, const float* d_losses, void* stream) {
  int rc = check(a);
  if (rc) return rc;
  if (!d_losses || !a->d_S || !a->d_R || !a->d_T || !a->d_eps1 || !a->d_eps2) return SGR_ERR_INVALID_ARGUMENT;
  const Layout L = layout(*a);
  if (!a->scratch || a->scratch_bytes < L.end) return SGR_ERR_WORKSPACE;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* sp = static_cast<char*>(a->scratch);
  const int ctas = L.ray_ctas_bwd + L.ovl_ctas;
  if (ctas > 0) {
    k_sq_backward<<<ctas, kThreads, 0, st>>>(*a, L, sp, d_losses);
    sgr::count_launches(1);
  }
  const int e = a->n_blocks * kG;
  k_sq_grad_reduce<<<(e + 255) / 256, 256, 0, st>>>(*a, L, sp);
  sgr::count_launches(1);
  return cudaGetLastError() == cudaSuccess ? SGR_OK : SGR_ERR_CUDA;
}

int sgr_sq_sdf(const sgr_sq_loss_args* a, const float* points, int64_t n_points, float* out, void* stream) {
  if (!a || a->n_blocks < 1 || a->n_blocks > SGR_SQ_MAX_BLOCKS || !a->S || !a->R || !a->T || !a->eps1 ||
      !a->eps2 || !(a->ratio > 0.f) || n_points < 0 || (n_points > 0 && (!points || !out)))
    return SGR_ERR_INVALID_ARGUMENT;
  if (n_points == 0) return SGR_OK;
  k_sq_sdf<<<(unsigned)((n_points + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(*a, points, n_points,
                                                                                              out);
  sgr::count_launches(1);
  return cudaGetLastError() == cudaSuccess ? SGR_OK : SGR_ERR_CUDA;
}

}  // extern "C"
