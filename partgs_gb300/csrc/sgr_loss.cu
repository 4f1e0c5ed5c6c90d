// Fused point-level training loss: value and gradients in one pass.
//
// Restates, for a batch of views, the loss of the reference's point stage:
//   photometric  (1 - ls) L1 + ls (1 - SSIM)      train.py:229-231,
//                                                 utils/loss_utils.py:8-54
//   distortion   ld mean(rend_dist)               train.py:247
//   normal       ln mean(1 - n_render . n_surf)   train.py:244-246,
//       n_render = rendered normal in world space (renderer/gaussian_renderer/__init__.py:115-117)
//       n_surf   = normals of the surface depth from finite differences of the
//                  back-projected depth map (utils/point_utils.py:4-33) times
//                  the detached alpha (renderer/gaussian_renderer/__init__.py:135-141)
// The gradients are the exact adjoints of those PyTorch expressions.
//
// SSIM uses the 11-tap Gaussian (sigma 1.5) with zero padding, evaluated as
// two separable passes over a shared-memory tile; its adjoint is three more
// separable convolutions: with g = dL/dSSIM(p),
//   dL/dx(q) = (w * A)(q) + 2 x(q) (w * B)(q) + y(q) (w * C)(q),
//   A = g (dS/dmu_x - 2 mu_x dS/dvar_x - mu_y dS/dcov),  B = g dS/dvar_x,  C = g dS/dcov.
#include <cuda_runtime.h>

#include <cmath>

#include "../../include/sgr.h"

namespace sgr {
void count_launches(int n);   // sgr_api.cu
}  // namespace sgr

namespace sgrloss {

constexpr int kR = 5;                 // window radius
constexpr int kTX = 32, kTY = 16;     // SSIM output tile
constexpr int kIX = kTX + 2 * kR, kIY = kTY + 2 * kR;
constexpr float kC1 = 0.01f * 0.01f, kC2 = 0.03f * 0.03f;

struct Weights {
  float g[2 * kR + 1];
};

Weights gaussian_weights() {
  // the reference builds them in double and normalises in float
  // (utils/loss_utils.py:13-15)
  Weights w;
  float raw[2 * kR + 1];
  float sum = 0.f;
  for (int k = 0; k <= 2 * kR; ++k) {
    raw[k] = (float)std::exp(-(double)((k - kR) * (k - kR)) / (2.0 * 1.5 * 1.5));
    sum += raw[k];
  }
  for (int k = 0; k <= 2 * kR; ++k) w.g[k] = raw[k] / sum;
  return w;
}

struct Accum {
  double l1, ssim, dist, normal;
};

__device__ __forceinline__ float block_sum(float v, float* sh) {
  for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  float t = 0.f;
  if (threadIdx.x == 0)
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sh[k];
  return t;
}

// SSIM forward per (view, channel) plane tile: the ssim map's partials A, B,
// C (already multiplied by dL/dSSIM), and the SSIM and L1 sums.
__global__ void __launch_bounds__(256) k_ssim_fwd(sgr_loss_args a, Weights w, float gscale, float* __restrict__ abc,
                                                  Accum* acc) {
  __shared__ float sx[kIY][kIX], sy[kIY][kIX];
  __shared__ float hs[5][kIY][kTX];
  __shared__ float red[8];
  const int plane = blockIdx.z;
  const int H = a.H, W = a.W;
  const size_t HW = (size_t)H * W;
  const float* X = a.color + plane * HW;
  const float* Y = a.target + plane * HW;
  const int ox = blockIdx.x * kTX, oy = blockIdx.y * kTY;
  for (int i = threadIdx.x; i < kIX * kIY; i += blockDim.x) {
    const int r = i / kIX, c = i - r * kIX;
    const int gy = oy + r - kR, gx = ox + c - kR;
    const bool in = gy >= 0 && gy < H && gx >= 0 && gx < W;
    sx[r][c] = in ? X[(size_t)gy * W + gx] : 0.f;
    sy[r][c] = in ? Y[(size_t)gy * W + gx] : 0.f;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kIY * kTX; i += blockDim.x) {
    const int r = i / kTX, c = i - r * kTX;
    float m1 = 0.f, m2 = 0.f, e11 = 0.f, e22 = 0.f, e12 = 0.f;
#pragma unroll
    for (int k = 0; k <= 2 * kR; ++k) {
      const float x = sx[r][c + k], y = sy[r][c + k], g = w.g[k];
      m1 += g * x;
      m2 += g * y;
      e11 += g * (x * x);
      e22 += g * (y * y);
      e12 += g * (x * y);
    }
    hs[0][r][c] = m1;
    hs[1][r][c] = m2;
    hs[2][r][c] = e11;
    hs[3][r][c] = e22;
    hs[4][r][c] = e12;
  }
  __syncthreads();
  float s_sum = 0.f, l1_sum = 0.f;
  for (int i = threadIdx.x; i < kTY * kTX; i += blockDim.x) {
    const int r = i / kTX, c = i - r * kTX;
    const int gy = oy + r, gx = ox + c;
    if (gy >= H || gx >= W) continue;
    float v[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k <= 2 * kR; ++k) {
      const float g = w.g[k];
#pragma unroll
      for (int q = 0; q < 5; ++q) v[q] += g * hs[q][r + k][c];
    }
    const float mu1 = v[0], mu2 = v[1];
    const float mu1_sq = mu1 * mu1, mu2_sq = mu2 * mu2, mu12 = mu1 * mu2;
    const float s11 = v[2] - mu1_sq, s22 = v[3] - mu2_sq, s12 = v[4] - mu12;
    const float n1 = 2 * mu12 + kC1, n2 = 2 * s12 + kC2;
    const float d1 = mu1_sq + mu2_sq + kC1, d2 = s11 + s22 + kC2;
    const float S = (n1 * n2) / (d1 * d2);
    s_sum += S;
    const float x = sx[r + kR][c + kR], y = sy[r + kR][c + kR];
    l1_sum += fabsf(x - y);
    const float dS_dmu1 = S * (2.f * mu2 / n1 - 2.f * mu1 / d1);
    const float dS_ds11 = -S / d2;
    const float dS_ds12 = 2.f * S / n2;
    const size_t pix = (size_t)gy * W + gx;
    float* o = abc + (size_t)plane * 3 * HW;
    o[pix] = gscale * (dS_dmu1 - 2.f * mu1 * dS_ds11 - mu2 * dS_ds12);
    o[HW + pix] = gscale * dS_ds11;
    o[2 * HW + pix] = gscale * dS_ds12;
  }
  const float ts = block_sum(s_sum, red);
  const float tl = block_sum(l1_sum, red);
  if (threadIdx.x == 0) {
    atomicAdd(&acc->ssim, (double)ts);
    atomicAdd(&acc->l1, (double)tl);
  }
}

// SSIM backward + L1 gradient per plane tile.
__global__ void __launch_bounds__(256) k_ssim_bwd(sgr_loss_args a, Weights w, float l1scale,
                                                  const float* __restrict__ abc, float* __restrict__ dcolor) {
  __shared__ float s[3][kIY][kIX];
  __shared__ float hs[3][kIY][kTX];
  const int plane = blockIdx.z;
  const int H = a.H, W = a.W;
  const size_t HW = (size_t)H * W;
  const float* in = abc + (size_t)plane * 3 * HW;
  const int ox = blockIdx.x * kTX, oy = blockIdx.y * kTY;
  for (int i = threadIdx.x; i < kIX * kIY; i += blockDim.x) {
    const int r = i / kIX, c = i - r * kIX;
    const int gy = oy + r - kR, gx = ox + c - kR;
    const bool ok = gy >= 0 && gy < H && gx >= 0 && gx < W;
    const size_t pix = (size_t)gy * W + gx;
#pragma unroll
    for (int q = 0; q < 3; ++q) s[q][r][c] = ok ? in[q * HW + pix] : 0.f;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kIY * kTX; i += blockDim.x) {
    const int r = i / kTX, c = i - r * kTX;
    float v0 = 0.f, v1 = 0.f, v2 = 0.f;
#pragma unroll
    for (int k = 0; k <= 2 * kR; ++k) {
      const float g = w.g[k];
      v0 += g * s[0][r][c + k];
      v1 += g * s[1][r][c + k];
      v2 += g * s[2][r][c + k];
    }
    hs[0][r][c] = v0;
    hs[1][r][c] = v1;
    hs[2][r][c] = v2;
  }
  __syncthreads();
  const float* X = a.color + plane * HW;
  const float* Y = a.target + plane * HW;
  for (int i = threadIdx.x; i < kTY * kTX; i += blockDim.x) {
    const int r = i / kTX, c = i - r * kTX;
    const int gy = oy + r, gx = ox + c;
    if (gy >= H || gx >= W) continue;
    float v0 = 0.f, v1 = 0.f, v2 = 0.f;
#pragma unroll
    for (int k = 0; k <= 2 * kR; ++k) {
      const float g = w.g[k];
      v0 += g * hs[0][r + k][c];
      v1 += g * hs[1][r + k][c];
      v2 += g * hs[2][r + k][c];
    }
    const size_t pix = (size_t)gy * W + gx;
    const float x = X[pix], y = Y[pix];
    const float d = x - y;
    const float sgn = d > 0.f ? 1.f : (d < 0.f ? -1.f : 0.f);
    dcolor[plane * HW + pix] = v0 + 2.f * x * v1 + y * v2 + l1scale * sgn;
  }
}

// Normal consistency and distortion: per view, 32x8 tiles with a two-pixel
// halo of back-projected surface points.
constexpr int kGX = 32, kGY = 8;

__device__ __forceinline__ float nan0(float v) { return isfinite(v) ? v : 0.f; }

__global__ void __launch_bounds__(256) k_geom(sgr_loss_args a, float kn, float kd, float* __restrict__ dothers,
                                              Accum* acc) {
  __shared__ float P[3][kGY + 4][kGX + 4];
  __shared__ float GX[3][kGY + 2][kGX + 2];   // dL/d(vertical difference) at tile + 1 halo
  __shared__ float GY[3][kGY + 2][kGX + 2];   // dL/d(horizontal difference)
  __shared__ float red[8];
  const int v = blockIdx.z;
  const int H = a.H, W = a.W;
  const size_t HW = (size_t)H * W;
  const float* oth = a.others + (size_t)v * 7 * HW;
  const float* Rm = a.view_to_world + 9 * v;
  const float* rb = a.ray_basis + 9 * v;
  const float* ro = a.ray_origin + 3 * v;
  const float r = a.depth_ratio;
  const int ox = blockIdx.x * kGX, oy = blockIdx.y * kGY;

  auto surf_depth = [&](int gy, int gx) {
    const size_t pix = (size_t)gy * W + gx;
    const float med = nan0(oth[5 * HW + pix]);
    const float ex = nan0(oth[pix] / oth[HW + pix]);
    return ex * (1.f - r) + r * med;
  };
  // back-projected surface points on the tile + 2 halo
  for (int i = threadIdx.x; i < (kGY + 4) * (kGX + 4); i += blockDim.x) {
    const int ly = i / (kGX + 4), lx = i - ly * (kGX + 4);
    const int gy = oy + ly - 2, gx = ox + lx - 2;
    float p0 = 0.f, p1 = 0.f, p2 = 0.f;
    if (gy >= 0 && gy < H && gx >= 0 && gx < W) {
      const float d = surf_depth(gy, gx);
      const float fx = (float)gx, fy = (float)gy;
      p0 = d * (fx * rb[0] + fy * rb[3] + rb[6]) + ro[0];
      p1 = d * (fx * rb[1] + fy * rb[4] + rb[7]) + ro[1];
      p2 = d * (fx * rb[2] + fy * rb[5] + rb[8]) + ro[2];
    }
    P[0][ly][lx] = p0;
    P[1][ly][lx] = p1;
    P[2][ly][lx] = p2;
  }
  __syncthreads();
  float err_sum = 0.f;
  // normals on the tile + 1 halo, and the adjoints of their differences
  for (int i = threadIdx.x; i < (kGY + 2) * (kGX + 2); i += blockDim.x) {
    const int ly = i / (kGX + 2), lx = i - ly * (kGX + 2);
    const int gy = oy + ly - 1, gx = ox + lx - 1;
    float gdx[3] = {0.f, 0.f, 0.f}, gdy[3] = {0.f, 0.f, 0.f};
    const bool in_img = gy >= 0 && gy < H && gx >= 0 && gx < W;
    const bool interior = gy >= 1 && gy < H - 1 && gx >= 1 && gx < W - 1;
    const bool own = ly >= 1 && ly <= kGY && lx >= 1 && lx <= kGX && in_img;
    float n[3] = {0.f, 0.f, 0.f};
    float dxv[3], dyv[3], cl = 0.f, cvec[3] = {0.f, 0.f, 0.f};
    if (interior) {
      const int py = ly + 1, px = lx + 1;     // position in P
      for (int k = 0; k < 3; ++k) {
        dxv[k] = P[k][py + 1][px] - P[k][py - 1][px];
        dyv[k] = P[k][py][px + 1] - P[k][py][px - 1];
      }
      cvec[0] = dxv[1] * dyv[2] - dxv[2] * dyv[1];
      cvec[1] = dxv[2] * dyv[0] - dxv[0] * dyv[2];
      cvec[2] = dxv[0] * dyv[1] - dxv[1] * dyv[0];
      cl = sqrtf(cvec[0] * cvec[0] + cvec[1] * cvec[1] + cvec[2] * cvec[2]);
      const float den = fmaxf(cl, 1e-12f);
      for (int k = 0; k < 3; ++k) n[k] = cvec[k] / den;
    }
    if (in_img) {
      const size_t pix = (size_t)gy * W + gx;
      const float alpha = oth[HW + pix];
      const float Nv[3] = {oth[2 * HW + pix], oth[3 * HW + pix], oth[4 * HW + pix]};
      float rend[3];
      for (int d = 0; d < 3; ++d) rend[d] = Nv[0] * Rm[d] + Nv[1] * Rm[3 + d] + Nv[2] * Rm[6 + d];
      if (own) {
        float dotp = 0.f;
        for (int d = 0; d < 3; ++d) dotp += rend[d] * (n[d] * alpha);
        err_sum += 1.f - dotp;
      }
      if (interior) {
        // dL/dn = -kn rend alpha; through n = c / max(|c|, eps); c = dx x dy
        float gn[3], gc[3];
        for (int d = 0; d < 3; ++d) gn[d] = -kn * rend[d] * alpha;
        if (cl > 1e-12f) {
          const float ng = n[0] * gn[0] + n[1] * gn[1] + n[2] * gn[2];
          for (int d = 0; d < 3; ++d) gc[d] = (gn[d] - n[d] * ng) / cl;
        } else {
          for (int d = 0; d < 3; ++d) gc[d] = gn[d] / 1e-12f;
        }
        gdx[0] = dyv[1] * gc[2] - dyv[2] * gc[1];      // dy x gc
        gdx[1] = dyv[2] * gc[0] - dyv[0] * gc[2];
        gdx[2] = dyv[0] * gc[1] - dyv[1] * gc[0];
        gdy[0] = gc[1] * dxv[2] - gc[2] * dxv[1];      // gc x dx
        gdy[1] = gc[2] * dxv[0] - gc[0] * dxv[2];
        gdy[2] = gc[0] * dxv[1] - gc[1] * dxv[0];
      }
      if (own) {
        // dL/dN_view[c] = -kn sum_d surf[d] R[c][d]
        float* go = dothers + (size_t)v * 7 * HW;
        for (int c = 0; c < 3; ++c) {
          float s = 0.f;
          for (int d = 0; d < 3; ++d) s += n[d] * alpha * Rm[3 * c + d];
          go[(2 + c) * HW + pix] = -kn * s;
        }
      }
    }
    for (int k = 0; k < 3; ++k) {
      GX[k][ly][lx] = gdx[k];
      GY[k][ly][lx] = gdy[k];
    }
  }
  __syncthreads();
  float dist_sum = 0.f;
  for (int i = threadIdx.x; i < kGY * kGX; i += blockDim.x) {
    const int ty = i / kGX, tx = i - ty * kGX;
    const int gy = oy + ty, gx = ox + tx;
    if (gy >= H || gx >= W) continue;
    const int ly = ty + 1, lx = tx + 1;          // position in GX / GY
    float gp[3];
    for (int k = 0; k < 3; ++k)
      gp[k] = GX[k][ly - 1][lx] - GX[k][ly + 1][lx] + GY[k][ly][lx - 1] - GY[k][ly][lx + 1];
    const float fx = (float)gx, fy = (float)gy;
    const float ray[3] = {fx * rb[0] + fy * rb[3] + rb[6], fx * rb[1] + fy * rb[4] + rb[7],
                          fx * rb[2] + fy * rb[5] + rb[8]};
    const float gs = ray[0] * gp[0] + ray[1] * gp[1] + ray[2] * gp[2];
    const size_t pix = (size_t)gy * W + gx;
    float* go = dothers + (size_t)v * 7 * HW;
    const float med_raw = oth[5 * HW + pix];
    go[5 * HW + pix] = isfinite(med_raw) ? r * gs : 0.f;
    const float D = oth[pix], A = oth[HW + pix];
    const float ex = D / A;
    if (isfinite(ex) && r != 1.f) {
      const float ge = (1.f - r) * gs;
      go[pix] = ge / A;
      go[HW + pix] = -ge * D / (A * A);
    } else {
      go[pix] = 0.f;
      go[HW + pix] = 0.f;
    }
    go[6 * HW + pix] = kd;
    dist_sum += oth[6 * HW + pix];
  }
  const float te = block_sum(err_sum, red);
  const float td = block_sum(dist_sum, red);
  if (threadIdx.x == 0) {
    atomicAdd(&acc->normal, (double)te);
    atomicAdd(&acc->dist, (double)td);
  }
}

__global__ void k_finalize(sgr_loss_args a, const Accum* acc, float* loss) {
  const double n3 = 3.0 * a.V * (double)a.H * a.W, n1 = (double)a.V * a.H * a.W;
  const double L = (1.0 - a.lambda_dssim) * acc->l1 / n3 + a.lambda_dssim * (1.0 - acc->ssim / n3) +
                   a.lambda_dist * acc->dist / n1 + a.lambda_normal * acc->normal / n1;
  *loss = (float)L;
}

}  // namespace sgrloss

using namespace sgrloss;

extern "C" {

size_t sgr_loss_scratch_bytes(const sgr_loss_args* a) {
  if (!a) return 0;
  return 256 + (size_t)a->V * 3 * 3 * a->H * a->W * sizeof(float);
}

int sgr_loss_forward_backward(const sgr_loss_args* a, float* loss, float* dL_dcolor, float* dL_dothers, void* scratch,
                              void* stream) {
  if (!a || !loss || !dL_dcolor || !dL_dothers || !scratch || a->V < 1 || a->H < 1 || a->W < 1)
    return SGR_ERR_INVALID_ARGUMENT;
  if (!a->color || !a->target || !a->others || !a->view_to_world || !a->ray_basis || !a->ray_origin)
    return SGR_ERR_INVALID_ARGUMENT;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  Accum* acc = static_cast<Accum*>(scratch);
  float* abc = reinterpret_cast<float*>(static_cast<char*>(scratch) + 256);
  if (cudaMemsetAsync(acc, 0, sizeof(Accum), st) != cudaSuccess) return SGR_ERR_CUDA;
  const Weights w = gaussian_weights();
  const double n3 = 3.0 * a->V * (double)a->H * a->W, n1 = (double)a->V * a->H * a->W;
  const dim3 grid_s((a->W + kTX - 1) / kTX, (a->H + kTY - 1) / kTY, 3 * a->V);
  k_ssim_fwd<<<grid_s, 256, 0, st>>>(*a, w, (float)(-a->lambda_dssim / n3), abc, acc);
  k_ssim_bwd<<<grid_s, 256, 0, st>>>(*a, w, (float)((1.0 - a->lambda_dssim) / n3), abc, dL_dcolor);
  const dim3 grid_g((a->W + kGX - 1) / kGX, (a->H + kGY - 1) / kGY, a->V);
  k_geom<<<grid_g, 256, 0, st>>>(*a, (float)(a->lambda_normal / n1), (float)(a->lambda_dist / n1), dL_dothers, acc);
  k_finalize<<<1, 1, 0, st>>>(*a, acc, loss);
  sgr::count_launches(4);
  return cudaGetLastError() == cudaSuccess ? SGR_OK : SGR_ERR_CUDA;
}

}  // extern "C"
