// Backward kernels of the GB300 surfel rasteriser.
#include "sgr_kernels.cuh"

namespace sgr {

// ---------------------------------------------------------------------------
// preprocess backward: one thread per surfel, summing over its scene's views
// (P0/cr/backward.cu:443-630; P1/cr/backward.cu:473-671)
// ---------------------------------------------------------------------------
// sh and dsh_acc hold coefficient k, channel c at index (3 k + c) * STRIDE.
template <int STRIDE>
__device__ __forceinline__ void sh_backward(int deg, const float* sh, V3 dir_orig, uint32_t clamped, V3 dL_dRGB_in,
                                            float* dsh_acc, V3& dmean) {
  const float len = sqrtf(dot3(dir_orig, dir_orig));
  const V3 dir = v3(dir_orig.x / len, dir_orig.y / len, dir_orig.z / len);
  V3 g = dL_dRGB_in;
  g.x *= (clamped & 1u) ? 0 : 1;
  g.y *= (clamped & 2u) ? 0 : 1;
  g.z *= (clamped & 4u) ? 0 : 1;
  auto c = [&](int k) { return v3(sh[3 * k * STRIDE], sh[(3 * k + 1) * STRIDE], sh[(3 * k + 2) * STRIDE]); };
  auto add = [&](int k, float coef) {
    dsh_acc[3 * k * STRIDE] += coef * g.x;
    dsh_acc[(3 * k + 1) * STRIDE] += coef * g.y;
    dsh_acc[(3 * k + 2) * STRIDE] += coef * g.z;
  };
  V3 dx = v3(0, 0, 0), dy = v3(0, 0, 0), dz = v3(0, 0, 0);
  const float x = dir.x, y = dir.y, z = dir.z;
  add(0, kShC0);
  if (deg > 0) {
    add(1, -kShC1 * y);
    add(2, kShC1 * z);
    add(3, -kShC1 * x);
    dx = -kShC1 * c(3);
    dy = -kShC1 * c(1);
    dz = kShC1 * c(2);
    if (deg > 1) {
      const float xx = x * x, yy = y * y, zz = z * z;
      const float xy = x * y, yz = y * z, xz = x * z;
      add(4, kShC2[0] * xy);
      add(5, kShC2[1] * yz);
      add(6, kShC2[2] * (2.f * zz - xx - yy));
      add(7, kShC2[3] * xz);
      add(8, kShC2[4] * (xx - yy));
      dx = dx + kShC2[0] * y * c(4) + kShC2[2] * 2.f * -x * c(6) + kShC2[3] * z * c(7) + kShC2[4] * 2.f * x * c(8);
      dy = dy + kShC2[0] * x * c(4) + kShC2[1] * z * c(5) + kShC2[2] * 2.f * -y * c(6) + kShC2[4] * 2.f * -y * c(8);
      dz = dz + kShC2[1] * y * c(5) + kShC2[2] * 2.f * 2.f * z * c(6) + kShC2[3] * x * c(7);
      if (deg > 2) {
        add(9, kShC3[0] * y * (3.f * xx - yy));
        add(10, kShC3[1] * xy * z);
        add(11, kShC3[2] * y * (4.f * zz - xx - yy));
        add(12, kShC3[3] * z * (2.f * zz - 3.f * xx - 3.f * yy));
        add(13, kShC3[4] * x * (4.f * zz - xx - yy));
        add(14, kShC3[5] * z * (xx - yy));
        add(15, kShC3[6] * x * (xx - 3.f * yy));
        dx = dx + (kShC3[0] * c(9) * 3.f * 2.f * xy + kShC3[1] * c(10) * yz + kShC3[2] * c(11) * -2.f * xy +
                   kShC3[3] * c(12) * -3.f * 2.f * xz + kShC3[4] * c(13) * (-3.f * xx + 4.f * zz - yy) +
                   kShC3[5] * c(14) * 2.f * xz + kShC3[6] * c(15) * 3.f * (xx - yy));
        dy = dy + (kShC3[0] * c(9) * 3.f * (xx - yy) + kShC3[1] * c(10) * xz +
                   kShC3[2] * c(11) * (-3.f * yy + 4.f * zz - xx) + kShC3[3] * c(12) * -3.f * 2.f * yz +
                   kShC3[4] * c(13) * -2.f * xy + kShC3[5] * c(14) * -2.f * yz + kShC3[6] * c(15) * -3.f * 2.f * xy);
        dz = dz + (kShC3[1] * c(10) * xy + kShC3[2] * c(11) * 4.f * 2.f * yz +
                   kShC3[3] * c(12) * 3.f * (2.f * zz - xx - yy) + kShC3[4] * c(13) * 4.f * 2.f * xz +
                   kShC3[5] * c(14) * (xx - yy));
      }
    }
  }
  const V3 dL_ddir = v3(dot3(dx, g), dot3(dy, g), dot3(dz, g));
  dmean = dmean + dnormvdv(dir_orig, dL_ddir);
}

// The CTA's SH coefficients and their gradients live in shared memory,
// coefficient-major ([3 M][128]: conflict-free per thread), loaded and
// stored as contiguous runs of the [P, M, 3] arrays.
constexpr int kPreBwdThreads = 128;
#ifndef SGR_PREBWD_MIN_CTAS
#define SGR_PREBWD_MIN_CTAS 4
#endif

// One surfel of the preprocess backward: sh and dsh point at its column of
// the CTA's shared arrays (stride kPreBwdThreads).
template <int VARIANT>
__device__ __forceinline__ void preprocess_bwd_surfel(const sgr_batch& b, const GeomView& g,
                                                      const float* __restrict__ grads, const sgr_bwd_outputs& out,
                                                      int i, const float* sh, float* dsh) {
  const bool has_sh = b.shs != nullptr;
  const int s = find_scene(b.scenes, b.num_scenes, i);
  const sgr_scene_desc sd = b.scenes[s];
  const int local = i - sd.surfel_offset;
  const int W = b.width, H = b.height;
  const bool precomp = b.transmat_precomp != nullptr;
  const V3 p = v3(b.means3D[3 * i + 0], b.means3D[3 * i + 1], b.means3D[3 * i + 2]);
  float2 sc = make_float2(0.f, 0.f);
  float4 q = make_float4(1.f, 0.f, 0.f, 0.f);
  if (!precomp) {
    sc = make_float2(b.scales[2 * i + 0], b.scales[2 * i + 1]);
    q = reinterpret_cast<const float4*>(b.rotations)[i];
  }
  const M3 R = quat_to_rot(q);
  V3 dmean = v3(0, 0, 0), dcol = v3(0, 0, 0);
  float dsx = 0.f, dsy = 0.f, dop = 0.f;
  float4 drot = make_float4(0.f, 0.f, 0.f, 0.f);

  for (int vi = 0; vi < sd.view_count; ++vi) {
    const int v = sd.view_begin + vi;
    const sgr_view_desc vd = b.views[v];
    const int r = vd.record_offset + local;
    const float* gr = grads + (size_t)r * kGradF;
    const bool vis = g.radii[r] > 0;
    float* o2 = out.dL_dmeans2D ? out.dL_dmeans2D + (size_t)r * 3 : nullptr;
    float* oT = out.dL_dtransmat ? out.dL_dtransmat + (size_t)r * 9 : nullptr;
    if (!vis) {
      if (o2) o2[0] = o2[1] = o2[2] = 0.f;
      if (oT) for (int k = 0; k < 9; ++k) oT[k] = gr[k];
      continue;
    }
    const float* vm = b.viewmatrix + 16 * v;
    const float* pm = b.projmatrix + 16 * v;
    const float focal_x = W / (2.0f * vd.tanfovx);
    const float focal_y = H / (2.0f * vd.tanfovy);
    float dT[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) dT[k] = gr[k];
    const float dm2x = gr[9], dm2y = gr[10];
    const V3 dn = v3(gr[11], gr[12], gr[13]);
    const V3 dc = v3(gr[14], gr[15], gr[16]);
    dop += gr[17];
    dcol = dcol + dc;
    const float4 rc0 = g.records[(size_t)r * kRecF4 + 0];
    const float4 rc1 = g.records[(size_t)r * kRecF4 + 1];
    const float4 rc2 = g.records[(size_t)r * kRecF4 + 2];
    const float4 rc4 = g.records[(size_t)r * kRecF4 + 4];
    const float stored_depth = rc2.x;

    if (VARIANT == SGR_VARIANT_PLAIN) {
      // image size recovered from focal * tan * 2 with truncation, as
      // P0/cr/backward.cu:607-608 does (it can come out one pixel short)
      const int Wb = int(focal_x * vd.tanfovx * 2);
      const int Hb = int(focal_y * vd.tanfovy * 2);
      V3 T0, T1, T2, normal;
      V3 L0, L1;
      float4 P0c, P1c, P2c;
      if (precomp) {
        const float* tp = b.transmat_precomp + 9 * i;
        T0 = v3(tp[0], tp[1], tp[2]);
        T1 = v3(tp[3], tp[4], tp[5]);
        T2 = v3(tp[6], tp[7], tp[8]);
        normal = v3(0, 0, 0);
      } else {
        L0 = R.c[0] * sc.x;
        L1 = R.c[1] * sc.y;
        // P = world2ndc * ndc2pix (columns), with the recovered Wb, Hb
        const float4 w0 = make_float4(pm[0], pm[4], pm[8], pm[12]);
        const float4 w1 = make_float4(pm[1], pm[5], pm[9], pm[13]);
        const float4 w3 = make_float4(pm[3], pm[7], pm[11], pm[15]);
        const float wh = float(Wb) / 2.0f, wc = float(Wb - 1) / 2.0f;
        const float hh = float(Hb) / 2.0f, hc = float(Hb - 1) / 2.0f;
        P0c = make_float4(w0.x * wh + w3.x * wc, w0.y * wh + w3.y * wc, w0.z * wh + w3.z * wc, w0.w * wh + w3.w * wc);
        P1c = make_float4(w1.x * hh + w3.x * hc, w1.y * hh + w3.y * hc, w1.z * hh + w3.z * hc, w1.w * hh + w3.w * hc);
        P2c = w3;
        auto row = [&](float4 Pc) {
          return v3(L0.x * Pc.x + L0.y * Pc.y + L0.z * Pc.z, L1.x * Pc.x + L1.y * Pc.y + L1.z * Pc.z,
                    p.x * Pc.x + p.y * Pc.y + p.z * Pc.z + Pc.w);
        };
        T0 = row(P0c);
        T1 = row(P1c);
        T2 = row(P2c);
        normal = xform_vec43(R.c[2], vm);
      }
      V3 dT0 = v3(dT[0], dT[1], dT[2]), dT1 = v3(dT[3], dT[4], dT[5]), dT2 = v3(dT[6], dT[7], dT[8]);
      if (dm2x != 0 || dm2y != 0) {
        // adjoint of the screen-space centre (P0/cr/backward.cu:514-543)
        const V3 tv = v3(9.0f, 9.0f, -1.0f);
        const float d = dot3(tv, T2 * T2);
        const V3 fv = tv * (1.0f / d);
        const V3 a0 = dm2x * fv * T2;
        const V3 a1 = dm2y * fv * T2;
        V3 a3 = dm2x * fv * T0 + dm2y * fv * T1;
        const V3 dL_df = dm2x * T0 * T2 + dm2y * T1 * T2;
        const float dL_dd = (float)((double)dot3(dL_df, fv) * (-1.0 / (double)d));
        a3 = a3 + dL_dd * (tv * T2 * 2.0f);
        dT0 = dT0 + a0;
        dT1 = dT1 + a1;
        dT2 = dT2 + a3;
        if (precomp) {
          dT[0] = dT0.x; dT[1] = dT0.y; dT[2] = dT0.z;
          dT[3] = dT1.x; dT[4] = dT1.y; dT[5] = dT1.z;
          dT[6] = dT2.x; dT[7] = dT2.y; dT[8] = dT2.z;
        }
      }
      if (!precomp) {
        // dL/dM = P * dL/dT^T, columns (L0, L1, p)
        auto dMcol = [&](int c) {
          const float a = c == 0 ? dT0.x : (c == 1 ? dT0.y : dT0.z);
          const float bb = c == 0 ? dT1.x : (c == 1 ? dT1.y : dT1.z);
          const float cc = c == 0 ? dT2.x : (c == 1 ? dT2.y : dT2.z);
          return v3(P0c.x * a + P1c.x * bb + P2c.x * cc, P0c.y * a + P1c.y * bb + P2c.y * cc,
                    P0c.z * a + P1c.z * bb + P2c.z * cc);
        };
        const V3 dRS0 = dMcol(0), dRS1 = dMcol(1), dP = dMcol(2);
        V3 dtn = xform_vec43_t(dn, vm);
        const V3 pv = xform_point43(p, vm);
        const float cosv = -sum3(pv * normal);
        dtn = (cosv > 0 ? 1.f : -1.f) * dtn;
        M3 dR;
        dR.c[0] = dRS0 * sc.x;
        dR.c[1] = dRS1 * sc.y;
        dR.c[2] = dtn;
        const float4 dq = quat_to_rot_vjp(q, dR);
        drot = make_float4(drot.x + dq.x, drot.y + dq.y, drot.z + dq.z, drot.w + dq.w);
        dsx += dot3(dRS0, R.c[0]);
        dsy += dot3(dRS1, R.c[1]);
        dmean = dmean + dP;
      }
      // densification proxy (P0/cr/backward.cu:626-629)
      if (o2) {
        o2[0] = (float)((double)(dT[2] * stored_depth) * 0.5 * (double)float(Wb));
        o2[1] = (float)((double)(dT[5] * stored_depth) * 0.5 * (double)float(Hb));
        o2[2] = 0.f;
      }
    } else {
      // adjoint of the screen-space centre (P1/cr/backward.cu:621-671)
      const V3 T0 = v3(rc0.x, rc0.y, rc0.z), T1 = v3(rc0.w, rc1.x, rc1.y), T3 = v3(rc1.z, rc1.w, rc2.x);
      const V3 tv = v3(1.0f, 1.0f, -1.0f);
      const float d = dot3(tv, T3 * T3);
      const V3 fv = tv * (1.0f / d);
      const V3 a0 = dm2x * fv * T3;
      const V3 a1 = dm2y * fv * T3;
      V3 a3 = dm2x * fv * T0 + dm2y * fv * T1;
      const V3 dL_df = (dm2x * T0 * T3) + (dm2y * T1 * T3);
      const float dL_dd = (float)((double)dot3(dL_df, fv) * (-1.0 / (double)d));
      a3 = a3 + dL_dd * (tv * T3 * 2.0f);
      dT[0] += a0.x; dT[1] += a0.y; dT[2] += a0.z;
      dT[3] += a1.x; dT[4] += a1.y; dT[5] += a1.z;
      dT[6] += a3.x; dT[7] += a3.y; dT[8] += a3.z;
      if (o2) {
        const float z = T3.z;
        const float Wf = focal_x * vd.tanfovx, Hf = focal_y * vd.tanfovy;
        o2[0] = dT[2] * z * Wf;
        o2[1] = dT[5] * z * Hf;
        o2[2] = 0.f;
      }
      if (!precomp) {
        // computeTransMat adjoint (P1/cr/backward.cu:473-551)
        const float cxb = focal_x * vd.tanfovx, cyb = focal_y * vd.tanfovy;
        auto dMcol = [&](int c) {
          return v3(focal_x * dT[c], focal_y * dT[3 + c], cxb * dT[c] + cyb * dT[3 + c] + dT[6 + c]);
        };
        const V3 dRS0 = xform_vec43_t(dMcol(0), vm);
        const V3 dRS1 = xform_vec43_t(dMcol(1), vm);
        const V3 dpw = xform_vec43_t(dMcol(2), vm);
        V3 dtn = xform_vec43_t(dn, vm);
        const V3 tn = xform_vec43(R.c[2], vm);
        const V3 pv = xform_point43(p, vm);
        const float cosv = dot3(v3(-tn.x, -tn.y, -tn.z), pv);
        dtn = (cosv > 0 ? 1.f : -1.f) * dtn;
        M3 dR;
        dR.c[0] = dRS0 * sc.x;
        dR.c[1] = dRS1 * sc.y;
        dR.c[2] = dtn;
        const float4 dq = quat_to_rot_vjp(q, dR);
        drot = make_float4(drot.x + dq.x, drot.y + dq.y, drot.z + dq.z, drot.w + dq.w);
        dsx += dot3(dRS0, R.c[0]);
        dsy += dot3(dRS1, R.c[1]);
        dmean = dmean + dpw;
      }
    }
    if (oT)
      for (int k = 0; k < 9; ++k) oT[k] = dT[k];
    if (has_sh) {
      const V3 cp = v3(b.campos[3 * v], b.campos[3 * v + 1], b.campos[3 * v + 2]);
      sh_backward<kPreBwdThreads>(b.sh_degree, sh, p - cp, __float_as_uint(rc4.w), dc, dsh, dmean);
    }
  }
  if (out.dL_dmeans3D) {
    out.dL_dmeans3D[3 * i] = dmean.x;
    out.dL_dmeans3D[3 * i + 1] = dmean.y;
    out.dL_dmeans3D[3 * i + 2] = dmean.z;
  }
  if (out.dL_dscales) {
    out.dL_dscales[2 * i] = dsx;
    out.dL_dscales[2 * i + 1] = dsy;
  }
  if (out.dL_drotations) reinterpret_cast<float4*>(out.dL_drotations)[i] = drot;
  if (out.dL_dopacity) out.dL_dopacity[i] = dop;
  if (out.dL_dcolors) {
    out.dL_dcolors[3 * i] = dcol.x;
    out.dL_dcolors[3 * i + 1] = dcol.y;
    out.dL_dcolors[3 * i + 2] = dcol.z;
  }
}

template <int VARIANT>
__global__ void __launch_bounds__(kPreBwdThreads, SGR_PREBWD_MIN_CTAS)
    k_preprocess_bwd(const sgr_batch b, GeomView g, const float* __restrict__ grads, sgr_bwd_outputs out) {
  constexpr int NT = kPreBwdThreads;
  __shared__ float s_sh[kMaxShCoeffs * 3][NT];
  __shared__ float s_dsh[kMaxShCoeffs * 3][NT];
  const int i0 = blockIdx.x * NT;
  const int i = i0 + threadIdx.x;
  const int M = b.sh_coeffs;
  const int row = M * 3;
  const int here = min(NT, b.num_surfels - i0);
  const bool has_sh = b.shs != nullptr;
#pragma unroll
  for (int k = 0; k < kMaxShCoeffs * 3; ++k) {
    s_sh[k][threadIdx.x] = 0.f;
    s_dsh[k][threadIdx.x] = 0.f;
  }
  __syncthreads();
  if (has_sh)
    for (int e = threadIdx.x; e < here * row; e += NT) {
      const int t = e / row;
      s_sh[e - t * row][t] = b.shs[(size_t)i0 * row + e];
    }
  __syncthreads();
  if (i < b.num_surfels) preprocess_bwd_surfel<VARIANT>(b, g, grads, out, i, &s_sh[0][threadIdx.x],
                                                          &s_dsh[0][threadIdx.x]);
  __syncthreads();
  if (out.dL_dsh && M > 0)
    for (int e = threadIdx.x; e < here * row; e += NT) {
      const int t = e / row;
      out.dL_dsh[(size_t)i0 * row + e] = s_dsh[e - t * row][t];
    }
}

void launch_preprocess_bwd(const sgr_batch& b, const GeomView& g, const float* grads, const sgr_bwd_outputs& out,
                           cudaStream_t st) {
  const int threads = kPreBwdThreads;
  const int blocks = (b.num_surfels + threads - 1) / threads;
  if (blocks == 0) return;
  if (b.variant == SGR_VARIANT_PLAIN) k_preprocess_bwd<SGR_VARIANT_PLAIN><<<blocks, threads, 0, st>>>(b, g, grads, out);
  else k_preprocess_bwd<SGR_VARIANT_PART><<<blocks, threads, 0, st>>>(b, g, grads, out);
  count_launches();
}

}  // namespace sgr
