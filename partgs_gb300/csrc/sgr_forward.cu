// Forward kernels of the GB300 surfel rasteriser: preprocess (both
// variants), key duplication, tile ranges, blend, near-plane visibility.
#include "sgr_kernels.cuh"

namespace sgr {

// ---------------------------------------------------------------------------
// preprocess
// ---------------------------------------------------------------------------
// One thread per surfel; the surfel's attributes are read once and every view
// of its scene is processed from registers (the reference reads them once per
// view: P0/cr/forward.cu:148-251, P1/cr/forward.cu:166-260).
template <int VARIANT>
__global__ void __launch_bounds__(128) k_preprocess(const sgr_batch b, GeomView g) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.num_surfels) return;
  const int s = find_scene(b.scenes, b.num_scenes, i);
  const sgr_scene_desc sd = b.scenes[s];
  const int local = i - sd.surfel_offset;
  const int W = b.width, H = b.height;
  const int gx = g.tiles_x, gy = g.tiles_y;

  const V3 p = v3(b.means3D[3 * i + 0], b.means3D[3 * i + 1], b.means3D[3 * i + 2]);
  const float opac = b.opacities[i];
  const bool precomp = b.transmat_precomp != nullptr;
  float2 sc = make_float2(0.f, 0.f);
  float4 q = make_float4(1.f, 0.f, 0.f, 0.f);
  if (!precomp) {
    sc = make_float2(b.scales[2 * i + 0], b.scales[2 * i + 1]);
    q = reinterpret_cast<const float4*>(b.rotations)[i];
  }
  // SH coefficients live in registers for all views of this surfel.
  const int M = b.sh_coeffs;
  float sh[kMaxShCoeffs * 3];
  if (b.shs != nullptr) {
#pragma unroll
    for (int k = 0; k < kMaxShCoeffs * 3; ++k) sh[k] = (k < M * 3) ? b.shs[(size_t)i * M * 3 + k] : 0.f;
  }
  V3 cpre = v3(0.f, 0.f, 0.f);
  if (b.colors_precomp != nullptr)
    cpre = v3(b.colors_precomp[3 * i + 0], b.colors_precomp[3 * i + 1], b.colors_precomp[3 * i + 2]);

  for (int vi = 0; vi < sd.view_count; ++vi) {
    const int v = sd.view_begin + vi;
    const sgr_view_desc vd = b.views[v];
    const int r = vd.record_offset + local;
    const float* vm = b.viewmatrix + 16 * v;
    const float* pm = b.projmatrix + 16 * v;
    g.radii[r] = 0;
    g.tiles_touched[r] = 0;
    g.depth_keys[r] = ((unsigned long long)v << 32) | 0xffffffffull;
    g.depth_vals[r] = (uint32_t)r;

    // near-plane test (in_frustum, P0/cr/auxiliary.h:185-210)
    const V3 pv = xform_point43(p, vm);
    if (pv.z <= 0.2f) {
      if (b.prefiltered) atomicOr(&g.status->flags, SGR_FLAG_PREFILTERED);
      continue;
    }
    const float focal_x = W / (2.0f * vd.tanfovx);
    const float focal_y = H / (2.0f * vd.tanfovy);

    V3 Tu, Tv, Tw, normal;
    if (precomp) {
      const float* t = b.transmat_precomp + 9 * i;
      Tu = v3(t[0], t[1], t[2]);
      Tv = v3(t[3], t[4], t[5]);
      Tw = v3(t[6], t[7], t[8]);
      normal = (VARIANT == SGR_VARIANT_PLAIN) ? v3(0.f, 0.f, 1.f) : v3(0.f, 0.f, 0.f);
    } else if (VARIANT == SGR_VARIANT_PLAIN) {
      // splat-to-pixel homography T = splat2world^T * world2ndc * ndc2pix
      // (P0/cr/forward.cu:75-115)
      const M3 R = quat_to_rot(q);
      const float mod = b.scale_modifier;
      const V3 L0 = R.c[0] * (mod * sc.x);
      const V3 L1 = R.c[1] * (mod * sc.y);
      // X[j] = (L0, L1, p-hom) . world2ndc column j
      auto xcol = [&](int j) {
        return v3(L0.x * pm[j] + L0.y * pm[4 + j] + L0.z * pm[8 + j],
                  L1.x * pm[j] + L1.y * pm[4 + j] + L1.z * pm[8 + j],
                  p.x * pm[j] + p.y * pm[4 + j] + p.z * pm[8 + j] + pm[12 + j]);
      };
      const V3 X0 = xcol(0), X1 = xcol(1), X3 = xcol(3);
      const float wh = float(W) / 2.0f, wc = float(W - 1) / 2.0f;
      const float hh = float(H) / 2.0f, hc = float(H - 1) / 2.0f;
      Tu = X0 * wh + X3 * wc;
      Tv = X1 * hh + X3 * hc;
      Tw = X3;
      normal = xform_vec43(R.c[2], vm);
    } else {
      // camera-space homography (P1/cr/forward.cu:75-128)
      const M3 R = quat_to_rot(q);
      const V3 m0 = xform_vec43(R.c[0] * sc.x, vm);
      const V3 m1 = xform_vec43(R.c[1] * sc.y, vm);
      V3 tn = xform_vec43(R.c[2], vm);
      const float cosv = dot3(v3(-tn.x, -tn.y, -tn.z), pv);
      if (cosv == 0.0f) continue;
      tn = (cosv > 0 ? 1.f : -1.f) * tn;
      const float cx = (float)(W / 2.0), cy = (float)(H / 2.0);
      Tu = v3(focal_x * m0.x + cx * m0.z, focal_x * m1.x + cx * m1.z, focal_x * pv.x + cx * pv.z);
      Tv = v3(focal_y * m0.y + cy * m0.z, focal_y * m1.y + cy * m1.z, focal_y * pv.y + cy * pv.z);
      Tw = v3(m0.z, m1.z, pv.z);
      normal = tn;
    }
    if (VARIANT == SGR_VARIANT_PLAIN) {
      // dual visibility: orient the normal toward the camera (P0/cr/forward.cu:209-214)
      const float cosv = -sum3(pv * normal);
      if (cosv == 0.f) continue;
      normal = (cosv > 0 ? 1.f : -1.f) * normal;
    }

    // screen-space centre and extent (P0/cr/forward.cu:119-145, P1/cr/forward.cu:133-163)
    float cxp, cyp, radius;
    {
      const V3 tw2 = Tw * Tw;
      if (VARIANT == SGR_VARIANT_PLAIN) {
        const V3 t = v3(9.f, 9.f, -1.f);
        const float d = dot3(t, tw2);
        if (d == 0.0f) continue;
        const V3 f = (1 / d) * t;
        cxp = dot3(f, Tu * Tw);
        cyp = dot3(f, Tv * Tw);
        const float h0x = cxp * cxp - dot3(f, Tu * Tu);
        const float h0y = cyp * cyp - dot3(f, Tv * Tv);
        const float hx = sqrtf(fmaxf(1e-4f, h0x));
        const float hy = sqrtf(fmaxf(1e-4f, h0y));
        radius = ceilf(fmaxf(fmaxf(hx, hy), 3.0f * kFilterSizeP0));
      } else {
        const V3 t = v3(1.f, 1.f, -1.f);
        const float d = dot3(t, tw2);
        if (d == 0.0f) continue;
        const V3 f = t * (1.0f / d);
        cxp = dot3(f, Tu * Tw);
        cyp = dot3(f, Tv * Tw);
        const float h0x = cxp * cxp - dot3(f, Tu * Tu);
        const float h0y = cyp * cyp - dot3(f, Tv * Tv);
        const float hx = sqrtf(fmaxf(0.f, h0x));
        const float hy = sqrtf(fmaxf(0.f, h0y));
        radius = (float)ceil(3.0 * fmax((double)fmaxf(hx, hy), kFilterSizeP1));
      }
    }
    int x0, y0, x1, y1;
    tile_rect(cxp, cyp, (int)radius, gx, gy, x0, y0, x1, y1);
    const int touched = (y1 - y0) * (x1 - x0);
    if (touched == 0) continue;

    // view-dependent colour (P0/cr/forward.cu:20-71)
    V3 rgb = cpre;
    uint32_t clamped = 0;
    if (b.shs != nullptr) rgb = sh_to_rgb(b.sh_degree, sh, p, v3(b.campos[3 * v], b.campos[3 * v + 1], b.campos[3 * v + 2]), clamped);

    float reach_c;
    float4 box;
    reach_box(Tu, Tv, Tw, cxp, cyp, opac, reach_c, box);
    float4* rec = g.records + (size_t)r * kRecF4;
    rec[0] = make_float4(Tu.x, Tu.y, Tu.z, Tv.x);
    rec[1] = make_float4(Tv.y, Tv.z, Tw.x, Tw.y);
    rec[2] = make_float4(Tw.z, cxp, cyp, opac);
    rec[3] = make_float4(normal.x, normal.y, normal.z, reach_c);
    rec[4] = make_float4(rgb.x, rgb.y, rgb.z, __uint_as_float(clamped));
    rec[5] = box;
    g.radii[r] = (int)radius;
    g.tiles_touched[r] = (uint32_t)touched;
    g.depth_keys[r] = ((unsigned long long)v << 32) | (unsigned long long)__float_as_uint(pv.z);
  }
}

__global__ void k_store_key_count(GeomView g, long long R) {
  if (threadIdx.x == 0 && blockIdx.x == 0) g.status->num_keys = R > 0 ? g.offsets[R - 1] : 0ull;
}

// Near-plane visibility (P0/cr/rasterizer_impl.cu:54-66).
__global__ void k_mark_visible(int P, const float* __restrict__ means3D, const float* __restrict__ viewmatrix,
                               uint8_t* __restrict__ present) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P) return;
  const V3 p = v3(means3D[3 * i], means3D[3 * i + 1], means3D[3 * i + 2]);
  present[i] = xform_point43(p, viewmatrix).z > 0.2f ? 1 : 0;
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
void launch_preprocess(const sgr_batch& b, const GeomView& g, cudaStream_t st) {
  const int threads = 128;
  const int blocks = (b.num_surfels + threads - 1) / threads;
  if (blocks == 0) return;
  if (b.variant == SGR_VARIANT_PLAIN) k_preprocess<SGR_VARIANT_PLAIN><<<blocks, threads, 0, st>>>(b, g);
  else k_preprocess<SGR_VARIANT_PART><<<blocks, threads, 0, st>>>(b, g);
  count_launches();
}

void launch_store_key_count(const GeomView& g, long long R, cudaStream_t st) {
  k_store_key_count<<<1, 32, 0, st>>>(g, R);
  count_launches();
}

void launch_mark_visible(int P, const float* means3D, const float* viewmatrix, uint8_t* present, cudaStream_t st) {
  const int threads = 256;
  const int blocks = (P + threads - 1) / threads;
  if (blocks == 0) return;
  k_mark_visible<<<blocks, threads, 0, st>>>(P, means3D, viewmatrix, present);
  count_launches();
}

}  // namespace sgr
