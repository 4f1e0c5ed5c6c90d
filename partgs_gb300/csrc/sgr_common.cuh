// Shared device definitions of the GB300 surfel rasteriser.
//
// Per-view surfel record (96 B, six float4, 16-B aligned), written by the
// preprocess and gathered by both blends:
//   r0 = (Tu.x, Tu.y, Tu.z, Tv.x)
//   r1 = (Tv.y, Tv.z, Tw.x, Tw.y)
//   r2 = (Tw.z, centre.x, centre.y, opacity)
//   r3 = (normal.x, normal.y, normal.z, reach threshold c)
//   r4 = (r, g, b, clamped bits as a float bit pattern)
//   r5 = (x_min, x_max, y_min, y_max) pixel box the surfel can reach
// Tu/Tv/Tw are the rows of the splat-to-pixel homography (the reference's
// transMat, cuda_rasterizer/forward.cu:75-115), the centre and normal are
// the reference's points_xy_image and normal_opacity.
//
// Reach: a fragment contributes only if opacity * exp(-rho/2) >= 1/255,
// i.e. rho <= 2 ln(255 opacity).  c is that bound with a safety margin, and
// r5 bounds every pixel centre whose rho (the smaller of the splat-space
// distance rho3d and the screen-space filter distance rho2d) can be <= c.
// Pixels outside the box, or with both distances above c, are skipped
// without evaluating them: the reference would skip them at its alpha test.
//
// Per-view gradient record (80 B, 20 floats), accumulated by the blend
// backward and reduced over views by the preprocess backward:
//   [0..8] dL/dT (Tu, Tv, Tw), [9..10] dL/dcentre, [11..13] dL/dnormal,
//   [14..16] dL/dcolour, [17] dL/dopacity, [18..19] unused.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/sgr.h"

namespace sgr {

constexpr int kTile = SGR_TILE;
constexpr int kBlock = kTile * kTile;
constexpr int kRecF4 = 6;          // float4 per record
constexpr int kGradF = 20;         // floats per gradient record
constexpr int kGradUsed = 18;
// Records per chunk of the depth order, and list entries per streaming window
// of a blend CTA (four per thread), sgr_binning.cu / sgr_blend.cu.
constexpr int kChunk = 4 * kBlock;
// Edge, in tiles, of the square cells records are binned into
// (sgr_binning.cu): the batch's cell_tiles, or the default.
__host__ __device__ inline int cell_tiles_of(const sgr_batch& b) {
  return b.cell_tiles > 0 ? b.cell_tiles : SGR_DEFAULT_CELL_TILES;
}

// Host-side count of this library's kernel launches (sgr_kernel_launches).
void count_launches(int n = 1);

// P0/cr/auxiliary.h:37-40 (float) and P1/cr/auxiliary.h:20-36 (double macros)
constexpr float kNearP0 = 0.2f;
constexpr float kFarP0 = 100.0f;
constexpr float kFilterSizeP0 = 0.707106f;
// 1 / filter size^2.  Both variants scale by exactly 2: the part variant's
// double constant 1 / 0.7071067811865476^2 times a float rounds to 2x.
constexpr float kFilterInvSquareP0 = 2.0f;
constexpr double kFilterSizeP1 = 0.7071067811865476;
constexpr double kNearP1 = 0.2;
constexpr double kFarP1 = 100.0;

// Spherical-harmonics constants of the degree-3 real basis.
__device__ __constant__ static const float kShC0 = 0.28209479177387814f;
__device__ __constant__ static const float kShC1 = 0.4886025119029199f;
__device__ __constant__ static const float kShC2[5] = {1.0925484305920792f, -1.0925484305920792f,
                                                        0.31539156525252005f, -1.0925484305920792f,
                                                        0.5462742152960396f};
__device__ __constant__ static const float kShC3[7] = {-0.5900435899266435f, 2.890611442640554f,
                                                        -0.4570457994644658f, 0.3731763325901154f,
                                                        -0.4570457994644658f, 1.445305721320277f,
                                                        -0.5900435899266435f};

struct V3 {
  float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator*(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V3 operator*(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float sum3(V3 a) { return a.x + a.y + a.z; }
__device__ __forceinline__ V3 cross3(V3 a, V3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// 3x3 matrix stored by columns: c[0], c[1], c[2].
struct M3 {
  V3 c[3];
};

// Rotation of a (w,x,y,z) quaternion after normalisation, columns as in
// P0/cr/auxiliary.h:213-235 (rsqrtf normalisation).
__device__ __forceinline__ M3 quat_to_rot(float4 q) {
  const float s = rsqrtf(q.w * q.w + q.x * q.x + q.y * q.y + q.z * q.z);
  const float w = q.x * s, x = q.y * s, y = q.z * s, z = q.w * s;
  M3 R;
  R.c[0] = v3(1.f - 2.f * (y * y + z * z), 2.f * (x * y + w * z), 2.f * (x * z - w * y));
  R.c[1] = v3(2.f * (x * y - w * z), 1.f - 2.f * (x * x + z * z), 2.f * (y * z + w * x));
  R.c[2] = v3(2.f * (x * z + w * y), 2.f * (y * z - w * x), 1.f - 2.f * (x * x + y * y));
  return R;
}

// Vector-Jacobian product of quat_to_rot; vR holds dL/dR by columns.  The
// result is with respect to the normalised components, stored (w,x,y,z) in
// (x,y,z,w) as P0/cr/auxiliary.h:238-282 does.
__device__ __forceinline__ float4 quat_to_rot_vjp(float4 q, const M3& vR) {
  const float s = rsqrtf(q.w * q.w + q.x * q.x + q.y * q.y + q.z * q.z);
  const float w = q.x * s, x = q.y * s, y = q.z * s, z = q.w * s;
  auto g = [&](int c, int r) -> float {
    const V3& col = vR.c[c];
    return r == 0 ? col.x : (r == 1 ? col.y : col.z);
  };
  float4 o;
  o.x = 2.f * (x * (g(1, 2) - g(2, 1)) + y * (g(2, 0) - g(0, 2)) + z * (g(0, 1) - g(1, 0)));
  o.y = 2.f * (-2.f * x * (g(1, 1) + g(2, 2)) + y * (g(0, 1) + g(1, 0)) + z * (g(0, 2) + g(2, 0)) +
               w * (g(1, 2) - g(2, 1)));
  o.z = 2.f * (x * (g(0, 1) + g(1, 0)) - 2.f * y * (g(0, 0) + g(2, 2)) + z * (g(1, 2) + g(2, 1)) +
               w * (g(2, 0) - g(0, 2)));
  o.w = 2.f * (x * (g(0, 2) + g(2, 0)) + y * (g(1, 2) + g(2, 1)) - 2.f * z * (g(0, 0) + g(1, 1)) +
               w * (g(0, 1) - g(1, 0)));
  return o;
}

// p * M for a column-major 4x4 stored as 16 floats (the matrices torch hands
// over are the transposed, row-vector form), P0/cr/auxiliary.h:79-118.
__device__ __forceinline__ V3 xform_point43(V3 p, const float* m) {
  return v3(m[0] * p.x + m[4] * p.y + m[8] * p.z + m[12], m[1] * p.x + m[5] * p.y + m[9] * p.z + m[13],
            m[2] * p.x + m[6] * p.y + m[10] * p.z + m[14]);
}
__device__ __forceinline__ V3 xform_vec43(V3 p, const float* m) {
  return v3(m[0] * p.x + m[4] * p.y + m[8] * p.z, m[1] * p.x + m[5] * p.y + m[9] * p.z,
            m[2] * p.x + m[6] * p.y + m[10] * p.z);
}
__device__ __forceinline__ V3 xform_vec43_t(V3 p, const float* m) {
  return v3(m[0] * p.x + m[1] * p.y + m[2] * p.z, m[4] * p.x + m[5] * p.y + m[6] * p.z,
            m[8] * p.x + m[9] * p.y + m[10] * p.z);
}

// d(normalize(v))/dv applied to dv, P0/cr/auxiliary.h:128-138.
__device__ __forceinline__ V3 dnormvdv(V3 v, V3 dv) {
  const float sum2 = v.x * v.x + v.y * v.y + v.z * v.z;
  const float inv = 1.0f / sqrtf(sum2 * sum2 * sum2);
  return v3(((sum2 - v.x * v.x) * dv.x - v.y * v.x * dv.y - v.z * v.x * dv.z) * inv,
            (-v.x * v.y * dv.x + (sum2 - v.y * v.y) * dv.y - v.z * v.y * dv.z) * inv,
            (-v.x * v.z * dv.x - v.y * v.z * dv.y + (sum2 - v.z * v.z) * dv.z) * inv);
}

// Tile rectangle of a screen-space circle, P0/cr/auxiliary.h:67-77:
// truncation toward zero, clamped to the tile grid.
__device__ __forceinline__ void tile_rect(float px, float py, int radius, int gx, int gy, int& x0, int& y0,
                                          int& x1, int& y1) {
  x0 = min(gx, max(0, (int)((px - radius) / kTile)));
  y0 = min(gy, max(0, (int)((py - radius) / kTile)));
  x1 = min(gx, max(0, (int)((px + radius + kTile - 1) / kTile)));
  y1 = min(gy, max(0, (int)((py + radius + kTile - 1) / kTile)));
}

// A tile rectangle [x0, x1) x [y0, y1) in 8 bytes: (x0 | y0 << 16, x1 | y1 << 16).
__device__ __forceinline__ uint2 pack_rect(int x0, int y0, int x1, int y1) {
  return make_uint2((uint32_t)x0 | ((uint32_t)y0 << 16), (uint32_t)x1 | ((uint32_t)y1 << 16));
}

__device__ __forceinline__ void unpack_rect(uint2 r, int& x0, int& y0, int& x1, int& y1) {
  x0 = (int)(r.x & 0xffffu);
  y0 = (int)(r.x >> 16);
  x1 = (int)(r.y & 0xffffu);
  y1 = (int)(r.y >> 16);
}

// True when packed rectangle r holds tile (tx, ty).
__device__ __forceinline__ bool rect_holds(uint2 r, uint32_t tx, uint32_t ty) {
  return tx - (r.x & 0xffffu) < (r.y & 0xffffu) - (r.x & 0xffffu) && ty - (r.x >> 16) < (r.y >> 16) - (r.x >> 16);
}

// Scene of a surfel / view of a record: binary search over the tables.
__device__ __forceinline__ int find_scene(const sgr_scene_desc* scenes, int n, int surfel) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (scenes[mid].surfel_offset <= surfel) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Device status word (sgr_sizes.off_status).
struct Status {
  unsigned long long num_keys;          // (surfel, tile) pairs, the reference's num_rendered
  unsigned int flags;                   // SGR_FLAG_*
  unsigned int pad;
  unsigned long long num_bin_entries;   // (record, cell) pairs: the entries of the cell lists
  unsigned long long num_fragments;     // (pixel, list entry) pairs the forward blend visits
};

}  // namespace sgr
