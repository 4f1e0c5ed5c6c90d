// Device functions shared by the forward and backward kernels, the views of
// the workspaces the kernels receive, and the launcher declarations.
#pragma once

#include "sgr_common.cuh"
#include "sgr_sort.cuh"

namespace sgr {

constexpr int kMaxShCoeffs = 16;

// Pointers into the geometry workspace and the forward scratch.
struct GeomView {
  float4* records;                       // [R][5]
  int* radii;                            // [R]
  uint32_t* tiles_touched;               // [R]
  unsigned long long* depth_keys;        // [R] (view << 32 | depth bits), forward scratch
  uint32_t* depth_vals;                  // [R] record ids, forward scratch
  unsigned long long* depth_keys_sorted; // [R] forward scratch
  uint32_t* depth_order;                 // [R] record ids in (view, depth, id) order
  unsigned long long* offsets;           // [R] inclusive scan of tiles_touched in that order
  uint2* ranges;                         // [V*tiles] [start, end) of the written-out tile lists
  uint2* rects;                          // [R] packed tile rectangles in depth order
  uint32_t* bin_start;                   // [V*cells] start of each cell list in `bins`
  uint32_t* bin_count;                   // [V*cells] length of each cell list
  uint2* tile_resume;                    // [V*tiles] (cell-list entries the forward scanned, tile entries found)
  uint32_t* tile_queue;                  // [V*tiles + 1] queue order of the tiles, then the queue head
  const uint32_t* bins;                  // cell lists: depth-order positions
  long long bin_capacity;                // entries `bins` holds
  int cell_tiles;                        // cell edge in tiles
  float* final_T;                        // [V][3][H][W]
  uint32_t* n_contrib;                   // [V][2][H][W]
  Status* status;
  int tiles_x, tiles_y;
};

// Mapped depth of the part variant, (far d - far near) / ((far - near) d)
// (P1/cr/forward.cu:415), written as kMdP1 - kDmdP1f / d so that the blends
// need only a reciprocal of the depth.  The reference evaluates it in double
// (its macros are double); here it is fp32 with the constants rounded once.
// It feeds only the distortion and depth terms, never a decision, and
// differs from the double result by a few fp32 ulps of its constant term.
// (A double division per fragment costs more than the rest of the fragment
// on this GPU.)
constexpr float kMdP1 = (float)(kFarP1 / (kFarP1 - kNearP1));
constexpr float kDmdP1f = (float)((kFarP1 * kNearP1) / (kFarP1 - kNearP1));   // d m / d depth = this / depth^2
__device__ __forceinline__ float mapped_depth_p1(float inv_depth) { return kMdP1 - kDmdP1f * inv_depth; }

// View-dependent colour from degree <= 3 SH (P0/cr/forward.cu:20-71).
__device__ __forceinline__ V3 sh_to_rgb(int deg, const float* sh, V3 pos, V3 campos, uint32_t& clamped) {
  V3 dir = pos - campos;
  const float len = sqrtf(dot3(dir, dir));
  dir = v3(dir.x / len, dir.y / len, dir.z / len);
  auto c = [&](int k) { return v3(sh[3 * k], sh[3 * k + 1], sh[3 * k + 2]); };
  V3 res = kShC0 * c(0);
  if (deg > 0) {
    const float x = dir.x, y = dir.y, z = dir.z;
    res = res - kShC1 * y * c(1) + kShC1 * z * c(2) - kShC1 * x * c(3);
    if (deg > 1) {
      const float xx = x * x, yy = y * y, zz = z * z;
      const float xy = x * y, yz = y * z, xz = x * z;
      res = res + kShC2[0] * xy * c(4) + kShC2[1] * yz * c(5) + kShC2[2] * (2.0f * zz - xx - yy) * c(6) +
            kShC2[3] * xz * c(7) + kShC2[4] * (xx - yy) * c(8);
      if (deg > 2) {
        res = res + kShC3[0] * y * (3.0f * xx - yy) * c(9) + kShC3[1] * xy * z * c(10) +
              kShC3[2] * y * (4.0f * zz - xx - yy) * c(11) + kShC3[3] * z * (2.0f * zz - 3.0f * xx - 3.0f * yy) * c(12) +
              kShC3[4] * x * (4.0f * zz - xx - yy) * c(13) + kShC3[5] * z * (xx - yy) * c(14) +
              kShC3[6] * x * (xx - 3.0f * yy) * c(15);
      }
    }
  }
  res = res + v3(0.5f, 0.5f, 0.5f);
  clamped = (res.x < 0 ? 1u : 0u) | (res.y < 0 ? 2u : 0u) | (res.z < 0 ? 4u : 0u);
  return v3(fmaxf(res.x, 0.0f), fmaxf(res.y, 0.0f), fmaxf(res.z, 0.0f));
}

// Reach of one record (see sgr_common.cuh): the threshold c and the box of
// pixel centres where rho = min(rho3d, rho2d) <= c is possible.
//  * rho2d <= c is the disk |pixel - centre| <= sqrt(c / 2).
//  * rho3d <= c is the image of the splat-space disk u^2 + v^2 <= c under
//    the homography x = Tu.S / Tw.S (S = (u, v, 1)).  A vertical line x = X
//    pulls back to (Tu - X Tw).S = 0, which is tangent to the circle when
//    (Tu.z - X Tw.z)^2 = c ((Tu.x - X Tw.x)^2 + (Tu.y - X Tw.y)^2); with
//    d = c (Tw.x^2 + Tw.y^2) - Tw.z^2, p = c (Tu.x Tw.x + Tu.y Tw.y) - Tu.z Tw.z
//    and q = c (Tu.x^2 + Tu.y^2) - Tu.z^2 the extreme X are p/d +- sqrt(p^2/d^2 - q/d).
//    The image is a bounded ellipse only when d < 0 (Tw.S keeps its sign on
//    the disk); near that limit (|d| under 1e-3 of its terms) or for a
//    centre far outside any image the reach is treated as unbounded and
//    nothing is skipped.
// Evaluated in single precision in coordinates relative to the integer pixel
// (X0, Y0) under the surfel's centre: Tu' = Tu - X0 Tw keeps p, q and e small,
// so the cancellation in e^2 - q/d is relative to the offset from that pixel
// (errors ~1e-4 px), not to the absolute pixel coordinate.  The box is
// widened by half a pixel plus 1e-4 of its size.
__device__ __forceinline__ void reach_box(V3 Tu, V3 Tv, V3 Tw, float cx, float cy, float opac, float& c_out,
                                          float4& box) {
  const float kBig = 3.0e38f;
  if (!(opac >= 1.0f / 255.0f)) {   // alpha <= opacity < 1/255 everywhere
    c_out = -1.0f;
    box = make_float4(kBig, -kBig, kBig, -kBig);
    return;
  }
  const float c = 2.0f * logf(255.0f * opac) * 1.001f + 0.01f;
  c_out = c;
  const float r2 = sqrtf(0.5f * c) * 1.0001f + 1e-3f;
  float x0 = cx - r2, x1 = cx + r2, y0 = cy - r2, y1 = cy + r2;
  const float sxy = Tw.x * Tw.x + Tw.y * Tw.y;
  const float d = c * sxy - Tw.z * Tw.z;
  const bool bounded = d < -1e-3f * (c * sxy + Tw.z * Tw.z) && fabsf(cx) < 1e6f && fabsf(cy) < 1e6f;
  if (!bounded) {
    box = make_float4(-kBig, kBig, -kBig, kBig);
    return;
  }
  const float inv = 1.0f / d;
  auto extent = [&](V3 T, float O, float& lo, float& hi) {
    const V3 Ts = v3(T.x - O * Tw.x, T.y - O * Tw.y, T.z - O * Tw.z);
    const float p = c * (Ts.x * Tw.x + Ts.y * Tw.y) - Ts.z * Tw.z;
    const float q = c * (Ts.x * Ts.x + Ts.y * Ts.y) - Ts.z * Ts.z;
    const float e = p * inv;
    const float h = sqrtf(fmaxf(0.0f, e * e - q * inv));
    const float m = 1e-4f * (fabsf(e) + h);
    lo = O + (e - h - m);
    hi = O + (e + h + m);
  };
  float ex0, ex1, ey0, ey1;
  extent(Tu, floorf(cx), ex0, ex1);
  extent(Tv, floorf(cy), ey0, ey1);
  x0 = fminf(x0, ex0);
  x1 = fmaxf(x1, ex1);
  y0 = fminf(y0, ey0);
  y1 = fmaxf(y1, ey1);
  box = make_float4(x0 - 0.5f, x1 + 0.5f, y0 - 0.5f, y1 + 0.5f);
}

__device__ __forceinline__ int find_view(const sgr_view_desc* views, int n, int record) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (views[mid].record_offset <= record) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Warp sum of 32 values per lane, transposed: afterwards lane l holds the
// warp total of value l.  31 shuffles instead of 5 per value.
__device__ __forceinline__ float warp_transpose_sum(float (&v)[32], int lane) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    const bool upper = (lane & o) != 0;
#pragma unroll
    for (int k = 0; k < o; ++k) {
      const float send = upper ? v[k] : v[k + o];
      const float keep = upper ? v[k + o] : v[k];
      v[k] = keep + __shfl_xor_sync(0xffffffffu, send, o);
    }
  }
  return v[0];
}

// One halving step of a warp reduction of N values per lane over lane bit
// o: with h = ceil(N / 2), lanes with the bit clear keep values [0, h) and
// lanes with it set keep values [h, N) (renumbered from 0, plus a zero when
// N is odd), each adding its partner's copy.  h shuffles.
template <int N>
__device__ __forceinline__ void fold_half(float (&v)[32], bool upper, int o) {
  constexpr int h = (N + 1) / 2;
#pragma unroll
  for (int k = 0; k < h; ++k) {
    const float a = v[k];
    const float b = (k + h < N) ? v[k + h] : 0.0f;
    const float send = upper ? a : b;
    const float keep = upper ? b : a;
    v[k] = keep + __shfl_xor_sync(0xffffffffu, send, o);
  }
}

// Warp sum of values 0..17 of every lane with uneven halvings (18, 9, 5, 3,
// 2 values: 20 shuffles instead of the 31 of a full transpose).  Afterwards
// 18 lanes each hold one total; `index` is the value a lane holds, -1 for
// the other 14.
__device__ __forceinline__ float warp_sum18(float (&v)[32], int lane, int& index) {
  fold_half<18>(v, (lane & 16) != 0, 16);
  fold_half<9>(v, (lane & 8) != 0, 8);
  fold_half<5>(v, (lane & 4) != 0, 4);
  fold_half<3>(v, (lane & 2) != 0, 2);
  fold_half<2>(v, (lane & 1) != 0, 1);
  // each halving maps a kept slot s to value s + h when the lane bit is set
  int i = lane & 1;
  bool ok = true;
  i += 2 * ((lane >> 1) & 1);
  ok &= i < 3;
  i += 3 * ((lane >> 2) & 1);
  ok &= i < 5;
  i += 5 * ((lane >> 3) & 1);
  ok &= i < 9;
  i += 9 * ((lane >> 4) & 1);
  ok &= i < 18;
  index = ok ? i : -1;
  return v[0];
}

// Warp sum of values 0..15 of every lane by halvings (16, 8, 4, 2 values,
// then lane pairs: 16 shuffles).  Afterwards the even lanes hold the totals,
// lane l that of value (l >> 1) & 15; `index` is -1 in the odd lanes.
__device__ __forceinline__ float warp_sum16(float (&v)[32], int lane, int& index) {
  fold_half<16>(v, (lane & 16) != 0, 16);
  fold_half<8>(v, (lane & 8) != 0, 8);
  fold_half<4>(v, (lane & 4) != 0, 4);
  fold_half<2>(v, (lane & 2) != 0, 2);
  fold_half<1>(v, (lane & 1) != 0, 1);
  index = (lane & 1) ? -1 : (lane >> 1) & 15;
  return v[0];
}

// The same for values 0..7 (8, 4, 2 values, then two pair sums: 9
// shuffles): lane l with l % 4 == 0 holds the total of value l >> 2.
__device__ __forceinline__ float warp_sum8(float (&v)[32], int lane, int& index) {
  fold_half<8>(v, (lane & 16) != 0, 16);
  fold_half<4>(v, (lane & 8) != 0, 8);
  fold_half<2>(v, (lane & 4) != 0, 4);
  fold_half<1>(v, (lane & 2) != 0, 2);
  fold_half<1>(v, (lane & 1) != 0, 1);
  index = (lane & 3) ? -1 : lane >> 2;
  return v[0];
}

void launch_preprocess(const sgr_batch& b, const GeomView& g, cudaStream_t st);
void launch_store_key_count(const GeomView& g, long long R, cudaStream_t st);
// Cell lists (sgr_binning.cu).  binning_supported is false for tile grids
// whose cell difference array does not fit in shared memory.
inline int bin_cells(int g, int B) { return (g + B - 1) / B; }
bool binning_supported(int gx, int gy, int B);
size_t bin_scratch_bytes(long long R, int V, int gx, int gy, int B);
size_t tile_list_scratch_bytes(long long R, int V, int gx, int gy);
void launch_gather_rects(const GeomView& g, long long R, cudaStream_t st);
int launch_binning(const sgr_batch& b, const GeomView& g, void* scratch, cudaStream_t st);
int launch_tile_lists(const sgr_batch& b, const GeomView& g, uint32_t* lists, long long capacity, void* scratch,
                      cudaStream_t st);
void launch_render_fwd(const sgr_batch& b, const GeomView& g, const sgr_fwd_outputs& out, cudaStream_t st);
void launch_mark_visible(int P, const float* means3D, const float* viewmatrix, uint8_t* present, cudaStream_t st);

void launch_render_bwd(const sgr_batch& b, const GeomView& g, const sgr_bwd_inputs& in, float* grads,
                       float* dL_dsemantics, cudaStream_t st);
void launch_preprocess_bwd(const sgr_batch& b, const GeomView& g, const float* grads, const sgr_bwd_outputs& out,
                           cudaStream_t st);

}  // namespace sgr
