// Blend kernels: per-tile front-to-back compositing (forward) and its
// back-to-front adjoint (backward), for both variants.
//
// Both follow the reference's per-pixel recurrences exactly
// (P0/cr/forward.cu:256-441, P1/cr/forward.cu:265-474,
//  P0/cr/backward.cu:143-440, P1/cr/backward.cu:143-470).  What differs is
// where the tile's list comes from and which (surfel, pixel) pairs get
// evaluated.
//
// A CTA owns one 16x16 tile.  Its list is streamed from the depth-ordered
// list of the cell that holds the tile (sgr_binning.cu), 1024 entries at a
// time: the entries whose tile rectangle holds the tile go, in order, into a
// ring of record ids in shared memory; their count gives list positions.
// The forward records how far it scanned; the backward streams the same
// span back to front.  256 ring entries at a time are staged; each entry is
// tested once against the warps' pixel strips (16x2 in the forward, 16x4 in
// the backward): its reach box (sgr_common.cuh) first, then, for the strips
// the box admits, row by row (row_reaches).  Each warp then walks only the
// entries that can reach its strip, in list order.  Entries that cannot
// reach a pixel are ones the reference skips at its alpha test, so outputs,
// contributor counts and median indices are unchanged.  Per pixel, a
// fragment whose splat and filter distances both exceed the reach threshold
// is rejected before the reciprocal and the exponential.  The splat-plane
// coordinates take one reciprocal and two products instead of the
// reference's two divisions (splat_coords), and the exponential and the
// backward's reciprocals are the hardware's approximate ones (splat_exp,
// blend_rcp): a few 1e-7 relative on alpha, far inside the tolerances.
#include <algorithm>
#include <mutex>
#include <type_traits>

#include "sgr_kernels.cuh"

namespace sgr {

namespace {

constexpr int kWarps = kBlock / 32;
// Entries per staged batch of the blends (sgr_batch.stage_entries): the
// default, and the smaller options.
constexpr int kStageDefault = 256, kStageSmall = 128, kStageTiny = 64;
constexpr int kRing = 2048;            // ring of streamed list entries: >= a batch + kChunk, a power of two
static_assert(kRing >= kStageDefault + kChunk && (kRing & (kRing - 1)) == 0, "ring size");
static_assert(kStageDefault <= 256 && kStageTiny <= kStageSmall && kStageSmall <= kStageDefault,
              "staged slots are indexed by uint8_t");

struct Strip {
  float x0, x1;       // pixel-centre x range of the tile
  float y0;           // pixel-centre y of the tile's first row
};

// True when some pixel centre (x, y), x in [xa, xb], may be within reach of
// the record: rho2d <= c (the filter disk, radius sqrt(c / 2)) or
// |p.xy|^2 <= c p.z^2 (the splat disk), the per-pixel test of the blends.
// Along the row, p(x) = k(x) x l with l = y Tw - Tv and k(xa + u) =
// (xa Tw - Tu) + u Tw, so p(u) = B + u A (B = k(xa) x l, A = Tw x l) and
// |p.xy|^2 - c p.z^2 is a quadratic in u.  The expansion around the row's
// first pixel keeps the cancellation of the blends' own k and l.  The test
// is conservative: the threshold is raised by 1% and the interval widened
// by half a pixel each side, far beyond the fp32 differences between this
// form and the per-pixel one (tests/test_strip_culling.py checks it against
// the per-pixel test on every (record, strip) pair of tilted and large
// surfels; on the 500k-surfel scene, 6.6M pairs, none was wrongly
// rejected).  Non-finite coefficients keep the entry.
__device__ __forceinline__ bool row_reaches(const V3& Tu, const V3& Tv, const V3& Tw, float cx, float cy, float c,
                                            float y, float xa, float xb) {
  const float cc = c * 1.01f;
  const float dy = cy - y;
  const float h2 = 0.5f * cc - dy * dy;
  if (h2 >= 0.0f) {
    const float h = sqrtf(h2);
    if (cx + h >= xa - 0.5f && cx - h <= xb + 0.5f) return true;
  }
  const V3 l = y * Tw - Tv;
  const V3 A = cross3(Tw, l);
  const V3 B = cross3(xa * Tw - Tu, l);
  const float a = A.x * A.x + A.y * A.y - cc * (A.z * A.z);
  const float bh = A.x * B.x + A.y * B.y - cc * (A.z * B.z);
  const float e = B.x * B.x + B.y * B.y - cc * (B.z * B.z);
  if (!(isfinite(a) && isfinite(bh) && isfinite(e))) return true;
  const float ua = -0.5f, ub = (xb - xa) + 0.5f;
  if ((a * ua + 2.0f * bh) * ua + e <= 0.0f || (a * ub + 2.0f * bh) * ub + e <= 0.0f) return true;
  if (a > 0.0f) {
    const float us = -bh / a;
    if (us > ua && us < ub && e - bh * (bh / a) <= 0.0f) return true;
  }
  return false;
}

#ifndef SGR_EXACT_STRIPS
#define SGR_EXACT_STRIPS 1
#endif
// SGR_BWD_SPLIT 1 gives the backward one strip bit per pixel row pair of a
// thread, so that a warp skips a pixel whose rows an entry cannot reach.
// Measured slower (blend backward 27.9 -> 33.2 ms on the 500k x 16 view
// scene: the extra branches cost more than the skipped pixels), so it is off.
#ifndef SGR_BWD_SPLIT
#define SGR_BWD_SPLIT 0
#endif

// Splat-plane coordinates s = p.xy / p.z of a fragment.  0: two IEEE
// divisions, the reference's arithmetic.  1: one correctly rounded
// reciprocal and two products (within 1.5 ulp of the quotients).  2: the
// hardware's approximate reciprocal (1 ulp) and two products, within 2 ulp
// of the quotients.  The forward and the backward use the same form, so
// their alpha and tests agree bit for bit; against the reference's fp32
// arithmetic, alpha moves by a few 1e-7 relative, well inside the parity
// tolerances (and the parity tests' margins around the alpha cut-off).
// Measured on the 500k-surfel 16-view 800x600 step: blend forward 11.37 /
// 10.84 / 10.64 ms, backward 27.77 / 26.11 / 24.74 ms for 0 / 1 / 2.
#ifndef SGR_SPLAT_DIV
#define SGR_SPLAT_DIV 2
#endif

// SGR_FAST_EXP 1: the splat weight exp(power) by the hardware's base-2
// exponential (__expf, within 2 + 1.2 |power| ulp: at most 8 ulp, 5e-7
// relative, over the powers that pass the alpha cut-off) instead of expf.
// SGR_FAST_RCP 1: the backward's reciprocals of 1 - alpha (transmittance
// recovery) and of the depth, and the forward's of the depth (distortion
// terms), by the approximate reciprocal (2 ulp) instead of the correctly
// rounded one.  Both
// blends use the same forms, so their decisions agree bit for bit; the
// parity tests (images 1e-5, gradients 1e-4 relative, contributor counts
// exact) pass at the full bench size with both on.  Measured on the
// 500k-surfel 16-view 800x600 step (with SGR_SPLAT_DIV 2): forward 10.61 ->
// 10.16 ms, backward 24.76 -> 22.54 ms with both (the correctly rounded
// reciprocal of 1 - alpha was most of it).
#ifndef SGR_FAST_EXP
#define SGR_FAST_EXP 1
#endif
#ifndef SGR_FAST_RCP
#define SGR_FAST_RCP 1
#endif

__device__ __forceinline__ float splat_exp(float power) {
#if SGR_FAST_EXP
  return __expf(power);
#else
  return expf(power);
#endif
}

__device__ __forceinline__ float blend_rcp(float x) {
#if SGR_FAST_RCP
  return __fdividef(1.0f, x);
#else
  return __frcp_rn(x);
#endif
}

// Sets sx, sy; returns the reciprocal of z it used (0 with divisions).
// (The scalar helpers here serve the one-pixel-per-thread builds,
// SGR_FWD_PACKED / SGR_PART_PACKED 0; the packed default leaves some unused.)
[[maybe_unused]] __device__ __forceinline__ float splat_coords(float x, float y, float z, float& sx, float& sy) {
#if SGR_SPLAT_DIV == 0
  sx = x / z;
  sy = y / z;
  return 0.0f;
#else
#if SGR_SPLAT_DIV == 1
  const float iz = __frcp_rn(z);
#else
  const float iz = __fdividef(1.0f, z);
#endif
  sx = x * iz;
  sy = y * iz;
  return iz;
#endif
}

// The reciprocal of p.z the explicit geometry uses: the approximate one
// (SGR_SPLAT_DIV 2) or the correctly rounded one (0, 1).
__device__ __forceinline__ float splat_rcp(float z) {
#if SGR_SPLAT_DIV == 2
  return __fdividef(1.0f, z);
#else
  return __frcp_rn(z);
#endif
}

// ---------------------------------------------------------------------------
// Fragment geometry in an explicit order of IEEE round-to-nearest
// operations, for one pixel (float) or for a thread's two pixels at once
// (float2: the packed FP32 instructions, __ffma2_rn and friends).  Both forms
// give identical results element by element, so a forward and a backward in
// either form make the same decisions -- the near-plane, power and alpha
// tests -- bit for bit.  The packed blends of both variants use it, and the
// plain variant's one-pixel forms too.
// The operations follow P0/cr/forward.cu:349-378: k = px Tw - Tu,
// l = py Tw - Tv, p = k x l (each component fma(a, b, -(c d))), the filter
// distance 2 (dx^2 + dy^2), s = p.xy / p.z by one approximate reciprocal,
// rho3d = sx^2 + sy^2, depth (sx Tw.x + sy Tw.y) + Tw.z on the 3D branch.
// ---------------------------------------------------------------------------
[[maybe_unused]] __device__ __forceinline__ float lmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float2 lmul(float2 a, float2 b) { return __fmul2_rn(a, b); }
[[maybe_unused]] __device__ __forceinline__ float lfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float2 lfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
[[maybe_unused]] __device__ __forceinline__ float ladd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float2 ladd(float2 a, float2 b) { return __fadd2_rn(a, b); }
// Per-lane select of a pair.
__device__ __forceinline__ float2 sel2(bool a, bool b, float2 x, float2 y) {
  return make_float2(a ? x.x : y.x, b ? x.y : y.y);
}
template <class T> __device__ __forceinline__ T bc(float s);
template <> [[maybe_unused]] __device__ __forceinline__ float bc<float>(float s) { return s; }
template <> __device__ __forceinline__ float2 bc<float2>(float s) { return make_float2(s, s); }

// -k for k = fma(px, w, -u): -k itself for one pixel, fma(px, -w, u) for a
// pair (a packed negation would cost an instruction).
[[maybe_unused]] __device__ __forceinline__ float negk(float, float, float, float k) { return -k; }
__device__ __forceinline__ float2 negk(float2 px, float w, float u, float2) {
  return lfma(px, bc<float2>(-w), bc<float2>(u));
}

template <class T>
struct FragGeom {
  T kx, ky, kz, lx, ly, lz, px, py, pz, dx, dy, rho2d;
};

// Stage 1: the ray-splat intersection and the filter distance.  npx, npy
// are the negated pixel coordinates.
template <class T>
__device__ __forceinline__ void frag_intersect(T pxf, T pyf, T npx, T npy, const float4& r0, const float4& r1,
                                               const float4& r2, FragGeom<T>& f) {
  f.kx = lfma(pxf, bc<T>(r1.z), bc<T>(-r0.x));
  f.ky = lfma(pxf, bc<T>(r1.w), bc<T>(-r0.y));
  f.kz = lfma(pxf, bc<T>(r2.x), bc<T>(-r0.z));
  f.lx = lfma(pyf, bc<T>(r1.z), bc<T>(-r0.w));
  f.ly = lfma(pyf, bc<T>(r1.w), bc<T>(-r1.x));
  f.lz = lfma(pyf, bc<T>(r2.x), bc<T>(-r1.y));
  // -(c d) as (-c) d with -k: a negation for one pixel (free as an operand
  // modifier), the same fma with negated operands for two (rounding is
  // symmetric, so both give exactly -k)
  const T nkx = negk(pxf, r1.z, r0.x, f.kx);
  const T nky = negk(pxf, r1.w, r0.y, f.ky);
  const T nkz = negk(pxf, r2.x, r0.z, f.kz);
  f.px = lfma(f.ky, f.lz, lmul(nkz, f.ly));
  f.py = lfma(f.kz, f.lx, lmul(nkx, f.lz));
  f.pz = lfma(f.kx, f.ly, lmul(nky, f.lx));
  f.dx = ladd(bc<T>(r2.y), npx);
  f.dy = ladd(bc<T>(r2.z), npy);
  f.rho2d = lmul(bc<T>(kFilterInvSquareP0), lfma(f.dx, f.dx, lmul(f.dy, f.dy)));
}

// The reach test's two squared lengths: |p.xy|^2 and reach p.z^2.
template <class T>
__device__ __forceinline__ void frag_reach_terms(const FragGeom<T>& f, float reach, T& pxy2, T& rpz2) {
  pxy2 = lfma(f.px, f.px, lmul(f.py, f.py));
  rpz2 = lmul(bc<T>(reach), lmul(f.pz, f.pz));
}

// The warp patches of a record, each split into SPLIT groups of rows: bit
// w * SPLIT + g is set when group g of warp w's patch (WX x WY pixels; the
// tile holds kTile / WX patches across) may reach the record -- the reach
// box first, then, for each group the box admits, row_reaches on its rows
// inside the box.  With two pixels per thread the groups are the thread's
// pixels.
template <int WX, int WY, int NWARPS, int SPLIT>
__device__ __forceinline__ uint32_t strip_mask_rows(const float4& r0, const float4& r1, const float4& r2,
                                                    float reach, const float4& box, const Strip& s) {
  constexpr int RG = WY / SPLIT;
  constexpr int ACROSS = kTile / WX;
  static_assert(RG * SPLIT == WY && NWARPS * SPLIT <= 8, "strip groups");
  if (box.y < s.x0 || box.x > s.x1) return 0u;
  const V3 Tu = v3(r0.x, r0.y, r0.z), Tv = v3(r0.w, r1.x, r1.y), Tw = v3(r1.z, r1.w, r2.x);
  uint32_t m = 0u;
#pragma unroll
  for (int w = 0; w < NWARPS; ++w) {
    const float xa = s.x0 + (float)((w % ACROSS) * WX), xb = xa + (float)(WX - 1);
    if (ACROSS > 1 && (box.y < xa || box.x > xb)) continue;
#pragma unroll
    for (int gi = 0; gi < SPLIT; ++gi) {
      const float ya = s.y0 + (float)((w / ACROSS) * WY + RG * gi);
      if (!(box.w >= ya && box.z <= ya + (float)(RG - 1))) continue;
      bool any = !SGR_EXACT_STRIPS;
      for (int r = 0; r < RG && !any; ++r) {
        const float y = ya + (float)r;
        if (y < box.z || y > box.w) continue;
        any = row_reaches(Tu, Tv, Tw, r2.y, r2.z, reach, y, xa, xb);
      }
      if (any) m |= 1u << (w * SPLIT + gi);
    }
  }
  return m;
}

// Compacts this warp's surviving slots of a staged batch into `list`, in
// slot order; returns their number.
template <int SPLIT = 1>
__device__ __forceinline__ int warp_survivors(const uint8_t* mask, int n, int warp, int lane, uint8_t* list) {
  int cnt = 0;
#pragma unroll
  for (int k = 0; k < kWarps; ++k) {
    const int j = k * 32 + lane;
    const bool keep = j < n && ((mask[j] >> (warp * SPLIT)) & ((1u << SPLIT) - 1u));
    const unsigned bal = __ballot_sync(0xffffffffu, keep);
    if (keep) list[cnt + __popc(bal & ((1u << lane) - 1u))] = (uint8_t)j;
    cnt += __popc(bal);
  }
  __syncwarp();
  return cnt;
}

// One window [i0, i1) (at most kChunk entries) of a cell list: the entries
// whose tile rectangle holds tile (tx, ty), `found` of them, in list order.
// They are written to the ring from slot `tail` on as record ids: all of
// them in list order, or, when REVERSE, in reverse list order only those
// whose tile-list position is below `top`, given that the window's entries
// end at position `pos_end`.  Returns how many were written (the same value
// in every thread).  Every thread of the CTA calls it; it synchronises the
// CTA.
template <bool REVERSE, int NT>
__device__ int stream_window(const GeomView& g, const uint32_t* __restrict__ list, int i0, int i1, uint32_t tx,
                             uint32_t ty, int pos_end, int top, uint32_t* ring, int tail, int* s_count, int& found) {
  constexpr int RPT = kChunk / NT;                 // entries per thread
  constexpr int NW = NT / 32;
  static_assert(RPT * NW == 32, "one scan lane per (entry slot, warp)");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  bool hit[RPT];
  uint32_t pos[RPT], bal[RPT];
#pragma unroll
  for (int k = 0; k < RPT; ++k) {
    const int i = i0 + k * NT + (int)threadIdx.x;
    pos[k] = i < i1 ? list[i] : 0u;
    hit[k] = i < i1 && rect_holds(g.rects[pos[k]], tx, ty);
    bal[k] = __ballot_sync(0xffffffffu, hit[k]);
  }
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < RPT; ++k) s_count[k * NW + warp] = __popc(bal[k]);
  }
  __syncthreads();
  // exclusive scan over the 32 (slot, warp) groups, which are in list order
  const int own = s_count[lane];
  int incl = own;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  const int m = REVERSE ? max(0, min(total, top - (pos_end - total))) : total;
  const uint32_t below = (1u << lane) - 1u;
#pragma unroll
  for (int k = 0; k < RPT; ++k) {
    const int base = __shfl_sync(0xffffffffu, incl - own, k * NW + warp);
    if (hit[k]) {
      const int rank = base + __popc(bal[k] & below);
      if (rank < m) {
        const int slot = REVERSE ? tail + (m - 1 - rank) : tail + rank;
        ring[slot & (kRing - 1)] = g.depth_order[pos[k]];
      }
    }
  }
  __syncthreads();
  found = total;
  return m;
}

// The cell list of tile (tx, ty) of view v: its start in g.bins and its
// length, clipped to the entries the buffer holds.
__device__ __forceinline__ void cell_list(const GeomView& g, int v, int tx, int ty, const uint32_t*& list, int& len) {
  const int B = g.cell_tiles;
  const int cx = (g.tiles_x + B - 1) / B, cy = (g.tiles_y + B - 1) / B;
  const size_t cell = (size_t)v * cx * cy + (size_t)(ty / B) * cx + (tx / B);
  const long long s = g.bin_start[cell];
  const long long n = g.bin_count[cell];
  list = g.bins + s;
  len = (int)max(0LL, min(n, g.bin_capacity - s));
}

}  // namespace

// ---------------------------------------------------------------------------
// CTA shapes.  A thread owns PX pixels of one column, two rows apart, so a
// warp covers a 16 x (2 PX) strip and a CTA of 256 / PX threads the tile.
// The packed blends (the default, both variants, both directions) use
// PX = 2: per-entry work (shared-memory loads, the loop, the backward's warp
// reduction) is shared by two pixels, whose arithmetic runs as the two lanes
// of FP32x2 instructions.  With packing switched off the forward uses
// PX = 1 (its pixels terminate independently), the plain backward PX = 2,
// and the part backward PX = 1 (SGR_PART_BWD_PX): unpacked, 3 CTAs of 256
// threads beat two pixels per thread at 3 or 4 CTAs of 128 (49.5 ms against
// 56.3 and 50.7 on 500k surfels x 16 views, 8 semantic channels).
// ---------------------------------------------------------------------------
template <int PX_, int WX_ = kTile>
struct BlendShape {
  static constexpr int PX = PX_;                                      // pixels per thread
  static constexpr int NT = kBlock / PX;                              // threads per CTA
  static constexpr int NW = NT / 32;                                  // warps, one patch each
  static constexpr int WX = WX_;                                      // patch width
  static constexpr int LANE_ROWS = 32 / WX;                           // rows one pixel of each lane spans
  static constexpr int WY = LANE_ROWS * PX;                           // patch height
  static constexpr int ACROSS = kTile / WX;                           // patches across the tile
  static constexpr int ROWS = WY;
  static_assert(ACROSS * WX == kTile && (NW / ACROSS) * WY == kTile && NW % ACROSS == 0, "patches tile the tile");
};
#ifndef SGR_PART_BWD_PX
#define SGR_PART_BWD_PX 1
#endif
// SGR_FWD_PACKED 1: the forward gives each thread two pixels of one column
// (a warp covers 16x4), their fragment geometry and accumulation as the two
// lanes of packed FP32 operations (fwd_fragment2); SGR_BWD_PACKED 1 does the
// same for the backward (bwd_update2).
#ifndef SGR_FWD_PACKED
#define SGR_FWD_PACKED 1
#endif
#ifndef SGR_BWD_PACKED
#define SGR_BWD_PACKED 1
#endif
// SGR_PART_PACKED 1: the part variant's blends take the packed form too, its
// semantic sums and gradients per pixel in shared memory; 0 keeps it at one
// pixel per thread.
#ifndef SGR_PART_PACKED
#define SGR_PART_PACKED 1
#endif
template <int VARIANT>
constexpr bool kPackedBlend = VARIANT == SGR_VARIANT_PLAIN || SGR_PART_PACKED;
template <int VARIANT, int WX = kTile>
using FwdShapeT = BlendShape<(SGR_FWD_PACKED && kPackedBlend<VARIANT>) ? 2 : 1, WX>;
template <int VARIANT, int WX = kTile>
using BwdShapeT = BlendShape<(SGR_BWD_PACKED && kPackedBlend<VARIANT>) ? 2 : (VARIANT == SGR_VARIANT_PLAIN) ? 2
                                                                                      : SGR_PART_BWD_PX, WX>;
template <int VARIANT>
constexpr int kSemSlots = (VARIANT == SGR_VARIANT_PART) ? SGR_MAX_SEMANTICS : 1;

// Pixel i of a thread: warp w owns patch (w % ACROSS, w / ACROSS) of WX x WY
// pixels; lane l sits at column l % WX, row l / WX, and its pixel i
// LANE_ROWS * i rows further down.  With WX = 16 a warp covers a 16 x 2 PX
// strip (column lane % 16, row WY w + lane / 16 + 2 i).
template <class Shape>
__device__ __forceinline__ void pixel_of(int tx, int ty, int lane, int warp, int i, int& px, int& py) {
  px = tx * kTile + (warp % Shape::ACROSS) * Shape::WX + (lane % Shape::WX);
  py = ty * kTile + (warp / Shape::ACROSS) * Shape::WY + lane / Shape::WX + Shape::LANE_ROWS * i;
}

// Tiles taken from a device queue by persistent CTAs (order == NULL: one CTA
// per tile, tile = blockIdx.x).  `order` lists the tiles by decreasing
// estimated cost (k_tile_order); `next` is the queue head.
struct TileQueue {
  const uint32_t* order;
  uint32_t* next;
  int count;
};

// ---------------------------------------------------------------------------
// forward
// ---------------------------------------------------------------------------
// Per-pixel state of the forward recurrences (P0/cr/forward.cu:300-330).
template <int VARIANT>
struct FwdPixel {
  float pxf, pyf;
  bool done;
  float T;
  uint32_t last_contributor;
  float C[3], N[3];
  float D, M1, M2, dist, med_depth, med_weight;
  int med_contrib;
  uint32_t stop;   // list position (1-based) of the entry that ended the pixel, 0 while open
};

// One fragment of the forward for one pixel: entry j of the staged batch of
// SB entries, list position contributor - 1 (P0/cr/forward.cu:349-430).
template <int VARIANT, int SB>
__device__ __forceinline__ void fwd_fragment(FwdPixel<VARIANT>& q, const float4 (*s_rec)[SB],
                                             const float4* s_sem4, int j, uint32_t contributor, int S,
                                             float4* sem_acc4) {
  if (q.done) return;
  const float4 r0 = s_rec[0][j], r1 = s_rec[1][j], r2 = s_rec[2][j];
  const V3 Tu = v3(r0.x, r0.y, r0.z), Tv = v3(r0.w, r1.x, r1.y), Tw = v3(r1.z, r1.w, r2.x);
  const float reach = s_rec[3][j].w;
  float sx, sy, rho2d, depth, power, alpha;
  if (VARIANT == SGR_VARIANT_PLAIN) {
    // the explicit sequence the packed backward repeats
    FragGeom<float> f;
    frag_intersect<float>(q.pxf, q.pyf, -q.pxf, -q.pyf, r0, r1, r2, f);
    if (f.pz == 0.0f) return;
    rho2d = f.rho2d;
    float pxy2, rpz2;
    frag_reach_terms(f, reach, pxy2, rpz2);
    if (rho2d > reach && pxy2 > rpz2) return;
    const float iz = splat_rcp(f.pz);
    sx = lmul(f.px, iz);
    sy = lmul(f.py, iz);
    const float rho3d = lfma(sx, sx, lmul(sy, sy));
    const float rho = fminf(rho3d, rho2d);
    depth = (rho3d <= rho2d) ? ladd(lfma(sx, Tw.x, lmul(sy, Tw.y)), Tw.z) : Tw.z;
    if (depth < kNearP0) return;
    power = lmul(-0.5f, rho);
    if (power > 0.0f) return;
    alpha = fminf(0.99f, lmul(r2.w, splat_exp(power)));
  } else {
    const V3 k = v3(-Tu.x + q.pxf * Tw.x, -Tu.y + q.pxf * Tw.y, -Tu.z + q.pxf * Tw.z);
    const V3 l = v3(-Tv.x + q.pyf * Tw.x, -Tv.y + q.pyf * Tw.y, -Tv.z + q.pyf * Tw.z);
    const V3 p = cross3(k, l);
    if (p.z == 0.0f) return;
    const float dx = r2.y - q.pxf, dy = r2.z - q.pyf;
    rho2d = kFilterInvSquareP0 * (dx * dx + dy * dy);
    if (rho2d > reach && p.x * p.x + p.y * p.y > reach * (p.z * p.z)) return;
    splat_coords(p.x, p.y, p.z, sx, sy);
    const float rho3d = sx * sx + sy * sy;
    const float rho = fminf(rho3d, rho2d);
    depth = (rho3d <= rho2d) ? (sx * Tw.x + sy * Tw.y) + Tw.z : Tw.z;
    if (depth < kNearP0) return;
    power = -0.5f * rho;
    if (power > 0.0f) return;
    alpha = fminf(0.99f, r2.w * splat_exp(power));
  }
  if (alpha < 1.0f / 255.0f) return;
  const float test_T = q.T * (1 - alpha);
  if (test_T < 0.0001f) {
    q.done = true;
    q.stop = contributor;
    return;
  }
  const float4 r3 = s_rec[3][j], r4 = s_rec[4][j];
  const float A = 1 - q.T;
  if (VARIANT == SGR_VARIANT_PLAIN) {
    const float w = alpha * q.T;
#if SGR_SPLAT_DIV == 0
    const float m = kFarP0 / (kFarP0 - kNearP0) * (1 - kNearP0 / depth);
#else
    const float m = kFarP0 / (kFarP0 - kNearP0) * (1 - kNearP0 * blend_rcp(depth));
#endif
    q.dist += (m * m * A + q.M2 - 2 * m * q.M1) * w;
    q.D += depth * w;
    q.M1 += m * w;
    q.M2 += m * m * w;
    if (q.T > 0.5f) {
      q.med_depth = depth;
      q.med_contrib = (int)contributor;
    }
    q.N[0] += r3.x * w;
    q.N[1] += r3.y * w;
    q.N[2] += r3.z * w;
    q.C[0] += r4.x * w;
    q.C[1] += r4.y * w;
    q.C[2] += r4.z * w;
  } else {
    const float m = mapped_depth_p1(blend_rcp(depth));
    const float err = m * m * A + q.M2 - 2 * m * q.M1;
    q.dist += err * alpha * q.T;
    if (q.T > 0.5f) {
      q.med_depth = depth;
      q.med_weight = alpha * q.T;
      q.med_contrib = (int)contributor;
    }
    q.N[0] += r3.x * alpha * q.T;
    q.N[1] += r3.y * alpha * q.T;
    q.N[2] += r3.z * alpha * q.T;
    q.D += depth * alpha * q.T;
    q.M1 += m * alpha * q.T;
    q.M2 += m * m * alpha * q.T;
    q.C[0] += r4.x * alpha * q.T;
    q.C[1] += r4.y * alpha * q.T;
    q.C[2] += r4.z * alpha * q.T;
    // four channels at a time; channels past S are zero in the staged values
    for (int g4 = 0; g4 < (S + 3) / 4; ++g4) {
      const float4 x = s_sem4[g4 * SB + j];
      float4 a = sem_acc4[g4 * kBlock];
      a.x += x.x * alpha * q.T;
      a.y += x.y * alpha * q.T;
      a.z += x.z * alpha * q.T;
      a.w += x.w * alpha * q.T;
      sem_acc4[g4 * kBlock] = a;
    }
  }
  q.T = test_T;
  q.last_contributor = contributor;
}

// Per-pixel state of the forward for a thread's two pixels, lane i = pixel i
// (both in one column).
struct FwdPair {
  float pxf;
  float2 pyf, npx, npy;
  bool done[2];
  float2 T;
  uint32_t last_contributor[2];
  float2 C[3], N[3];
  float2 D, M1, M2, dist, med_depth, med_weight;
  int med_contrib[2];
  uint32_t stop[2];
};

// One entry of the list for both pixels of a thread (fwd_fragment's
// recurrences, P0/cr/forward.cu:349-430 and P1/cr/forward.cu:350-440): the
// geometry in the explicit sequence of frag_intersect, so every test decides
// as the backward does; the accumulation as packed operations, zero-weighted
// on a lane whose fragment does not count.  The part variant's semantic sums
// sit in shared memory: pixel i of this thread at sem_acc4[g4 * kBlock + i *
// NT] for channels 4 g4 .. 4 g4 + 3; the staged semantics of entry j at
// s_sem4[g4 * SB + j].
template <int VARIANT, int NT, int SB>
__device__ __forceinline__ void fwd_fragment2(FwdPair& q, const float4 (*s_rec)[SB], int j,
                                              uint32_t contributor, const float4* s_sem4, int S,
                                              float4* sem_acc4) {
  if (q.done[0] && q.done[1]) return;
  const float4 r0 = s_rec[0][j], r1 = s_rec[1][j], r2 = s_rec[2][j];
  const float reach = s_rec[3][j].w;
  FragGeom<float2> f;
  frag_intersect<float2>(make_float2(q.pxf, q.pxf), q.pyf, q.npx, q.npy, r0, r1, r2, f);
  float2 pxy2, rpz2;
  frag_reach_terms(f, reach, pxy2, rpz2);
  bool a0 = !q.done[0] && f.pz.x != 0.0f && !(f.rho2d.x > reach && pxy2.x > rpz2.x);
  bool a1 = !q.done[1] && f.pz.y != 0.0f && !(f.rho2d.y > reach && pxy2.y > rpz2.y);
  if (!a0 && !a1) return;
  const float Twx = r1.z, Twy = r1.w, Twz = r2.x;
  const float2 iz = make_float2(splat_rcp(a0 ? f.pz.x : 1.0f), splat_rcp(a1 ? f.pz.y : 1.0f));
  const float2 sx = lmul(f.px, iz), sy = lmul(f.py, iz);
  const float2 rho3d = lfma(sx, sx, lmul(sy, sy));
  const float2 d3 = ladd(lfma(sx, bc<float2>(Twx), lmul(sy, bc<float2>(Twy))), bc<float2>(Twz));
  const float2 depth = make_float2(rho3d.x <= f.rho2d.x ? d3.x : Twz, rho3d.y <= f.rho2d.y ? d3.y : Twz);
  a0 = a0 && !(depth.x < kNearP0);
  a1 = a1 && !(depth.y < kNearP0);
  const float2 power =
      lmul(bc<float2>(-0.5f), make_float2(fminf(rho3d.x, f.rho2d.x), fminf(rho3d.y, f.rho2d.y)));
  a0 = a0 && !(power.x > 0.0f);
  a1 = a1 && !(power.y > 0.0f);
  const float2 oa = lmul(bc<float2>(r2.w), make_float2(splat_exp(power.x), splat_exp(power.y)));
  const float2 alpha = make_float2(fminf(0.99f, oa.x), fminf(0.99f, oa.y));
  a0 = a0 && !(alpha.x < 1.0f / 255.0f);
  a1 = a1 && !(alpha.y < 1.0f / 255.0f);
  if (!a0 && !a1) return;
  const float2 one = bc<float2>(1.0f), zero = bc<float2>(0.0f);
  const float2 test_T = lmul(q.T, lfma(alpha, bc<float2>(-1.0f), one));     // T (1 - alpha)
  if (a0 && test_T.x < 0.0001f) {
    q.done[0] = true;
    q.stop[0] = contributor;
    a0 = false;
  }
  if (a1 && test_T.y < 0.0001f) {
    q.done[1] = true;
    q.stop[1] = contributor;
    a1 = false;
  }
  if (!a0 && !a1) return;
  const float4 r3 = s_rec[3][j], r4 = s_rec[4][j];
  const float2 w = sel2(a0, a1, lmul(alpha, q.T), zero);
  // a lane that does not accumulate gets a finite depth (its weight is zero)
  const float2 dep = sel2(a0, a1, depth, one);
  const float2 A = lfma(q.T, bc<float2>(-1.0f), one);                        // 1 - T
  const float2 inv_d = make_float2(blend_rcp(dep.x), blend_rcp(dep.y));
  const float2 m = (VARIANT == SGR_VARIANT_PLAIN)
                       ? lmul(bc<float2>(kFarP0 / (kFarP0 - kNearP0)), lfma(bc<float2>(-kNearP0), inv_d, one))
                       : lfma(bc<float2>(-kDmdP1f), inv_d, bc<float2>(kMdP1));   // mapped_depth_p1
  const float2 mm = lmul(m, m);
  // m^2 A + M2 - 2 m M1
  const float2 e = lfma(lmul(bc<float2>(-2.0f), m), q.M1, lfma(mm, A, q.M2));
  q.dist = lfma(e, w, q.dist);
  q.D = lfma(dep, w, q.D);
  q.M1 = lfma(m, w, q.M1);
  q.M2 = lfma(mm, w, q.M2);
  if (a0 && q.T.x > 0.5f) {
    q.med_depth.x = depth.x;
    q.med_weight.x = w.x;
    q.med_contrib[0] = (int)contributor;
  }
  if (a1 && q.T.y > 0.5f) {
    q.med_depth.y = depth.y;
    q.med_weight.y = w.y;
    q.med_contrib[1] = (int)contributor;
  }
  if (VARIANT == SGR_VARIANT_PART) {
    // four channels at a time; channels past S are zero in the staged values
    for (int g4 = 0; g4 < (S + 3) / 4; ++g4) {
      const float4 x = s_sem4[g4 * SB + j];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        if (!(i == 0 ? a0 : a1)) continue;
        const float wi = i == 0 ? w.x : w.y;
        float4& a = sem_acc4[g4 * kBlock + i * NT];
        a = make_float4(__fmaf_rn(x.x, wi, a.x), __fmaf_rn(x.y, wi, a.y), __fmaf_rn(x.z, wi, a.z),
                        __fmaf_rn(x.w, wi, a.w));
      }
    }
  }
  q.N[0] = lfma(bc<float2>(r3.x), w, q.N[0]);
  q.N[1] = lfma(bc<float2>(r3.y), w, q.N[1]);
  q.N[2] = lfma(bc<float2>(r3.z), w, q.N[2]);
  q.C[0] = lfma(bc<float2>(r4.x), w, q.C[0]);
  q.C[1] = lfma(bc<float2>(r4.y), w, q.C[1]);
  q.C[2] = lfma(bc<float2>(r4.z), w, q.C[2]);
  q.T = sel2(a0, a1, test_T, q.T);
  if (a0) q.last_contributor[0] = contributor;
  if (a1) q.last_contributor[1] = contributor;
}

// Resident CTAs per SM the forward is compiled for.  Plain: 5 CTAs of 128
// threads with two pixels each (96 registers, no spill; measured against 6,
// the same time with a small spill, and 8, 43% slower with 128 bytes of
// spill), or 4 of 256 threads with one pixel each (64 registers).  Part: 3
// (80 registers; its semantic sums and gradients live in shared memory).
#ifndef SGR_FWD_MIN_CTAS
#define SGR_FWD_MIN_CTAS (SGR_FWD_PACKED ? 5 : 4)
#endif
#ifndef SGR_PART_FWD_MIN_CTAS
#define SGR_PART_FWD_MIN_CTAS (SGR_FWD_PACKED && SGR_PART_PACKED ? 4 : 3)
#endif

// The forward of one tile (all threads of the CTA).
template <int VARIANT, int WX, int SB>
__device__ __forceinline__ void render_fwd_tile(const sgr_batch& b, const GeomView& g, const sgr_fwd_outputs& out,
                                                const int tile) {
  using Shape = FwdShapeT<VARIANT, WX>;
  constexpr int PX = Shape::PX, NT = Shape::NT, NW = Shape::NW;
  const int tiles_per_view = g.tiles_x * g.tiles_y;
  const int v = tile / tiles_per_view;
  const int t = tile - v * tiles_per_view;
  const int ty = t / g.tiles_x, tx = t - ty * g.tiles_x;
  const int W = b.width, H = b.height;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const float off = (VARIANT == SGR_VARIANT_PLAIN) ? 0.0f : 0.5f;
  const Strip strip{(float)(tx * kTile) + off, (float)(tx * kTile) + off + (kTile - 1), (float)(ty * kTile) + off};
  const int S = (VARIANT == SGR_VARIANT_PART) ? b.semantic_channels : 0;
  const sgr_view_desc vd = b.views[v];
  const int sid_base = b.scenes[vd.scene].surfel_offset - vd.record_offset;

  __shared__ float4 s_rec[kRecF4 - 1][SB];
  __shared__ uint8_t s_mask[SB];
  __shared__ uint8_t s_list[NW][SB];
  __shared__ uint32_t s_ring[kRing];
  __shared__ int s_count[32];
  // part variant, sized by S at launch (fwd_dynamic_bytes): the staged
  // semantics, four channels per float4 (rows of SB float4), then every
  // pixel's semantic sums (rows of kBlock float4, pixel i of a thread in
  // column i * NT + thread)
  extern __shared__ float4 s_dyn4[];
  static_assert(NT * PX == kBlock, "one column per pixel");
  const int NS4 = (S + 3) / 4;
  float4* const s_sem4 = s_dyn4;
  float4* const sem_acc4 = (VARIANT == SGR_VARIANT_PART) ? s_dyn4 + NS4 * SB + threadIdx.x : nullptr;

  const uint32_t* list;
  int len;
  cell_list(g, v, tx, ty, list, len);
  int head = 0, tail = 0, scanned = 0, base = 0;

  FwdPixel<VARIANT> q[PX];
  bool done = true;                                // every pixel of this thread
#pragma unroll
  for (int i = 0; i < PX; ++i) {
    int px, py;
    pixel_of<Shape>(tx, ty, lane, warp, i, px, py);
    FwdPixel<VARIANT>& Q = q[i];
    Q.pxf = (float)px + off;
    Q.pyf = (float)py + off;
    Q.done = !(px < W && py < H);
    Q.T = 1.0f;
    Q.last_contributor = 0;
#pragma unroll
    for (int c = 0; c < 3; ++c) Q.C[c] = Q.N[c] = 0.f;
    Q.D = Q.M1 = Q.M2 = Q.dist = Q.med_depth = Q.med_weight = 0.f;
    Q.med_contrib = -1;
    Q.stop = 0;
    if (VARIANT == SGR_VARIANT_PART)
      for (int g4 = 0; g4 < NS4; ++g4) sem_acc4[g4 * kBlock + i * NT] = make_float4(0.f, 0.f, 0.f, 0.f);
    done = done && Q.done;
  }

  // the two pixels of a thread as packed lanes
  constexpr bool PACKED = PX == 2;
  FwdPair qp;
  if constexpr (PACKED) {
    qp.pxf = q[0].pxf;
    qp.pyf = make_float2(q[0].pyf, q[1].pyf);
    qp.npx = make_float2(-q[0].pxf, -q[1].pxf);
    qp.npy = make_float2(-q[0].pyf, -q[1].pyf);
    qp.T = make_float2(1.0f, 1.0f);
    const float2 z = make_float2(0.0f, 0.0f);
    qp.C[0] = qp.C[1] = qp.C[2] = qp.N[0] = qp.N[1] = qp.N[2] = z;
    qp.D = qp.M1 = qp.M2 = qp.dist = qp.med_depth = qp.med_weight = z;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      qp.done[i] = q[i].done;
      qp.last_contributor[i] = 0;
      qp.med_contrib[i] = -1;
      qp.stop[i] = 0;
    }
  }

  for (;; base += SB, head += SB) {
    if (__syncthreads_count(done) == NT) break;
    while (tail - head < SB && scanned < len) {   // refill the ring (CTA-uniform)
      int found;
      tail += stream_window<false, NT>(g, list, scanned, min(scanned + kChunk, len), (uint32_t)tx, (uint32_t)ty, 0,
                                       0, s_ring, tail, s_count, found);
      scanned = min(scanned + kChunk, len);
    }
    const int n = min(SB, tail - head);
    if (n <= 0) break;
    for (int e = threadIdx.x; e < n; e += NT) {
      const uint32_t r = s_ring[(head + e) & (kRing - 1)];
      const float4* rec = g.records + (size_t)r * kRecF4;
#pragma unroll
      for (int k = 0; k < kRecF4 - 1; ++k) s_rec[k][e] = rec[k];
      {
        const float4 a0 = s_rec[0][e], a1 = s_rec[1][e], a2 = s_rec[2][e];
        s_mask[e] = (uint8_t)strip_mask_rows<Shape::WX, Shape::WY, NW, 1>(a0, a1, a2, s_rec[3][e].w, rec[5], strip);
      }
      if (VARIANT == SGR_VARIANT_PART) {
        const float* sem = b.semantics + (size_t)(sid_base + (int)r) * S;
        for (int g4 = 0; g4 < (S + 3) / 4; ++g4) {
          const int c = 4 * g4;
          s_sem4[g4 * SB + e] = make_float4(sem[c], c + 1 < S ? sem[c + 1] : 0.f, c + 2 < S ? sem[c + 2] : 0.f,
                                                c + 3 < S ? sem[c + 3] : 0.f);
        }
      }
    }
    __syncthreads();
    const int cnt = warp_survivors(s_mask, n, warp, lane, s_list[warp]);
    for (int si = 0; !done && si < cnt; ++si) {
      const int j = s_list[warp][si];
      const uint32_t contributor = (uint32_t)(base + j + 1);
      if constexpr (PACKED) {
        fwd_fragment2<VARIANT, NT>(qp, s_rec, j, contributor, s_sem4, S, sem_acc4);
        done = qp.done[0] && qp.done[1];
      } else {
        done = true;
#pragma unroll
        for (int i = 0; i < PX; ++i) {
          fwd_fragment<VARIANT>(q[i], s_rec, s_sem4, j, contributor, S, sem_acc4);
          done = done && q[i].done;
        }
      }
    }
  }
  if constexpr (PACKED) {   // back to the per-pixel state the outputs are written from
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      FwdPixel<VARIANT>& Q = q[i];
      auto lane_of = [i](float2 x) { return i == 0 ? x.x : x.y; };
      Q.done = qp.done[i];
      Q.T = lane_of(qp.T);
      Q.last_contributor = qp.last_contributor[i];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        Q.C[c] = lane_of(qp.C[c]);
        Q.N[c] = lane_of(qp.N[c]);
      }
      Q.D = lane_of(qp.D);
      Q.M1 = lane_of(qp.M1);
      Q.M2 = lane_of(qp.M2);
      Q.dist = lane_of(qp.dist);
      Q.med_depth = lane_of(qp.med_depth);
      Q.med_weight = lane_of(qp.med_weight);
      Q.med_contrib = qp.med_contrib[i];
      Q.stop = qp.stop[i];
    }
  }

  if (threadIdx.x == 0) g.tile_resume[tile] = make_uint2((uint32_t)scanned, (uint32_t)tail);
  {
    // fragments the reference's blend visits here: per pixel, the list
    // entries up to the one that ended it, or the whole list
    unsigned long long visited = 0;
#pragma unroll
    for (int i = 0; i < PX; ++i) {
      int px, py;
      pixel_of<Shape>(tx, ty, lane, warp, i, px, py);
      if (px < W && py < H) visited += q[i].stop ? q[i].stop : (uint32_t)tail;
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) visited += __shfl_xor_sync(0xffffffffu, visited, o);
    if (lane == 0 && visited) atomicAdd(&g.status->num_fragments, visited);
  }
  const size_t HW = (size_t)H * W;
  const float* bg = b.background;
  const int NO = (VARIANT == SGR_VARIANT_PLAIN) ? 7 : 8;
#pragma unroll
  for (int i = 0; i < PX; ++i) {
    int px, py;
    pixel_of<Shape>(tx, ty, lane, warp, i, px, py);
    if (!(px < W && py < H)) continue;
    const FwdPixel<VARIANT>& Q = q[i];
    const size_t pix = (size_t)py * W + px;
    float* fT = g.final_T + (size_t)v * 3 * HW;
    uint32_t* nc = g.n_contrib + (size_t)v * 2 * HW;
    fT[pix] = Q.T;
    fT[pix + HW] = Q.M1;
    fT[pix + 2 * HW] = Q.M2;
    nc[pix] = Q.last_contributor;
    nc[pix + HW] = Q.med_contrib > 0 ? (uint32_t)Q.med_contrib : 0u;
    float* col = out.color + (size_t)v * 3 * HW;
    col[pix] = Q.C[0] + Q.T * bg[0];
    col[pix + HW] = Q.C[1] + Q.T * bg[1];
    col[pix + 2 * HW] = Q.C[2] + Q.T * bg[2];
    float* oth = out.others + (size_t)v * NO * HW;
    oth[pix] = Q.D;
    oth[pix + HW] = 1 - Q.T;
    oth[pix + 2 * HW] = Q.N[0];
    oth[pix + 3 * HW] = Q.N[1];
    oth[pix + 4 * HW] = Q.N[2];
    oth[pix + 5 * HW] = Q.med_depth;
    oth[pix + 6 * HW] = Q.dist;
    if (VARIANT == SGR_VARIANT_PART) {
      oth[pix + 7 * HW] = Q.med_weight;
      float* sem = out.semantic + (size_t)v * S * HW;
      const float* acc = reinterpret_cast<const float*>(sem_acc4 + i * NT);   // pixel column: float4 stride kBlock
      for (int c = 0; c < S; ++c) sem[pix + c * HW] = acc[(c >> 2) * 4 * kBlock + (c & 3)];
    }
  }
}

// One CTA per tile, or persistent CTAs taking tiles from a queue; SB list
// entries per staged batch.
template <int VARIANT, int WX, int SB>
__global__ void __launch_bounds__(FwdShapeT<VARIANT, WX>::NT,
                                  (VARIANT == SGR_VARIANT_PLAIN) ? SGR_FWD_MIN_CTAS : SGR_PART_FWD_MIN_CTAS)
    k_render_fwd(const sgr_batch b, GeomView g, sgr_fwd_outputs out, TileQueue q) {
  __shared__ int s_item;
  for (int it = 0;; ++it) {
    int tile;
    if (q.order) {
      __syncthreads();                             // the previous tile is done with shared memory
      if (threadIdx.x == 0) s_item = (int)atomicAdd(q.next, 1u);
      __syncthreads();
      if (s_item >= q.count) return;
      tile = (int)q.order[s_item];
    } else {
      if (it > 0) return;
      tile = blockIdx.x;
    }
    render_fwd_tile<VARIANT, WX, SB>(b, g, out, tile);
  }
}

// ---------------------------------------------------------------------------
// backward
//
// Back to front over the positions before each pixel's last contributor,
// transmittance recovered by division from the stored final T.  The CTA
// starts at its tile's largest last contributor; each warp skips entries at
// or past its own largest one.
//
// Plain variant: each thread owns two pixels of one column, two rows apart,
// so a warp covers a 16x4 strip and a CTA of 128 threads the tile.  The part
// variant keeps one pixel per thread (its 48 floats of per-pixel semantic
// state would not fit twice).  The 18 per-fragment gradients of a warp's
// pixels are summed in registers over the thread's pixels, then over the
// warp with a transposed shuffle reduction, and one lane per value adds the
// total to the per-view gradient record (one atomic per value and warp
// instead of one per value and pixel).
// ---------------------------------------------------------------------------
static_assert(kGradUsed == 18, "warp_sum18 reduces the 18 gradient values of a fragment");

// SGR_BWD_DOT_REC 1: the backward's colour and normal recurrences
// (accum_rec, accum_normal: P0/cr/backward.cu:365-395) run on their dot
// products with dL/dpixel and dL/dnormal instead of per channel.  The
// recurrences are linear, so the alpha gradient is the same sum; it saves
// four channels' worth of registers and instructions per pixel.
#ifndef SGR_BWD_DOT_REC
#define SGR_BWD_DOT_REC 1
#endif

// Per-pixel state of the backward recurrences (P0/cr/backward.cu:160-260).
template <int VARIANT>
struct BwdPixel {
  static constexpr int NS = kSemSlots<VARIANT>;
  float pxf, pyf;
  float T, T_final, final_A, final_D, final_D2, bg_dot;
  int last_contributor, median_contributor;
  float dL_dpixel[3], dL_dnormal2D[3];
  float dL_ddepth, dL_daccum, dL_dreg, dL_dmedian, dL_dmaxw;
#if SGR_BWD_DOT_REC
  // the colour and normal recurrences kept as their dot products with the
  // pixel's upstream gradient, the only way the alpha gradient uses them
  float rec_dot, last_col_dot, nrm_dot, last_nrm_dot;
#else
  float accum_rec[3], last_color[3], last_normal[3], accum_normal[3];
#endif
  float last_alpha, last_depth, accum_depth, accum_alpha, last_dL_dT;
  float sem_w;   // part variant: alpha T of the pixel's fragment of the current entry
};

// Geometry of one backward fragment (P0/cr/backward.cu:290-330): the
// ray-splat intersection, alpha and the tests, computed without branches so
// that the two pixels of a thread interleave.  `live` is false when the
// fragment contributes nothing.
struct BwdGeom {
  V3 k, l, p;
  float sx, sy, iz, dx, dy, G, alpha, c_d;
  bool use3d, live;
};

// Stage 1: the reach test; true when the fragment may contribute.
template <int VARIANT>
__device__ __forceinline__ bool bwd_reach(const BwdPixel<VARIANT>& q, const float4& r0, const float4& r1,
                                          const float4& r2, float reach, int pos, BwdGeom& f) {
  if (VARIANT == SGR_VARIANT_PLAIN) {   // the forward's explicit sequence
    FragGeom<float> g;
    frag_intersect<float>(q.pxf, q.pyf, -q.pxf, -q.pyf, r0, r1, r2, g);
    f.k = v3(g.kx, g.ky, g.kz);
    f.l = v3(g.lx, g.ly, g.lz);
    f.p = v3(g.px, g.py, g.pz);
    f.dx = g.dx;
    f.dy = g.dy;
    float pxy2, rpz2;
    frag_reach_terms(g, reach, pxy2, rpz2);
    f.live = pos < q.last_contributor && g.pz != 0.0f && !(g.rho2d > reach && pxy2 > rpz2);
    return f.live;
  }
  const V3 Tu = v3(r0.x, r0.y, r0.z), Tv = v3(r0.w, r1.x, r1.y), Tw = v3(r1.z, r1.w, r2.x);
  f.k = v3(-Tu.x + q.pxf * Tw.x, -Tu.y + q.pxf * Tw.y, -Tu.z + q.pxf * Tw.z);
  f.l = v3(-Tv.x + q.pyf * Tw.x, -Tv.y + q.pyf * Tw.y, -Tv.z + q.pyf * Tw.z);
  f.p = cross3(f.k, f.l);
  f.dx = r2.y - q.pxf;
  f.dy = r2.z - q.pyf;
  const float rho2d = kFilterInvSquareP0 * (f.dx * f.dx + f.dy * f.dy);
  f.live = pos < q.last_contributor && f.p.z != 0.0f &&
           !(rho2d > reach && f.p.x * f.p.x + f.p.y * f.p.y > reach * (f.p.z * f.p.z));
  return f.live;
}

// Stage 2: alpha and the remaining tests, with the forward's divisions so
// that alpha and the tests agree with it bit for bit.
template <int VARIANT>
__device__ __forceinline__ void bwd_alpha(const float4& r1, const float4& r2, BwdGeom& f) {
  const float Twx = r1.z, Twy = r1.w, Twz = r2.x;
  const float pz = f.live ? f.p.z : 1.0f;
  if (VARIANT == SGR_VARIANT_PLAIN) {   // the forward's explicit sequence
    f.iz = splat_rcp(pz);
    f.sx = lmul(f.p.x, f.iz);
    f.sy = lmul(f.p.y, f.iz);
    const float rho3d = lfma(f.sx, f.sx, lmul(f.sy, f.sy));
    const float rho2d = lmul(kFilterInvSquareP0, lfma(f.dx, f.dx, lmul(f.dy, f.dy)));
    f.use3d = rho3d <= rho2d;
    const float rho = fminf(rho3d, rho2d);
    f.c_d = f.use3d ? ladd(lfma(f.sx, Twx, lmul(f.sy, Twy)), Twz) : Twz;
    const float power = lmul(-0.5f, rho);
    f.G = splat_exp(power);
    f.alpha = fminf(0.99f, lmul(r2.w, f.G));
    f.live = f.live && !(f.c_d < kNearP0) && !(power > 0.0f) && !(f.alpha < 1.0f / 255.0f);
    return;
  }
  f.iz = splat_coords(f.p.x, f.p.y, pz, f.sx, f.sy);
  const float rho3d = f.sx * f.sx + f.sy * f.sy;
  const float rho2d = kFilterInvSquareP0 * (f.dx * f.dx + f.dy * f.dy);
  f.use3d = rho3d <= rho2d;
  const float rho = fminf(rho3d, rho2d);
  f.c_d = f.use3d ? (f.sx * Twx + f.sy * Twy) + Twz : Twz;
  const float power = -0.5f * rho;
  f.G = splat_exp(power);
  f.alpha = fminf(0.99f, r2.w * f.G);
  f.live = f.live && !(f.c_d < kNearP0) && !(power > 0.0f) && !(f.alpha < 1.0f / 255.0f);
}

// Stage 3: the pixel's recurrences and its share of the entry's 18 gradient
// values (gv), for a live fragment; the part variant also keeps the
// fragment's weight for its semantic gradients.
template <int VARIANT>
__device__ __forceinline__ void bwd_update(BwdPixel<VARIANT>& q, const BwdGeom& f, const float4& r1, const float4& r2,
                                           const float4& r3, const float4& r4, int pos, float (&gv)[32]) {
  const float Twx = r1.z, Twy = r1.w;
  const float alpha = f.alpha, G = f.G, c_d = f.c_d;
  const float inv_1ma = blend_rcp(1.f - alpha);
  q.T = q.T * inv_1ma;
  const float wgt = alpha * q.T;
  float dL_dalpha = 0.0f;
  const float col[3] = {r4.x, r4.y, r4.z};
#if SGR_BWD_DOT_REC
  {
    const float cd = col[0] * q.dL_dpixel[0] + col[1] * q.dL_dpixel[1] + col[2] * q.dL_dpixel[2];
    q.rec_dot = q.last_alpha * q.last_col_dot + (1.f - q.last_alpha) * q.rec_dot;
    q.last_col_dot = cd;
    dL_dalpha += cd - q.rec_dot;
  }
#pragma unroll
  for (int ch = 0; ch < 3; ++ch) gv[14 + ch] += wgt * q.dL_dpixel[ch];
#else
#pragma unroll
  for (int ch = 0; ch < 3; ++ch) {
    q.accum_rec[ch] = q.last_alpha * q.last_color[ch] + (1.f - q.last_alpha) * q.accum_rec[ch];
    q.last_color[ch] = col[ch];
    dL_dalpha += (col[ch] - q.accum_rec[ch]) * q.dL_dpixel[ch];
    gv[14 + ch] += wgt * q.dL_dpixel[ch];
  }
#endif
  // The reference's semantic recurrence (accumulated and last semantics,
  // P1/cr/backward.cu:358-368) feeds only an alpha-gradient term that it
  // leaves commented out (:365), so it is not computed here.
  float dL_dz = 0.0f, dL_dweight = 0.f;
  float m_d, dmd_dd;
  if (VARIANT == SGR_VARIANT_PLAIN) {
    const float inv_d = blend_rcp(c_d);
    m_d = kFarP0 / (kFarP0 - kNearP0) * (1 - kNearP0 * inv_d);
    dmd_dd = (kFarP0 * kNearP0) / (kFarP0 - kNearP0) * (inv_d * inv_d);
  } else {
    const float inv_d = blend_rcp(c_d);
    m_d = mapped_depth_p1(inv_d);
    dmd_dd = kDmdP1f * (inv_d * inv_d);
  }
  if (pos == q.median_contributor - 1) {
    dL_dz += q.dL_dmedian;
    if (VARIANT == SGR_VARIANT_PART) dL_dweight += q.dL_dmaxw;
  }
  dL_dweight += (q.final_D2 + m_d * m_d * q.final_A - 2 * m_d * q.final_D) * q.dL_dreg;
  dL_dalpha += dL_dweight - q.last_dL_dT;
  q.last_dL_dT = dL_dweight * alpha + (1 - alpha) * q.last_dL_dT;
  const float dL_dmd = 2.0f * (q.T * alpha) * (m_d * q.final_A - q.final_D) * q.dL_dreg;
  dL_dz += dL_dmd * dmd_dd;
  q.accum_depth = q.last_alpha * q.last_depth + (1.f - q.last_alpha) * q.accum_depth;
  q.last_depth = c_d;
  dL_dalpha += (c_d - q.accum_depth) * q.dL_ddepth;
  // the reference adds last_alpha * 1.0 in double: one rounding of an exact
  // sum, i.e. a plain float add
  q.accum_alpha = __fadd_rn(q.last_alpha, __fmul_rn(1.f - q.last_alpha, q.accum_alpha));
  dL_dalpha += (1 - q.accum_alpha) * q.dL_daccum;
  const float nrm[3] = {r3.x, r3.y, r3.z};
#if SGR_BWD_DOT_REC
  {
    const float nd = nrm[0] * q.dL_dnormal2D[0] + nrm[1] * q.dL_dnormal2D[1] + nrm[2] * q.dL_dnormal2D[2];
    q.nrm_dot = q.last_alpha * q.last_nrm_dot + (1.f - q.last_alpha) * q.nrm_dot;
    q.last_nrm_dot = nd;
    dL_dalpha += nd - q.nrm_dot;
  }
#pragma unroll
  for (int ch = 0; ch < 3; ++ch) gv[11 + ch] += alpha * q.T * q.dL_dnormal2D[ch];
#else
#pragma unroll
  for (int ch = 0; ch < 3; ++ch) {
    q.accum_normal[ch] = q.last_alpha * q.last_normal[ch] + (1.f - q.last_alpha) * q.accum_normal[ch];
    q.last_normal[ch] = nrm[ch];
    dL_dalpha += (nrm[ch] - q.accum_normal[ch]) * q.dL_dnormal2D[ch];
    gv[11 + ch] += alpha * q.T * q.dL_dnormal2D[ch];
  }
#endif
  dL_dalpha *= q.T;
  q.last_alpha = alpha;
  dL_dalpha += (-q.T_final * inv_1ma) * q.bg_dot;
  const float dL_dG = r2.w * dL_dalpha;
  dL_dz += alpha * q.T * q.dL_ddepth;
  if (f.use3d) {
    const float inv_pz = SGR_SPLAT_DIV == 0 ? __frcp_rn(f.p.z) : f.iz;
    const float dsx_pz = (dL_dG * -G * f.sx + dL_dz * Twx) * inv_pz;
    const float dsy_pz = (dL_dG * -G * f.sy + dL_dz * Twy) * inv_pz;
    const V3 dL_dp = v3(dsx_pz, dsy_pz, -(dsx_pz * f.sx + dsy_pz * f.sy));
    const V3 dL_dk = cross3(f.l, dL_dp);
    const V3 dL_dl = cross3(dL_dp, f.k);
    gv[0] -= dL_dk.x; gv[1] -= dL_dk.y; gv[2] -= dL_dk.z;
    gv[3] -= dL_dl.x; gv[4] -= dL_dl.y; gv[5] -= dL_dl.z;
    gv[6] += q.pxf * dL_dk.x + q.pyf * dL_dl.x + dL_dz * f.sx;
    gv[7] += q.pxf * dL_dk.y + q.pyf * dL_dl.y + dL_dz * f.sy;
    gv[8] += q.pxf * dL_dk.z + q.pyf * dL_dl.z + dL_dz * 1.0f;
  } else {
    gv[9] += dL_dG * (-G * kFilterInvSquareP0 * f.dx);
    gv[10] += dL_dG * (-G * kFilterInvSquareP0 * f.dy);
    gv[8] += dL_dz;
  }
  gv[17] += G * dL_dalpha;
  if (VARIANT == SGR_VARIANT_PART) q.sem_w = wgt;   // dL/dsemantic[c] += wgt dL/dpixel_semantic[c]
}

// ---------------------------------------------------------------------------
// The backward's two pixels per thread as the two lanes of packed FP32
// operations (SGR_BWD_PACKED): the same recurrences as bwd_reach, bwd_alpha
// and bwd_update, with the fragment geometry in the forward's explicit
// sequence (frag_intersect), so the decisions -- which fragments count -- are
// the forward's bit for bit.  A pixel that a fragment does not reach keeps
// its state and adds nothing.
// ---------------------------------------------------------------------------


// Per-pixel state of the backward recurrences, lane i = pixel i.
struct BwdPair {
  float pxf;                                 // both pixels share the column
  float2 pyf, npx, npy;
  float2 T, T_final, final_A, final_D, final_D2, bg_dot;
  int last_contributor[2], median_contributor[2];
  float2 dL_dpixel[3], dL_dnormal2D[3];
  float2 dL_ddepth, dL_daccum, dL_dreg, dL_dmedian, dL_dmaxw;
  float2 rec_dot, last_col_dot, nrm_dot, last_nrm_dot;
  float2 last_alpha, last_depth, accum_depth, accum_alpha, last_dL_dT;
  float2 sem_w;   // part variant: alpha T of each pixel's fragment of the current entry, 0 where not live
};

template <int VARIANT>
__device__ __forceinline__ BwdPair to_pair(const BwdPixel<VARIANT> (&q)[2]) {
  BwdPair p;
  auto f2 = [](float a, float b) { return make_float2(a, b); };
  p.pxf = q[0].pxf;
  p.pyf = f2(q[0].pyf, q[1].pyf);
  p.npx = f2(-q[0].pxf, -q[1].pxf);
  p.npy = f2(-q[0].pyf, -q[1].pyf);
  p.T = f2(q[0].T, q[1].T);
  p.T_final = f2(q[0].T_final, q[1].T_final);
  p.final_A = f2(q[0].final_A, q[1].final_A);
  p.final_D = f2(q[0].final_D, q[1].final_D);
  p.final_D2 = f2(q[0].final_D2, q[1].final_D2);
  p.bg_dot = f2(q[0].bg_dot, q[1].bg_dot);
  for (int i = 0; i < 2; ++i) {
    p.last_contributor[i] = q[i].last_contributor;
    p.median_contributor[i] = q[i].median_contributor;
  }
  for (int c = 0; c < 3; ++c) {
    p.dL_dpixel[c] = f2(q[0].dL_dpixel[c], q[1].dL_dpixel[c]);
    p.dL_dnormal2D[c] = f2(q[0].dL_dnormal2D[c], q[1].dL_dnormal2D[c]);
  }
  p.dL_ddepth = f2(q[0].dL_ddepth, q[1].dL_ddepth);
  p.dL_daccum = f2(q[0].dL_daccum, q[1].dL_daccum);
  p.dL_dreg = f2(q[0].dL_dreg, q[1].dL_dreg);
  p.dL_dmedian = f2(q[0].dL_dmedian, q[1].dL_dmedian);
  p.dL_dmaxw = f2(q[0].dL_dmaxw, q[1].dL_dmaxw);
  const float2 z = f2(0.f, 0.f);
  p.sem_w = z;
  p.rec_dot = p.last_col_dot = p.nrm_dot = p.last_nrm_dot = z;
  p.last_alpha = p.last_depth = p.accum_depth = p.accum_alpha = p.last_dL_dT = z;
  return p;
}

// Geometry of the two fragments of one entry (stages 1 and 2 of the
// backward); live[i] is false when pixel i's fragment contributes nothing.
struct BwdGeom2 {
  FragGeom<float2> g;
  float2 sx, sy, iz, G, alpha, c_d;
  bool use3d[2], live[2];
};

// Stage 1: the reach test of both pixels.
__device__ __forceinline__ bool bwd_reach2(const BwdPair& q, const float4& r0, const float4& r1, const float4& r2,
                                           float reach, int pos, BwdGeom2& f) {
  frag_intersect<float2>(make_float2(q.pxf, q.pxf), q.pyf, q.npx, q.npy, r0, r1, r2, f.g);
  float2 pxy2, rpz2;
  frag_reach_terms(f.g, reach, pxy2, rpz2);
  f.live[0] = pos < q.last_contributor[0] && f.g.pz.x != 0.0f && !(f.g.rho2d.x > reach && pxy2.x > rpz2.x);
  f.live[1] = pos < q.last_contributor[1] && f.g.pz.y != 0.0f && !(f.g.rho2d.y > reach && pxy2.y > rpz2.y);
  return f.live[0] || f.live[1];
}

// Stage 2: alpha and the remaining tests, as the forward computes them.
__device__ __forceinline__ void bwd_alpha2(const float4& r1, const float4& r2, BwdGeom2& f) {
  const float Twx = r1.z, Twy = r1.w, Twz = r2.x;
  f.iz = make_float2(splat_rcp(f.live[0] ? f.g.pz.x : 1.0f), splat_rcp(f.live[1] ? f.g.pz.y : 1.0f));
  f.sx = lmul(f.g.px, f.iz);
  f.sy = lmul(f.g.py, f.iz);
  const float2 rho3d = lfma(f.sx, f.sx, lmul(f.sy, f.sy));
  f.use3d[0] = rho3d.x <= f.g.rho2d.x;
  f.use3d[1] = rho3d.y <= f.g.rho2d.y;
  const float2 rho = make_float2(fminf(rho3d.x, f.g.rho2d.x), fminf(rho3d.y, f.g.rho2d.y));
  const float2 d3 = ladd(lfma(f.sx, bc<float2>(Twx), lmul(f.sy, bc<float2>(Twy))), bc<float2>(Twz));
  f.c_d = make_float2(f.use3d[0] ? d3.x : Twz, f.use3d[1] ? d3.y : Twz);
  const float2 power = lmul(bc<float2>(-0.5f), rho);
  f.G = make_float2(splat_exp(power.x), splat_exp(power.y));
  const float2 oa = lmul(bc<float2>(r2.w), f.G);
  f.alpha = make_float2(fminf(0.99f, oa.x), fminf(0.99f, oa.y));
  f.live[0] = f.live[0] && !(f.c_d.x < kNearP0) && !(power.x > 0.0f) && !(f.alpha.x < 1.0f / 255.0f);
  f.live[1] = f.live[1] && !(f.c_d.y < kNearP0) && !(power.y > 0.0f) && !(f.alpha.y < 1.0f / 255.0f);
  // the splat-plane terms feed only the 3D branch's gradients: zero them on
  // lanes that do not take it, where they may be infinite (a p.z too small
  // for its reciprocal) and would turn the branch's zero weights into NaN
  const bool k0 = f.live[0] && f.use3d[0], k1 = f.live[1] && f.use3d[1];
  const float2 z2 = make_float2(0.0f, 0.0f);
  f.sx = sel2(k0, k1, f.sx, z2);
  f.sy = sel2(k0, k1, f.sy, z2);
  f.iz = sel2(k0, k1, f.iz, z2);
}

// Stage 3: both pixels' recurrences and their summed share of the entry's
// 18 gradient values, written to gv[0..17] (P0/cr/backward.cu:337-440,
// P1/cr/backward.cu:340-450).  A lane whose fragments are not live keeps its
// state and writes zeros, so the call needs no branch around it (the
// geometry of a non-live fragment is finite: p.z is replaced by 1 in
// bwd_alpha2).  The part variant also keeps each fragment's weight for its
// semantic gradients.
template <int VARIANT>
__device__ __forceinline__ void bwd_update2(BwdPair& q, const BwdGeom2& f, const float4& r1, const float4& r2,
                                            const float4& r3, const float4& r4, int pos, float (&gv)[32]) {
  const bool l0 = f.live[0], l1 = f.live[1];
  const float2 one = bc<float2>(1.0f), zero = bc<float2>(0.0f);
  // A lane whose fragment does not count runs the update with alpha = 0 and a
  // finite depth: every recurrence below is then exactly the identity in
  // effect (its "last" terms enter the next update with weight 1 - 0), so only
  // T and the gradients need masking.
  const float2 alpha = sel2(l0, l1, f.alpha, zero);
  const float2 G = f.G, c_d = sel2(l0, l1, f.c_d, one);
  const float2 oma = lfma(alpha, bc<float2>(-1.0f), one);                       // 1 - alpha
  const float2 inv_1ma = make_float2(blend_rcp(oma.x), blend_rcp(oma.y));
  const float2 T = sel2(l0, l1, lmul(q.T, inv_1ma), q.T);
  q.T = T;
  const float2 wgt = lmul(alpha, T);                                            // zero where not live
  if (VARIANT == SGR_VARIANT_PART) q.sem_w = wgt;
  const float2 oml = lfma(q.last_alpha, bc<float2>(-1.0f), one);               // 1 - last_alpha
  // colour recurrence on its dot product with dL/dpixel
  const float2 cd = lfma(bc<float2>(r4.z), q.dL_dpixel[2],
                         lfma(bc<float2>(r4.y), q.dL_dpixel[1], lmul(bc<float2>(r4.x), q.dL_dpixel[0])));
  const float2 rec = lfma(q.last_alpha, q.last_col_dot, lmul(oml, q.rec_dot));
  q.rec_dot = rec;
  q.last_col_dot = cd;
  float2 dL_dalpha = ladd(cd, make_float2(-rec.x, -rec.y));
  // depth distortion (mapped depth and its derivative)
  const float2 inv_d = make_float2(blend_rcp(c_d.x), blend_rcp(c_d.y));
  constexpr bool PLAIN = VARIANT == SGR_VARIANT_PLAIN;
  const float2 m_d = PLAIN ? lmul(bc<float2>(kFarP0 / (kFarP0 - kNearP0)), lfma(bc<float2>(-kNearP0), inv_d, one))
                           : lfma(bc<float2>(-kDmdP1f), inv_d, bc<float2>(kMdP1));   // mapped_depth_p1
  const float2 dmd_dd = lmul(bc<float2>(PLAIN ? (kFarP0 * kNearP0) / (kFarP0 - kNearP0) : kDmdP1f),
                             lmul(inv_d, inv_d));
  const bool med0 = pos == q.median_contributor[0] - 1, med1 = pos == q.median_contributor[1] - 1;
  float2 dL_dz = make_float2(med0 ? q.dL_dmedian.x : 0.0f, med1 ? q.dL_dmedian.y : 0.0f);
  // final_D2 + m^2 final_A - 2 m final_D
  const float2 reg = lfma(m_d, lfma(m_d, q.final_A, lmul(bc<float2>(-2.0f), q.final_D)), q.final_D2);
  // part: the median fragment's weight also carries the max-weight map's gradient
  const float2 dL_dweight =
      PLAIN ? lmul(reg, q.dL_dreg)
            : lfma(reg, q.dL_dreg, make_float2(med0 ? q.dL_dmaxw.x : 0.0f, med1 ? q.dL_dmaxw.y : 0.0f));
  dL_dalpha = ladd(dL_dalpha, ladd(dL_dweight, make_float2(-q.last_dL_dT.x, -q.last_dL_dT.y)));
  const float2 ldt = lfma(dL_dweight, alpha, lmul(lfma(alpha, bc<float2>(-1.0f), one), q.last_dL_dT));
  q.last_dL_dT = ldt;
  const float2 dL_dmd = lmul(lmul(bc<float2>(2.0f), wgt),
                             lmul(lfma(m_d, q.final_A, make_float2(-q.final_D.x, -q.final_D.y)), q.dL_dreg));
  dL_dz = lfma(dL_dmd, dmd_dd, dL_dz);
  const float2 acd = lfma(q.last_alpha, q.last_depth, lmul(oml, q.accum_depth));
  q.accum_depth = acd;
  q.last_depth = c_d;
  dL_dalpha = lfma(ladd(c_d, make_float2(-acd.x, -acd.y)), q.dL_ddepth, dL_dalpha);
  // accum_alpha = last_alpha + (1 - last_alpha) accum_alpha, one rounding each
  const float2 aca = ladd(q.last_alpha, lmul(oml, q.accum_alpha));
  q.accum_alpha = aca;
  dL_dalpha = lfma(lfma(aca, bc<float2>(-1.0f), one), q.dL_daccum, dL_dalpha);
  // normal recurrence on its dot product with dL/dnormal
  const float2 nd = lfma(bc<float2>(r3.z), q.dL_dnormal2D[2],
                         lfma(bc<float2>(r3.y), q.dL_dnormal2D[1], lmul(bc<float2>(r3.x), q.dL_dnormal2D[0])));
  const float2 nrec = lfma(q.last_alpha, q.last_nrm_dot, lmul(oml, q.nrm_dot));
  q.nrm_dot = nrec;
  q.last_nrm_dot = nd;
  dL_dalpha = ladd(dL_dalpha, ladd(nd, make_float2(-nrec.x, -nrec.y)));
  dL_dalpha = lmul(dL_dalpha, T);
  q.last_alpha = alpha;
  dL_dalpha = lfma(lmul(make_float2(-q.T_final.x, -q.T_final.y), inv_1ma), q.bg_dot, dL_dalpha);
  dL_dalpha = sel2(l0, l1, dL_dalpha, zero);
  dL_dz = sel2(l0, l1, lfma(wgt, q.dL_ddepth, dL_dz), zero);
  const float2 dL_dG = lmul(bc<float2>(r2.w), dL_dalpha);
  // per-value sums over the two pixels
#pragma unroll
  for (int ch = 0; ch < 3; ++ch) {
    const float2 c = lmul(wgt, q.dL_dpixel[ch]);
    gv[14 + ch] = c.x + c.y;
    const float2 n = lmul(wgt, q.dL_dnormal2D[ch]);
    gv[11 + ch] = n.x + n.y;
  }
  const float2 gG = lmul(G, dL_dalpha);
  gv[17] = gG.x + gG.y;
  // 3D branch (ray-splat intersection) where use3d, 2D (filter) branch elsewhere
  const bool u0 = f.use3d[0], u1 = f.use3d[1];
  const float2 dG3 = sel2(u0, u1, dL_dG, zero), dz3 = sel2(u0, u1, dL_dz, zero);
  const float2 nG = make_float2(-G.x, -G.y);
  const float2 dsx = lmul(lfma(lmul(dG3, nG), f.sx, lmul(dz3, bc<float2>(r1.z))), f.iz);
  const float2 dsy = lmul(lfma(lmul(dG3, nG), f.sy, lmul(dz3, bc<float2>(r1.w))), f.iz);
  const float2 dpz = lfma(dsx, make_float2(-f.sx.x, -f.sx.y), lmul(dsy, make_float2(-f.sy.x, -f.sy.y)));
  // dL/dk = l x dL/dp, dL/dl = dL/dp x k
  const FragGeom<float2>& g = f.g;
  const float2 dkx = lfma(g.ly, dpz, lmul(make_float2(-g.lz.x, -g.lz.y), dsy));
  const float2 dky = lfma(g.lz, dsx, lmul(make_float2(-g.lx.x, -g.lx.y), dpz));
  const float2 dkz = lfma(g.lx, dsy, lmul(make_float2(-g.ly.x, -g.ly.y), dsx));
  const float2 dlx = lfma(dsy, g.kz, lmul(make_float2(-dpz.x, -dpz.y), g.ky));
  const float2 dly = lfma(dpz, g.kx, lmul(make_float2(-dsx.x, -dsx.y), g.kz));
  const float2 dlz = lfma(dsx, g.ky, lmul(make_float2(-dsy.x, -dsy.y), g.kx));
  gv[0] = -(dkx.x + dkx.y);
  gv[1] = -(dky.x + dky.y);
  gv[2] = -(dkz.x + dkz.y);
  gv[3] = -(dlx.x + dlx.y);
  gv[4] = -(dly.x + dly.y);
  gv[5] = -(dlz.x + dlz.y);
  const float2 px2 = bc<float2>(q.pxf);
  const float2 u6 = lfma(px2, dkx, lfma(q.pyf, dlx, lmul(dz3, f.sx)));
  const float2 u7 = lfma(px2, dky, lfma(q.pyf, dly, lmul(dz3, f.sy)));
  const float2 dz2 = sel2(u0, u1, zero, dL_dz);
  const float2 u8 = lfma(px2, dkz, lfma(q.pyf, dlz, ladd(dz3, dz2)));
  gv[6] = u6.x + u6.y;
  gv[7] = u7.x + u7.y;
  gv[8] = u8.x + u8.y;
  const float2 dG2 = sel2(u0, u1, zero, dL_dG);
  const float2 kG = lmul(dG2, lmul(nG, bc<float2>(kFilterInvSquareP0)));
  const float2 u9 = lmul(kG, g.dx), u10 = lmul(kG, g.dy);
  gv[9] = u9.x + u9.y;
  gv[10] = u10.x + u10.y;
}

// Resident CTAs per SM the backward is compiled for (registers per thread =
// 65536 / (128 threads x this)); the part variant's, packed, as many.
#ifndef SGR_BWD_MIN_CTAS
#define SGR_BWD_MIN_CTAS 4
#endif

#ifndef SGR_PART_BWD_MIN_CTAS
#define SGR_PART_BWD_MIN_CTAS (SGR_BWD_PACKED && SGR_PART_PACKED ? 4 : 3)
#endif

// The backward of one tile (all threads of the CTA).
template <int VARIANT, int WX, int SB>
__device__ __forceinline__ void render_bwd_tile(const sgr_batch& b, const GeomView& g, const sgr_bwd_inputs& in,
                                                float* __restrict__ grads, float* __restrict__ dL_dsemantics,
                                                const int tile) {
  using Shape = BwdShapeT<VARIANT, WX>;
  constexpr int PX = Shape::PX, NT = Shape::NT, NW = Shape::NW, NS = kSemSlots<VARIANT>;
  // strip masks with one bit per pixel row pair of a thread, so a warp skips
  // a pixel whose rows the entry cannot reach
  constexpr int SPLIT = SGR_BWD_SPLIT ? PX : 1;
  const int tiles_per_view = g.tiles_x * g.tiles_y;
  const int v = tile / tiles_per_view;
  const int t = tile - v * tiles_per_view;
  const int ty = t / g.tiles_x, tx = t - ty * g.tiles_x;
  const int W = b.width, H = b.height;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const float off = (VARIANT == SGR_VARIANT_PLAIN) ? 0.0f : 0.5f;
  const Strip strip{(float)(tx * kTile) + off, (float)(tx * kTile) + off + (kTile - 1), (float)(ty * kTile) + off};
  const int S = (VARIANT == SGR_VARIANT_PART) ? b.semantic_channels : 0;
  const sgr_view_desc vd = b.views[v];
  const int sid_base = b.scenes[vd.scene].surfel_offset - vd.record_offset;

  __shared__ float4 s_rec[kRecF4 - 1][SB];
  __shared__ uint32_t s_id[SB];
  __shared__ uint8_t s_mask[SB];
  __shared__ uint8_t s_list[NW][SB];
  __shared__ __align__(16) float s_dsem[NS][NT * PX];   // part variant: each pixel's dL/dpixel semantics
  __shared__ int s_max[NW];
  __shared__ uint32_t s_ring[kRing];
  __shared__ int s_count[32];

  const size_t HW = (size_t)H * W;
  const float* fT = g.final_T + (size_t)v * 3 * HW;
  const uint32_t* nc = g.n_contrib + (size_t)v * 2 * HW;
  const int NO = (VARIANT == SGR_VARIANT_PLAIN) ? 7 : 8;
  const float* dpix = in.dL_dcolor + (size_t)v * 3 * HW;
  const float* doth = in.dL_dothers + (size_t)v * NO * HW;
  const float* bg = b.background;

  BwdPixel<VARIANT> q[PX];
  int thread_max = 0;
#pragma unroll
  for (int i = 0; i < PX; ++i) {
    BwdPixel<VARIANT>& Q = q[i];
    int px, py;
    pixel_of<Shape>(tx, ty, lane, warp, i, px, py);
    const bool inside = px < W && py < H;
    const size_t pix = inside ? (size_t)py * W + px : 0;
    Q.pxf = (float)px + off;
    Q.pyf = (float)py + off;
    Q.T_final = inside ? fT[pix] : 0.f;
    Q.T = Q.T_final;
    Q.last_contributor = inside ? (int)nc[pix] : 0;
    Q.median_contributor = inside ? (int)nc[pix + HW] : 0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      Q.dL_dpixel[c] = inside ? dpix[pix + c * HW] : 0.f;
      Q.dL_dnormal2D[c] = inside ? doth[pix + (2 + c) * HW] : 0.f;
#if !SGR_BWD_DOT_REC
      Q.accum_rec[c] = Q.last_color[c] = Q.last_normal[c] = Q.accum_normal[c] = 0.f;
#endif
    }
    Q.dL_ddepth = inside ? doth[pix] : 0.f;
    Q.dL_daccum = inside ? doth[pix + HW] : 0.f;
    Q.dL_dmedian = inside ? doth[pix + 5 * HW] : 0.f;
    Q.dL_dreg = inside ? doth[pix + 6 * HW] : 0.f;
    Q.dL_dmaxw = (VARIANT == SGR_VARIANT_PART && inside) ? doth[pix + 7 * HW] : 0.f;
    Q.sem_w = 0.f;
    if (VARIANT == SGR_VARIANT_PART) {
      const float* ds = in.dL_dsemantic + (size_t)v * S * HW;
      for (int c = 0; c < S; ++c) s_dsem[c][threadIdx.x * PX + i] = inside ? ds[pix + c * HW] : 0.f;
    }
    Q.final_D = inside ? fT[pix + HW] : 0.f;
    Q.final_D2 = inside ? fT[pix + 2 * HW] : 0.f;
    Q.final_A = 1 - Q.T_final;
    Q.bg_dot = bg[0] * Q.dL_dpixel[0] + bg[1] * Q.dL_dpixel[1] + bg[2] * Q.dL_dpixel[2];
    Q.last_alpha = Q.last_depth = Q.accum_depth = Q.accum_alpha = Q.last_dL_dT = 0.f;
#if SGR_BWD_DOT_REC
    Q.rec_dot = Q.last_col_dot = Q.nrm_dot = Q.last_nrm_dot = 0.f;
#endif
    thread_max = max(thread_max, Q.last_contributor);
  }
  // the two pixels of a thread as packed lanes
  constexpr bool PACKED = SGR_BWD_PACKED && kPackedBlend<VARIANT> && PX == 2 && SPLIT == 1;
  BwdPair qp;
  if constexpr (PACKED) qp = to_pair(q);

  int warp_max = thread_max;
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) warp_max = max(warp_max, __shfl_xor_sync(0xffffffffu, warp_max, o));
  if (lane == 0) s_max[warp] = warp_max;
  __syncthreads();
  int block_max = 0;
#pragma unroll
  for (int w = 0; w < NW; ++w) block_max = max(block_max, s_max[w]);

  // positions [0, block_max) of the list, streamed back to front over the
  // span of the cell list the forward scanned
  const uint2 resume = g.tile_resume[tile];
  const uint32_t* list;
  int len;
  cell_list(g, v, tx, ty, list, len);
  int scan_end = min((int)resume.x, len);          // cell-list entries left to stream
  int pos_end = (int)resume.y;                     // tile-list position after them
  const int top = min(block_max, pos_end);
  int head = 0, tail = 0;
  for (int hi = top; hi > 0; hi -= SB, head += SB) {
    while (tail - head < SB && scan_end > 0) {   // refill the ring (CTA-uniform)
      const int i0 = max(0, scan_end - kChunk);
      int found;
      tail += stream_window<true, NT>(g, list, i0, scan_end, (uint32_t)tx, (uint32_t)ty, pos_end, top, s_ring,
                                      tail, s_count, found);
      pos_end -= found;
      scan_end = i0;
    }
    const int n = min(SB, hi);
    if (tail - head < n) {                         // index inconsistent with the rectangles: stop
      if (threadIdx.x == 0) atomicOr(&g.status->flags, SGR_FLAG_LIST_INCONSISTENT);
      break;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < n; e += NT) {
      const uint32_t r = s_ring[(head + e) & (kRing - 1)];
      s_id[e] = r;
      const float4* rec = g.records + (size_t)r * kRecF4;
#pragma unroll
      for (int k = 0; k < kRecF4 - 1; ++k) s_rec[k][e] = rec[k];
      {
        const float4 a0 = s_rec[0][e], a1 = s_rec[1][e], a2 = s_rec[2][e];
        s_mask[e] = (uint8_t)strip_mask_rows<Shape::WX, Shape::WY, NW, SPLIT>(a0, a1, a2, s_rec[3][e].w, rec[5],
                                                                               strip);
      }
    }
    __syncthreads();
    const int cnt = warp_survivors<SPLIT>(s_mask, n, warp, lane, s_list[warp]);
    for (int si = 0; si < cnt; ++si) {
      const int j = s_list[warp][si];
      const int pos = hi - 1 - j;
      const uint32_t rows_live = (s_mask[j] >> (warp * SPLIT)) & ((1u << SPLIT) - 1u);   // which pixels may reach
      if (pos >= warp_max) continue;        // uniform: past every lane's last contributor
      float gv[32];
      const float4 r0 = s_rec[0][j], r1 = s_rec[1][j], r2 = s_rec[2][j];
      const float reach = s_rec[3][j].w;
      if constexpr (PACKED) {
        BwdGeom2 f2;
        if (!__any_sync(0xffffffffu, bwd_reach2(qp, r0, r1, r2, reach, pos, f2))) continue;   // uniform
        bwd_alpha2(r1, r2, f2);
        if (!__any_sync(0xffffffffu, f2.live[0] || f2.live[1])) continue;
        const float4 r3 = s_rec[3][j], r4 = s_rec[4][j];
        bwd_update2<VARIANT>(qp, f2, r1, r2, r3, r4, pos, gv);   // every lane: non-live lanes write zeros
        int which;
        const float total = warp_sum18(gv, lane, which);
        const uint32_t r = s_id[j];
        if (which >= 0 && total != 0.f) atomicAdd(grads + (size_t)r * kGradF + which, total);
        if (VARIANT == SGR_VARIANT_PART && S > 0) {
          // dL/dsemantic[c] = sum over the warp's pixels of weight x dL/dpixel semantic[c];
          // sem_w is zero on a lane whose fragment is not live
          float sv[32];
          int ch;
          float st;
          const float2 sw = qp.sem_w;
          if (S <= 8) {   // uniform: half the values and 9 shuffles instead of 16
#pragma unroll
            for (int c = 0; c < 8; ++c) {
              const float2 d = c < S ? reinterpret_cast<const float2*>(s_dsem[c])[threadIdx.x] : make_float2(0.f, 0.f);
              sv[c] = __fmaf_rn(sw.x, d.x, __fmul_rn(sw.y, d.y));
            }
            st = warp_sum8(sv, lane, ch);
          } else {
#pragma unroll
            for (int c = 0; c < SGR_MAX_SEMANTICS; ++c) {
              const float2 d = c < S ? reinterpret_cast<const float2*>(s_dsem[c])[threadIdx.x] : make_float2(0.f, 0.f);
              sv[c] = __fmaf_rn(sw.x, d.x, __fmul_rn(sw.y, d.y));
            }
            st = warp_sum16(sv, lane, ch);
          }
          if (ch >= 0 && ch < S && st != 0.f) atomicAdd(dL_dsemantics + (size_t)(sid_base + (int)r) * S + ch, st);
        }
      } else {
#pragma unroll
        for (int u = 0; u < 32; ++u) gv[u] = 0.f;
        BwdGeom f[PX];
        bool may = false;
#pragma unroll
        for (int i = 0; i < PX; ++i) {
          f[i].live = false;
          if (SPLIT == 1 || ((rows_live >> i) & 1u)) may |= bwd_reach<VARIANT>(q[i], r0, r1, r2, reach, pos, f[i]);
        }
        if (!__any_sync(0xffffffffu, may)) continue;  // uniform: no pixel of the warp within reach
        bool ok = false;
#pragma unroll
        for (int i = 0; i < PX; ++i) {
          if (SPLIT == 1 || ((rows_live >> i) & 1u)) bwd_alpha<VARIANT>(r1, r2, f[i]);   // uniform
          ok |= f[i].live;
        }
        if (!__any_sync(0xffffffffu, ok)) continue;
        const float4 r3 = s_rec[3][j], r4 = s_rec[4][j];
#pragma unroll
        for (int i = 0; i < PX; ++i)
          if (f[i].live) bwd_update<VARIANT>(q[i], f[i], r1, r2, r3, r4, pos, gv);
        {
          int which;
          const float total = warp_sum18(gv, lane, which);
          const uint32_t r = s_id[j];
          if (which >= 0 && total != 0.f) atomicAdd(grads + (size_t)r * kGradF + which, total);
          if (VARIANT == SGR_VARIANT_PART && S > 0) {
            float sv[32];
            int ch;
            float st;
            if (S <= 8) {   // uniform: half the values and 9 shuffles instead of 16
#pragma unroll
              for (int c = 0; c < 8; ++c) {
                float t = 0.f;
#pragma unroll
                for (int i = 0; i < PX; ++i)
                  if (f[i].live && c < S) t += q[i].sem_w * s_dsem[c][threadIdx.x * PX + i];
                sv[c] = t;
              }
              st = warp_sum8(sv, lane, ch);
            } else {
#pragma unroll
              for (int c = 0; c < SGR_MAX_SEMANTICS; ++c) {
                float t = 0.f;
#pragma unroll
                for (int i = 0; i < PX; ++i)
                  if (f[i].live && c < S) t += q[i].sem_w * s_dsem[c][threadIdx.x * PX + i];
                sv[c] = t;
              }
              st = warp_sum16(sv, lane, ch);
            }
            if (ch >= 0 && ch < S && st != 0.f) atomicAdd(dL_dsemantics + (size_t)(sid_base + (int)r) * S + ch, st);
          }
        }
      }
    }
  }
}

template <int VARIANT, int WX, int SB>
__global__ void __launch_bounds__(BwdShapeT<VARIANT>::NT,
                                  (VARIANT == SGR_VARIANT_PLAIN) ? SGR_BWD_MIN_CTAS : SGR_PART_BWD_MIN_CTAS)
    k_render_bwd(const sgr_batch b, GeomView g, const sgr_bwd_inputs in, float* __restrict__ grads,
                 float* __restrict__ dL_dsemantics, TileQueue q) {
  __shared__ int s_item;
  for (int it = 0;; ++it) {
    int tile;
    if (q.order) {
      __syncthreads();
      if (threadIdx.x == 0) s_item = (int)atomicAdd(q.next, 1u);
      __syncthreads();
      if (s_item >= q.count) return;
      tile = (int)q.order[s_item];
    } else {
      if (it > 0) return;
      tile = blockIdx.x;
    }
    render_bwd_tile<VARIANT, WX, SB>(b, g, in, grads, dL_dsemantics, tile);
  }
}

// Queue order of the tiles, by decreasing estimated cost: for the forward the
// length of the tile's cell list, for the backward the tile-list entries its
// forward found.  Tiles are bucketed by the bit length of their cost (one
// CTA; order inside a bucket is whatever the atomics give: the blends'
// results do not depend on the order tiles run in).  Also resets the queue.
__global__ void __launch_bounds__(1024) k_tile_order(GeomView g, int n, int backward, uint32_t* order,
                                                     uint32_t* next) {
  __shared__ uint32_t s_cnt[33];
  __shared__ uint32_t s_pos[33];
  const int T = g.tiles_x * g.tiles_y;
  const int B = g.cell_tiles;
  const int cx = (g.tiles_x + B - 1) / B, cy = (g.tiles_y + B - 1) / B;
  auto cost = [&](int tile) -> uint32_t {
    if (backward) return g.tile_resume[tile].y;
    const int v = tile / T, t = tile - v * T;
    const int ty = t / g.tiles_x, tx = t - ty * g.tiles_x;
    return g.bin_count[(size_t)v * cx * cy + (size_t)(ty / B) * cx + (tx / B)];
  };
  if (threadIdx.x < 33) s_cnt[threadIdx.x] = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) atomicAdd(&s_cnt[32 - __clz(cost(i))], 1u);
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t run = 0;
    for (int k = 32; k >= 0; --k) {
      s_pos[k] = run;
      run += s_cnt[k];
    }
    *next = 0u;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) order[atomicAdd(&s_pos[32 - __clz(cost(i))], 1u)] = (uint32_t)i;
}

// Host-side launch caches below are shared by every thread that calls the
// library (ctypes callers run without the interpreter lock).
std::mutex& launch_cache_mutex() {
  static std::mutex m;
  return m;
}

// Resident CTAs of a kernel on the current device with `dyn` bytes of
// dynamic shared memory (queried once per kernel, device and size).
template <class F>
int resident_ctas(F kernel, int threads, size_t dyn = 0) {
  struct Entry {
    const void* kernel;
    int dev;
    size_t dyn;
    int ctas;
  };
  constexpr int kEntries = 256;
  static Entry cache[kEntries] = {};
  static int used = 0;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  const void* key = reinterpret_cast<const void*>(kernel);
  std::lock_guard<std::mutex> lock(launch_cache_mutex());
  for (int i = 0; i < used; ++i)
    if (cache[i].kernel == key && cache[i].dev == dev && cache[i].dyn == dyn) return cache[i].ctas;
  int per_sm = 0, sms = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, dyn) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return 0;
  if (used < kEntries) cache[used++] = Entry{key, dev, dyn, per_sm * sms};
  return per_sm * sms;
}

// Bytes of the forward's dynamic shared memory: none for the plain variant;
// for the part variant, (S + 3) / 4 rows of SB float4 (staged semantics) and
// as many rows of kBlock float4 (every pixel's semantic sums).
template <int SB>
size_t fwd_dynamic_bytes(const sgr_batch& b) {
  const int rows = b.variant == SGR_VARIANT_PART ? (b.semantic_channels + 3) / 4 : 0;
  return (size_t)rows * (SB + kBlock) * sizeof(float4);
}

// Lets a kernel take the largest dynamic shared memory the part variant asks
// for (once per kernel and device).
template <class F>
void allow_dynamic_smem(F kernel, int bytes) {
  struct Entry {
    const void* kernel;
    int dev;
  };
  constexpr int kEntries = 256;
  static Entry done[kEntries] = {};
  static int used = 0;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return;
  const void* key = reinterpret_cast<const void*>(kernel);
  std::lock_guard<std::mutex> lock(launch_cache_mutex());
  for (int i = 0; i < used; ++i)
    if (done[i].kernel == key && done[i].dev == dev) return;
  // on failure nothing is recorded: the launch then fails and reports it, and
  // the next launch tries again
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess) return;
  if (used < kEntries) done[used++] = Entry{key, dev};
}

template <int VARIANT, int WX, int SB>
void launch_fwd(const sgr_batch& b, const GeomView& g, const sgr_fwd_outputs& out, TileQueue q, unsigned tiles,
                cudaStream_t st) {
  auto* k = k_render_fwd<VARIANT, WX, SB>;
  const size_t dyn = fwd_dynamic_bytes<SB>(b);
  if (VARIANT == SGR_VARIANT_PART)
    allow_dynamic_smem(k, (int)(((SGR_MAX_SEMANTICS + 3) / 4) * (SB + kBlock) * sizeof(float4)));
  unsigned grid = tiles;
  if (q.order) {
    k_tile_order<<<1, 1024, 0, st>>>(g, (int)tiles, 0, const_cast<uint32_t*>(q.order), q.next);
    count_launches();
    const int r = resident_ctas(k, FwdShapeT<VARIANT, WX>::NT, dyn);
    grid = r > 0 ? std::min<unsigned>(tiles, (unsigned)r) : tiles;
  }
  k<<<grid, FwdShapeT<VARIANT, WX>::NT, dyn, st>>>(b, g, out, q);
}

template <int VARIANT, int WX, int SB>
void launch_bwd(const sgr_batch& b, const GeomView& g, const sgr_bwd_inputs& in, float* grads, float* dsem,
                TileQueue q, unsigned tiles, cudaStream_t st) {
  auto* k = k_render_bwd<VARIANT, WX, SB>;
  constexpr int NT = BwdShapeT<VARIANT>::NT;
  unsigned grid = tiles;
  if (q.order) {
    k_tile_order<<<1, 1024, 0, st>>>(g, (int)tiles, 1, const_cast<uint32_t*>(q.order), q.next);
    count_launches();
    const int r = resident_ctas(k, NT);
    grid = r > 0 ? std::min<unsigned>(tiles, (unsigned)r) : tiles;
  }
  k<<<grid, NT, 0, st>>>(b, g, in, grads, dsem, q);
}

// Entries per staged batch for a batch's launch: as asked, or by default
// 256, except 128 for the part variant above 12 semantic channels.  There
// the 256-entry forward needs 62 KB of shared memory per CTA and fits 3 CTAs
// per SM; the 128-entry one needs 43 KB and fits 4 (measured at 16 channels:
// forward 19.4 -> 16.3 ms, backward unchanged).
inline int stage_entries_of(const sgr_batch& b) {
  if (b.stage_entries == SGR_STAGE_SMALL || b.stage_entries == SGR_STAGE_DEFAULT || b.stage_entries == SGR_STAGE_TINY)
    return b.stage_entries;
  return (b.variant == SGR_VARIANT_PART && b.semantic_channels > 12) ? SGR_STAGE_SMALL : SGR_STAGE_DEFAULT;
}

// Calls fn(variant, warp patch width, staged batch) as integral constants
// for the batch's launch options.
template <class Fn>
void with_blend_shape(const sgr_batch& b, Fn&& fn) {
  using std::integral_constant;
  static_assert(kStageSmall == SGR_STAGE_SMALL && kStageDefault == SGR_STAGE_DEFAULT && kStageTiny == SGR_STAGE_TINY,
                "staged batch sizes");
  const bool narrow = b.blend_shape == SGR_BLEND_PATCH8;
  const int stage = stage_entries_of(b);
  auto by_stage = [&](auto variant, auto wx) {
    if (stage == kStageSmall)
      fn(variant, wx, integral_constant<int, kStageSmall>{});
    else if (stage == kStageTiny)
      fn(variant, wx, integral_constant<int, kStageTiny>{});
    else
      fn(variant, wx, integral_constant<int, kStageDefault>{});
  };
  auto by_width = [&](auto variant) {
    narrow ? by_stage(variant, integral_constant<int, 8>{}) : by_stage(variant, integral_constant<int, kTile>{});
  };
  b.variant == SGR_VARIANT_PLAIN ? by_width(integral_constant<int, SGR_VARIANT_PLAIN>{})
                                 : by_width(integral_constant<int, SGR_VARIANT_PART>{});
}

TileQueue tile_queue(const sgr_batch& b, const GeomView& g, unsigned tiles) {
  TileQueue q{nullptr, nullptr, (int)tiles};
  if (b.tile_schedule == SGR_SCHEDULE_QUEUE && g.tile_queue) {
    q.order = g.tile_queue;
    q.next = g.tile_queue + tiles;
  }
  return q;
}

void launch_render_fwd(const sgr_batch& b, const GeomView& g, const sgr_fwd_outputs& out, cudaStream_t st) {
  const unsigned tiles = (unsigned)(g.tiles_x * g.tiles_y) * (unsigned)b.num_views;
  if (tiles == 0) return;
  const TileQueue q = tile_queue(b, g, tiles);
  with_blend_shape(b, [&](auto variant, auto wx, auto sb) {
    launch_fwd<decltype(variant)::value, decltype(wx)::value, decltype(sb)::value>(b, g, out, q, tiles, st);
  });
  count_launches();
}

void launch_render_bwd(const sgr_batch& b, const GeomView& g, const sgr_bwd_inputs& in, float* grads,
                       float* dL_dsemantics, cudaStream_t st) {
  const unsigned tiles = (unsigned)(g.tiles_x * g.tiles_y) * (unsigned)b.num_views;
  if (tiles == 0) return;
  const TileQueue q = tile_queue(b, g, tiles);
  with_blend_shape(b, [&](auto variant, auto wx, auto sb) {
    launch_bwd<decltype(variant)::value, decltype(wx)::value, decltype(sb)::value>(b, g, in, grads, dL_dsemantics,
                                                                                    q, tiles, st);
  });
  count_launches();
}

}  // namespace sgr
