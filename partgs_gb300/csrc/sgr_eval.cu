// Chamfer evaluation on the GPU (utils/blender_eval.py:25-111): exact
// nearest neighbours between point sets and the radius downsample.
//
// Nearest neighbours, brute force (sgr_nn_search): each thread owns 4 query
// points; the reference points stream through shared memory 1024 at a time
// and every thread tests all of them (squared distances, first minimum kept
// on ties).
//
// Nearest neighbours through a cell grid (sgr_nn_search_grid): the same
// squared distances in the same arithmetic, the same tie rule, so the same
// distances and indices bit for bit.  The reference points are counted into
// a uniform grid of about two cells per point and scattered in cell order;
// the queries are sorted by cell, so a warp's queries search neighbouring
// cells.  Each query visits shells of cells around its own (Chebyshev ring
// k = 0, 1, ...), skipping cells whose box is farther than the best distance
// so far, and stops once the best squared distance is below the squared
// distance to every cell outside the searched cube.  The bounds carry a
// margin that covers the fp32 rounding of the cell assignment, the cell
// faces and the squared distances.  Slabs and rows of cells beyond the best
// distance are skipped whole.  Queries still open after 6 shells (far from
// every reference point: in an empty region or outside the points' box) are
// listed and searched the same way in a second grid of cells eight times
// wider, up to 64 shells; the rare query that leaves open is finished by the
// brute-force scan.
//
// Radius downsample (sgr_radius_downsample): the reference keeps point i of
// its shuffled order unless an earlier kept point lies within the radius
// (a sequential greedy pass over scikit-learn's radius neighbours).  That is
// the lexicographically first maximal independent set of the radius graph in
// that order, which parallel rounds reproduce exactly: a point is removed
// once a kept neighbour exists and kept once every earlier neighbour is
// removed.  Neighbours come from a cell grid of edge `radius`: points sorted
// by packed cell key (CUB), 27 cells searched by binary search.  Each round
// synchronises the host to read the count of undecided points; this is an
// evaluation path, not part of the training step.

#include <cuda_runtime.h>

#include <cfloat>
#include <climits>
#include <cstdint>

#include "../../include/sgr.h"
#include "sgr_sort.cuh"

namespace sgr {
void count_launches(int n);   // sgr_api.cu
}  // namespace sgr

namespace sgreval {

constexpr int kNNThreads = 256;
constexpr int kNNQ = 4;           // queries per thread
constexpr int kNNTile = 1024;     // reference points per shared-memory tile

// Squared distance, rounded the same way in every search kernel.
__device__ __forceinline__ float nn_d2(float qx, float qy, float qz, float rx, float ry, float rz) {
  const float dx = qx - rx, dy = qy - ry, dz = qz - rz;
  return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

// Brute force over all of r.  With `list`, the queries are list[0 .. *count)
// (the grid search's open queries) instead of 0 .. n.
__global__ void __launch_bounds__(kNNThreads) k_nn(const float* __restrict__ q, long long n,
                                                  const float* __restrict__ r, long long m,
                                                  float* __restrict__ dist, int* __restrict__ idx,
                                                  const int* __restrict__ list, const unsigned* __restrict__ count) {
  __shared__ float s_r[kNNTile * 3];
  if (list) n = (long long)*count;
  const long long q0 = ((long long)blockIdx.x * kNNThreads + threadIdx.x) * kNNQ;
  if ((long long)blockIdx.x * kNNThreads * kNNQ >= n) return;   // uniform over the block
  float qx[kNNQ], qy[kNNQ], qz[kNNQ], best[kNNQ];
  int arg[kNNQ];
#pragma unroll
  for (int k = 0; k < kNNQ; ++k) {
    const long long i = q0 + k;
    const long long qi = i < n ? (list ? (long long)list[i] : i) : 0;
    qx[k] = i < n ? q[3 * qi] : 0.f;
    qy[k] = i < n ? q[3 * qi + 1] : 0.f;
    qz[k] = i < n ? q[3 * qi + 2] : 0.f;
    best[k] = FLT_MAX;
    arg[k] = -1;
  }
  for (long long t0 = 0; t0 < m; t0 += kNNTile) {
    const int cnt = (int)min((long long)kNNTile, m - t0);
    __syncthreads();
    for (int e = threadIdx.x; e < cnt * 3; e += kNNThreads) s_r[e] = r[3 * t0 + e];
    __syncthreads();
    for (int j = 0; j < cnt; ++j) {
      const float rx = s_r[3 * j], ry = s_r[3 * j + 1], rz = s_r[3 * j + 2];
#pragma unroll
      for (int k = 0; k < kNNQ; ++k) {
        const float d2 = nn_d2(qx[k], qy[k], qz[k], rx, ry, rz);
        if (d2 < best[k]) {
          best[k] = d2;
          arg[k] = (int)(t0 + j);
        }
      }
    }
  }
#pragma unroll
  for (int k = 0; k < kNNQ; ++k) {
    const long long i = q0 + k;
    if (i < n) {
      const long long qi = list ? (long long)list[i] : i;
      dist[qi] = sqrtf(best[k]);
      if (idx) idx[qi] = arg[k];
    }
  }
}

// ---- grid nearest neighbours -------------------------------------------------

struct NNGrid {
  float lox, loy, loz;   // grid origin (the reference points' box corner)
  float h, inv;          // cell edge and its inverse
  float margin;          // covers fp32 rounding of cell assignment, faces and distances
  float hix, hiy, hiz;   // far corner of the reference points' box (inside lo + n h)
  int nx, ny, nz;
  int shells;            // shells a query searches before the brute-force scan takes it
};

__device__ __forceinline__ int grid_axis(float p, float lo, float inv, int n) {
  return min(max((int)floorf((p - lo) * inv), 0), n - 1);
}

// Distance along one axis from p to cell c's slab [lo + c h, lo + (c+1) h].
__device__ __forceinline__ float slab_gap(float p, int c, float lo, float h) {
  const float a = lo + (float)c * h, b = lo + (float)(c + 1) * h;
  return fmaxf(0.0f, fmaxf(a - p, p - b));
}

__global__ void k_grid_count(const float* __restrict__ r, long long m, NNGrid g, uint32_t* __restrict__ count) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const int x = grid_axis(r[3 * i], g.lox, g.inv, g.nx), y = grid_axis(r[3 * i + 1], g.loy, g.inv, g.ny),
            z = grid_axis(r[3 * i + 2], g.loz, g.inv, g.nz);
  atomicAdd(count + ((long long)z * g.ny + y) * g.nx + x, 1u);
}

// Reference points in cell order as (x, y, z, index bits); the order within
// a cell does not matter (ties are decided by index).
__global__ void k_grid_scatter(const float* __restrict__ r, long long m, NNGrid g, const uint32_t* __restrict__ start,
                               uint32_t* __restrict__ cursor, float4* __restrict__ pts) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const float x = r[3 * i], y = r[3 * i + 1], z = r[3 * i + 2];
  const long long c = ((long long)grid_axis(z, g.loz, g.inv, g.nz) * g.ny + grid_axis(y, g.loy, g.inv, g.ny)) * g.nx +
                      grid_axis(x, g.lox, g.inv, g.nx);
  const uint32_t at = start[c] + atomicAdd(cursor + c, 1u);
  if (at < start[c + 1]) pts[at] = make_float4(x, y, z, __int_as_float((int)i));   // always: same cell as counted
}

__global__ void k_query_cells(const float* __restrict__ q, long long n, NNGrid g, uint32_t* __restrict__ keys,
                              int* __restrict__ ids) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  keys[i] = (uint32_t)(((long long)grid_axis(q[3 * i + 2], g.loz, g.inv, g.nz) * g.ny +
                        grid_axis(q[3 * i + 1], g.loy, g.inv, g.ny)) * g.nx +
                       grid_axis(q[3 * i], g.lox, g.inv, g.nx));
  ids[i] = (int)i;
}

// Squared lower bound of the distance from p to the grid cells outside the
// cube [c - k, c + k] on each axis, or FLT_MAX when the cube holds the whole
// grid.  Those cells lie in six slabs (beyond each face of the cube that is
// inside the grid); the distance to a slab is taken inside the reference
// points' box, so a query outside the box (or off a flat point set) gets its
// distance to the points' part of the slab.
__device__ __forceinline__ float outside_bound2(float px, float py, float pz, int cx, int cy, int cz, int k,
                                                const NNGrid& g) {
  const float ox = fmaxf(0.0f, fmaxf(g.lox - px, px - g.hix) - g.margin);
  const float oy = fmaxf(0.0f, fmaxf(g.loy - py, py - g.hiy) - g.margin);
  const float oz = fmaxf(0.0f, fmaxf(g.loz - pz, pz - g.hiz) - g.margin);
  float b2 = FLT_MAX;
  auto face = [&](float d, float o1, float o2) {
    const float t = fmaxf(0.0f, fmaxf(d, 0.0f) - g.margin);
    b2 = fminf(b2, t * t + o1 * o1 + o2 * o2);
  };
  if (cx - k > 0) face(px - (g.lox + (float)(cx - k) * g.h), oy, oz);
  if (cx + k + 1 < g.nx) face((g.lox + (float)(cx + k + 1) * g.h) - px, oy, oz);
  if (cy - k > 0) face(py - (g.loy + (float)(cy - k) * g.h), ox, oz);
  if (cy + k + 1 < g.ny) face((g.loy + (float)(cy + k + 1) * g.h) - py, ox, oz);
  if (cz - k > 0) face(pz - (g.loz + (float)(cz - k) * g.h), ox, oy);
  if (cz + k + 1 < g.nz) face((g.loz + (float)(cz + k + 1) * g.h) - pz, ox, oy);
  return b2;
}

// One thread per query, in cell order (order[0 .. n), or order[0 .. *n_in)
// for the queries the finer level left open).  A cell is searched unless its box
// lies farther than the best distance so far; the shell loop ends when the
// best squared distance is below the bound of everything outside, with a
// relative 2e-6 kept for the rounding of the squared distances, so no
// unsearched point can have a smaller (or equal) computed squared distance.
__global__ void __launch_bounds__(256) k_nn_grid(const float* __restrict__ q, const int* __restrict__ order,
                                                 long long n, const unsigned* __restrict__ n_in, NNGrid g,
                                                 const uint32_t* __restrict__ start, const float4* __restrict__ pts,
                                                 float* __restrict__ dist, int* __restrict__ idx,
                                                 int* __restrict__ open, unsigned* __restrict__ n_open) {
  if (n_in) n = (long long)*n_in;   // the previous level's open queries
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int qi = order[t];
  const float px = q[3 * (long long)qi], py = q[3 * (long long)qi + 1], pz = q[3 * (long long)qi + 2];
  const int cx = grid_axis(px, g.lox, g.inv, g.nx), cy = grid_axis(py, g.loy, g.inv, g.ny),
            cz = grid_axis(pz, g.loz, g.inv, g.nz);
  float best = FLT_MAX;
  int arg = INT_MAX;
  bool done = false;
  // true when every point of a box at squared gap g2 is farther than best
  auto beyond = [&](float g2) {
    const float gap = fmaxf(0.0f, sqrtf(g2) - g.margin);
    return gap * gap * (1.0f - 2e-6f) > best;
  };
  for (int k = 0; k <= g.shells && !done; ++k) {
    for (int dz = max(-k, -cz); dz <= min(k, g.nz - 1 - cz); ++dz) {
      const int z = cz + dz;
      const float gz = slab_gap(pz, z, g.loz, g.h);
      if (beyond(gz * gz)) continue;                 // the whole slab
      for (int dy = max(-k, -cy); dy <= min(k, g.ny - 1 - cy); ++dy) {
        const int y = cy + dy;
        const float gy = slab_gap(py, y, g.loy, g.h);
        if (beyond(gy * gy + gz * gz)) continue;     // the whole row
        const int step = (dz == -k || dz == k || dy == -k || dy == k) ? 1 : 2 * k;   // k = 0 takes the first
        for (int dx = -k; dx <= k; dx += step) {
          const int x = cx + dx;
          if (x < 0 || x >= g.nx) continue;
          const float gx = slab_gap(px, x, g.lox, g.h);
          if (beyond(gx * gx + gy * gy + gz * gz)) continue;
          const long long c = ((long long)z * g.ny + y) * g.nx + x;
          const uint32_t e = start[c + 1];
          for (uint32_t j = start[c]; j < e; ++j) {
            const float4 rp = pts[j];
            const float d2 = nn_d2(px, py, pz, rp.x, rp.y, rp.z);
            const int id = __float_as_int(rp.w);
            if (d2 < best || (d2 == best && id < arg)) {
              best = d2;
              arg = id;
            }
          }
        }
      }
    }
    const float b2 = outside_bound2(px, py, pz, cx, cy, cz, k, g);
    done = b2 == FLT_MAX || best < b2 * (1.0f - 2e-6f);
  }
  if (done) {
    dist[qi] = sqrtf(best);
    if (idx) idx[qi] = arg == INT_MAX ? -1 : arg;
  } else {
    open[atomicAdd(n_open, 1u)] = qi;
  }
}

struct NNLayout {
  size_t start, cursor, pts, start2, cursor2, pts2, keys, keys_sorted, ids, ids_sorted, open, n_open, open2, n_open2,
      temp, temp_bytes, end;
};

// Grid shape for m reference points in the box [lo, hi]: about
// `per_point` cells per point, at most 1024 cells on an axis, found by
// bisection on the edge.
bool nn_grid(int64_t m, const float* lo, const float* hi, NNGrid& g, double per_point, int shells) {
  double ext[3], maxext = 0.0, maxabs = 0.0;
  for (int a = 0; a < 3; ++a) {
    if (!(hi[a] >= lo[a]) || !isfinite(lo[a]) || !isfinite(hi[a])) return false;
    ext[a] = (double)hi[a] - (double)lo[a];
    maxext = fmax(maxext, ext[a]);
    maxabs = fmax(maxabs, fmax(fabs((double)lo[a]), fabs((double)hi[a])));
  }
  const double target = fmin(fmax(per_point * (double)m, 1.0), (double)(1 << 26));
  auto cells = [&](double h) {
    double c = 1.0;
    for (int a = 0; a < 3; ++a) c *= fmax(1.0, ceil(ext[a] / h));
    return c;
  };
  double h = 1.0;
  if (maxext > 0.0) {
    double a = maxext / 1024.0, b = maxext * 2.0;   // cells(b) = 1
    if (cells(a) <= target) {
      b = a;
    } else {
      for (int it = 0; it < 100; ++it) {
        const double mid = 0.5 * (a + b);
        if (cells(mid) <= target) b = mid; else a = mid;
      }
    }
    h = b * (1.0 + 1e-6);
  }
  int n[3];
  for (int a = 0; a < 3; ++a) n[a] = maxext > 0.0 ? (int)fmax(1.0, ceil(ext[a] / h)) : 1;
  g.lox = lo[0];
  g.loy = lo[1];
  g.loz = lo[2];
  g.h = (float)h;
  g.inv = (float)(1.0 / h);
  g.nx = n[0];
  g.ny = n[1];
  g.nz = n[2];
  g.hix = hi[0];
  g.hiy = hi[1];
  g.hiz = hi[2];
  g.margin = (float)(1e-3 * h + 1e-6 * maxabs);
  g.shells = shells;
  return true;
}

// The fine level (two cells per point, 6 shells) and the coarse one (edge
// about eight times longer, shells until the cube holds the grid, up to 64)
// that takes the queries the fine level leaves open: queries in empty
// regions, and far outside the points' box.
constexpr double kFinePerPoint = 2.0, kCoarsePerPoint = 2.0 / 512.0;
constexpr int kFineShells = 6, kCoarseShells = 64;

NNLayout nn_layout(long long n, long long m, long long cells, long long cells2) {
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  NNLayout L;
  size_t o = 0;
  L.start = o; o = al(o + (cells + 1) * 4);
  L.cursor = o; o = al(o + cells * 4);
  L.pts = o; o = al(o + m * 16);
  L.start2 = o; o = al(o + (cells2 + 1) * 4);
  L.cursor2 = o; o = al(o + cells2 * 4);
  L.pts2 = o; o = al(o + m * 16);
  L.keys = o; o = al(o + n * 4);
  L.keys_sorted = o; o = al(o + n * 4);
  L.ids = o; o = al(o + n * 4);
  L.ids_sorted = o; o = al(o + n * 4);
  L.open = o; o = al(o + n * 4);
  L.n_open = o; o = al(o + 4);
  L.open2 = o; o = al(o + n * 4);
  L.n_open2 = o; o = al(o + 4);
  const size_t ts = sgr::scan_temp_bytes<uint32_t>((long long)((cells > cells2 ? cells : cells2) + 1));
  const size_t tr = sgr::radix_sort_temp_bytes<uint32_t>((long long)n);
  L.temp = o;
  L.temp_bytes = ts > tr ? ts : tr;
  o = al(o + L.temp_bytes);
  L.end = o;
  return L;
}

int key_bits(long long cells) {
  int b = 1;
  while (b < 32 && (1ll << b) < cells) ++b;
  return b;
}

// ---- radius downsample -------------------------------------------------------
// In fp64 like the reference (numpy / scikit-learn): squared distances
// accumulated x, y, z in that order without contraction, compared with
// radius^2 inclusively.  The cell edge is radius (1 + 1e-7), so every pair
// within the radius lies in adjacent cells despite rounding.
__device__ __forceinline__ unsigned long long cell_key(int cx, int cy, int cz) {
  return ((unsigned long long)(cx & 0x1FFFFF) << 42) | ((unsigned long long)(cy & 0x1FFFFF) << 21) |
         (unsigned long long)(cz & 0x1FFFFF);
}

__device__ __forceinline__ void cell_of(const double* p, double3 lo, double inv, int& cx, int& cy, int& cz) {
  cx = (int)floor((p[0] - lo.x) * inv);
  cy = (int)floor((p[1] - lo.y) * inv);
  cz = (int)floor((p[2] - lo.z) * inv);
}

__device__ __forceinline__ double dist2(const double* a, const double* b) {
  const double ex = a[0] - b[0], ey = a[1] - b[1], ez = a[2] - b[2];
  return __dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez));
}

__global__ void k_cell_keys(const double* __restrict__ pts, long long n, double3 lo, double inv,
                            unsigned long long* __restrict__ keys, int* __restrict__ ids) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int cx, cy, cz;
  cell_of(pts + 3 * i, lo, inv, cx, cy, cz);
  keys[i] = cell_key(cx, cy, cz);
  ids[i] = (int)i;
}

__device__ __forceinline__ long long lower_bound(const unsigned long long* a, long long n, unsigned long long k) {
  long long lo = 0, hi = n;
  while (lo < hi) {
    const long long mid = (lo + hi) >> 1;
    if (a[mid] < k) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// One round of the parallel greedy.  state: 0 undecided, 1 kept, 2 removed;
// point order = index order.  A later neighbour is only ever kept after
// every earlier one was removed, so "a kept neighbour" means "an earlier
// kept neighbour", and a point with no undecided earlier neighbour left is
// kept, exactly as the sequential pass decides it.
__global__ void k_mis_round(const double* __restrict__ pts, long long n, double3 lo, double inv, double r2,
                            const unsigned long long* __restrict__ keys, const int* __restrict__ ids,
                            const uint8_t* __restrict__ state_in, uint8_t* __restrict__ state_out,
                            unsigned long long* __restrict__ undecided) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint8_t s = state_in[i];
  if (s != 0) {
    state_out[i] = s;
    return;
  }
  const double* p = pts + 3 * i;
  int cx, cy, cz;
  cell_of(p, lo, inv, cx, cy, cz);
  bool earlier_open = false, kept_near = false;
  for (int dz = -1; dz <= 1 && !kept_near; ++dz)
    for (int dy = -1; dy <= 1 && !kept_near; ++dy)
      for (int dx = -1; dx <= 1 && !kept_near; ++dx) {
        const unsigned long long k = cell_key(cx + dx, cy + dy, cz + dz);
        for (long long j = lower_bound(keys, n, k); j < n && keys[j] == k; ++j) {
          const int o = ids[j];
          if (o == (int)i) continue;
          const uint8_t so = state_in[o];
          if (so == 2 || (so == 0 && o > i)) continue;   // cannot decide i
          if (dist2(pts + 3 * (long long)o, p) > r2) continue;
          if (so == 1) {
            kept_near = true;
            break;
          }
          earlier_open = true;
        }
      }
  uint8_t out = 0;
  if (kept_near) out = 2;
  else if (!earlier_open) out = 1;
  state_out[i] = out;
  if (out == 0) atomicAdd(undecided, 1ull);
}

struct DSLayout {
  size_t keys, keys_sorted, ids, ids_sorted, state_a, state_b, count, temp, temp_bytes, end;
};

DSLayout ds_layout(long long n) {
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  DSLayout L;
  size_t o = 0;
  L.keys = o; o = al(o + n * 8);
  L.keys_sorted = o; o = al(o + n * 8);
  L.ids = o; o = al(o + n * 4);
  L.ids_sorted = o; o = al(o + n * 4);
  L.state_a = o; o = al(o + n);
  L.state_b = o; o = al(o + n);
  L.count = o; o = al(o + 8);
  const size_t tb = sgr::radix_sort_temp_bytes<unsigned long long>((long long)n);
  L.temp = o;
  L.temp_bytes = tb;
  o = al(o + tb);
  L.end = o;
  return L;
}

}  // namespace sgreval

using namespace sgreval;

extern "C" {

int sgr_nn_search(const float* q, int64_t n, const float* r, int64_t m, float* dist, int32_t* idx, void* stream) {
  if (n < 0 || m < 0 || (n > 0 && (!q || !dist)) || (n > 0 && m > 0 && !r)) return SGR_ERR_INVALID_ARGUMENT;
  if (m > 0x7fffffffLL) return SGR_ERR_UNSUPPORTED;
  if (n == 0) return SGR_OK;
  if (m == 0) return SGR_ERR_INVALID_ARGUMENT;
  const long long blocks = (n + (long long)kNNThreads * kNNQ - 1) / ((long long)kNNThreads * kNNQ);
  k_nn<<<(unsigned)blocks, kNNThreads, 0, static_cast<cudaStream_t>(stream)>>>(q, n, r, m, dist, idx, nullptr,
                                                                              nullptr);
  sgr::count_launches(1);
  return cudaGetLastError() == cudaSuccess ? SGR_OK : SGR_ERR_CUDA;
}

size_t sgr_nn_grid_scratch_bytes(int64_t n, int64_t m, const float* lo, const float* hi) {
  NNGrid g, g2;
  if (n < 0 || m < 0 || !lo || !hi || !nn_grid(m, lo, hi, g, kFinePerPoint, kFineShells) ||
      !nn_grid(m, lo, hi, g2, kCoarsePerPoint, kCoarseShells))
    return 0;
  return nn_layout(n, m, (long long)g.nx * g.ny * g.nz, (long long)g2.nx * g2.ny * g2.nz).end;
}

int sgr_nn_search_grid(const float* q, int64_t n, const float* r, int64_t m, const float* lo, const float* hi,
                       float* dist, int32_t* idx, void* scratch, size_t scratch_bytes, void* stream) {
  if (n < 0 || m < 0 || (n > 0 && (!q || !dist)) || (n > 0 && m > 0 && (!r || !lo || !hi)))
    return SGR_ERR_INVALID_ARGUMENT;
  if (m > 0x7fffffffLL || n > 0x7fffffffLL) return SGR_ERR_UNSUPPORTED;
  if (n == 0) return SGR_OK;
  if (m == 0) return SGR_ERR_INVALID_ARGUMENT;
  NNGrid g, g2;
  if (!nn_grid(m, lo, hi, g, kFinePerPoint, kFineShells) || !nn_grid(m, lo, hi, g2, kCoarsePerPoint, kCoarseShells))
    return SGR_ERR_INVALID_ARGUMENT;
  const long long cells = (long long)g.nx * g.ny * g.nz, cells2 = (long long)g2.nx * g2.ny * g2.nz;
  const NNLayout L = nn_layout(n, m, cells, cells2);
  if (!scratch || scratch_bytes < L.end) return SGR_ERR_WORKSPACE;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* sp = static_cast<char*>(scratch);
  auto* start = reinterpret_cast<uint32_t*>(sp + L.start);
  auto* cursor = reinterpret_cast<uint32_t*>(sp + L.cursor);
  auto* pts = reinterpret_cast<float4*>(sp + L.pts);
  auto* keys = reinterpret_cast<uint32_t*>(sp + L.keys);
  auto* keys_sorted = reinterpret_cast<uint32_t*>(sp + L.keys_sorted);
  auto* ids = reinterpret_cast<int*>(sp + L.ids);
  auto* ids_sorted = reinterpret_cast<int*>(sp + L.ids_sorted);
  auto* open = reinterpret_cast<int*>(sp + L.open);
  auto* n_open = reinterpret_cast<unsigned*>(sp + L.n_open);
  auto* start2 = reinterpret_cast<uint32_t*>(sp + L.start2);
  auto* cursor2 = reinterpret_cast<uint32_t*>(sp + L.cursor2);
  auto* pts2 = reinterpret_cast<float4*>(sp + L.pts2);
  auto* open2 = reinterpret_cast<int*>(sp + L.open2);
  auto* n_open2 = reinterpret_cast<unsigned*>(sp + L.n_open2);
  const unsigned mb = (unsigned)((m + 255) / 256), nb = (unsigned)((n + 255) / 256);
  if (cudaMemsetAsync(start, 0, (cells + 1) * 4, st) != cudaSuccess ||
      cudaMemsetAsync(cursor, 0, cells * 4, st) != cudaSuccess || cudaMemsetAsync(n_open, 0, 4, st) != cudaSuccess ||
      cudaMemsetAsync(start2, 0, (cells2 + 1) * 4, st) != cudaSuccess ||
      cudaMemsetAsync(cursor2, 0, cells2 * 4, st) != cudaSuccess || cudaMemsetAsync(n_open2, 0, 4, st) != cudaSuccess)
    return SGR_ERR_CUDA;
  for (int level = 0; level < 2; ++level) {   // both grids: count, scan, scatter
    const NNGrid& gl = level ? g2 : g;
    uint32_t* sl = level ? start2 : start;
    k_grid_count<<<mb, 256, 0, st>>>(r, m, gl, sl);
    if (sgr::prefix_sum<uint32_t, false>(sl, sl, (long long)((level ? cells2 : cells) + 1), sp + L.temp, L.temp_bytes,
                                         st) != SGR_OK)
      return SGR_ERR_CUDA;
    k_grid_scatter<<<mb, 256, 0, st>>>(r, m, gl, sl, level ? cursor2 : cursor, level ? pts2 : pts);
  }
  k_query_cells<<<nb, 256, 0, st>>>(q, n, g, keys, ids);
  if (sgr::radix_sort_pairs<uint32_t>(keys, keys_sorted, reinterpret_cast<const uint32_t*>(ids),
                                      reinterpret_cast<uint32_t*>(ids_sorted), (long long)n, key_bits(cells),
                                      sp + L.temp, L.temp_bytes, st) != SGR_OK)
    return SGR_ERR_CUDA;
  k_nn_grid<<<nb, 256, 0, st>>>(q, ids_sorted, n, nullptr, g, start, pts, dist, idx, open, n_open);
  // the open queries (count known only on the device): blocks past it return at once
  k_nn_grid<<<nb, 256, 0, st>>>(q, open, n, n_open, g2, start2, pts2, dist, idx, open2, n_open2);
  const long long blocks = (n + (long long)kNNThreads * kNNQ - 1) / ((long long)kNNThreads * kNNQ);
  k_nn<<<(unsigned)blocks, kNNThreads, 0, st>>>(q, n, r, m, dist, idx, open2, n_open2);
  sgr::count_launches(8);
  return cudaGetLastError() == cudaSuccess ? SGR_OK : SGR_ERR_CUDA;
}

size_t sgr_downsample_scratch_bytes(int64_t n) { return n < 0 ? 0 : ds_layout(n).end; }

int sgr_radius_downsample(const double* pts, int64_t n, const double* lo, const double* hi, double radius,
                          uint8_t* state, void* scratch, size_t scratch_bytes, int32_t* rounds, void* stream) {
  if (n < 0 || !(radius > 0.0) || (n > 0 && (!pts || !lo || !hi || !state))) return SGR_ERR_INVALID_ARGUMENT;
  if (n > 0x7fffffffLL) return SGR_ERR_UNSUPPORTED;
  if (n == 0) return SGR_OK;
  for (int k = 0; k < 3; ++k)   // cells must fit the 21-bit key fields, with a spare cell on each side
    if (!(hi[k] >= lo[k]) || (hi[k] - lo[k]) / radius > (double)(1 << 20)) return SGR_ERR_UNSUPPORTED;
  const DSLayout L = ds_layout(n);
  if (!scratch || scratch_bytes < L.end) return SGR_ERR_WORKSPACE;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* sp = static_cast<char*>(scratch);
  auto* keys = reinterpret_cast<unsigned long long*>(sp + L.keys);
  auto* keys_sorted = reinterpret_cast<unsigned long long*>(sp + L.keys_sorted);
  auto* ids = reinterpret_cast<int*>(sp + L.ids);
  auto* ids_sorted = reinterpret_cast<int*>(sp + L.ids_sorted);
  auto* sa = reinterpret_cast<uint8_t*>(sp + L.state_a);
  auto* sb = reinterpret_cast<uint8_t*>(sp + L.state_b);
  auto* count = reinterpret_cast<unsigned long long*>(sp + L.count);
  const double edge = radius * (1.0 + 1e-7);
  const double3 lo3 = make_double3(lo[0] - edge, lo[1] - edge, lo[2] - edge);
  const double inv = 1.0 / edge;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  k_cell_keys<<<blocks, 256, 0, st>>>(pts, n, lo3, inv, keys, ids);
  sgr::count_launches(1);
  if (sgr::radix_sort_pairs<unsigned long long>(keys, keys_sorted, reinterpret_cast<const uint32_t*>(ids),
                                                reinterpret_cast<uint32_t*>(ids_sorted), (long long)n, 63,
                                                sp + L.temp, L.temp_bytes, st) != SGR_OK)
    return SGR_ERR_CUDA;
  if (cudaMemsetAsync(sa, 0, n, st) != cudaSuccess) return SGR_ERR_CUDA;
  // Every round decides at least the lowest-index undecided point (its
  // earlier neighbours are all decided), so n rounds always suffice.
  long long r = 0;
  unsigned long long left = 1;
  for (; r <= n && left != 0; ++r) {
    left = 0;
    if (cudaMemsetAsync(count, 0, 8, st) != cudaSuccess) return SGR_ERR_CUDA;
    k_mis_round<<<blocks, 256, 0, st>>>(pts, n, lo3, inv, radius * radius, keys_sorted, ids_sorted, sa, sb, count);
    sgr::count_launches(1);
    if (cudaMemcpyAsync(&left, count, 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return SGR_ERR_CUDA;
    uint8_t* t = sa;
    sa = sb;
    sb = t;
  }
  if (left != 0) return SGR_ERR_CUDA;   // cannot happen: see above
  if (rounds) *rounds = (int32_t)min(r, (long long)INT32_MAX);
  if (cudaMemcpyAsync(state, sa, n, cudaMemcpyDeviceToDevice, st) != cudaSuccess) return SGR_ERR_CUDA;
  return cudaGetLastError() == cudaSuccess ? SGR_OK : SGR_ERR_CUDA;
}

}  // extern "C"
