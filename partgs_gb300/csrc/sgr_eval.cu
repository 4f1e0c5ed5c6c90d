// Chamfer evaluation on the GPU (utils/blender_eval.py:25-111): exact
// nearest neighbours between point sets and the radius downsample.
//
// Nearest neighbours (sgr_nn_search): brute force, exact in fp32.  Each
// thread owns 4 query points; the reference points stream through shared
// memory 1024 at a time and every thread tests all of them (squared
// distances, first minimum kept on ties).
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
#include <cub/device/device_radix_sort.cuh>

#include <cuda_runtime.h>

#include <cfloat>
#include <climits>
#include <cstdint>

#include "../../include/sgr.h"

namespace sgr {
void count_launches(int n);   // sgr_api.cu
}  // namespace sgr

namespace sgreval {

constexpr int kNNThreads = 256;
constexpr int kNNQ = 4;           // queries per thread
constexpr int kNNTile = 1024;     // reference points per shared-memory tile

__global__ void __launch_bounds__(kNNThreads) k_nn(const float* __restrict__ q, long long n,
                                                  const float* __restrict__ r, long long m,
                                                  float* __restrict__ dist, int* __restrict__ idx) {
  __shared__ float s_r[kNNTile * 3];
  float qx[kNNQ], qy[kNNQ], qz[kNNQ], best[kNNQ];
  int arg[kNNQ];
  const long long q0 = ((long long)blockIdx.x * kNNThreads + threadIdx.x) * kNNQ;
#pragma unroll
  for (int k = 0; k < kNNQ; ++k) {
    const long long i = q0 + k;
    qx[k] = i < n ? q[3 * i] : 0.f;
    qy[k] = i < n ? q[3 * i + 1] : 0.f;
    qz[k] = i < n ? q[3 * i + 2] : 0.f;
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
        const float dx = qx[k] - rx, dy = qy[k] - ry, dz = qz[k] - rz;
        const float d2 = dx * dx + dy * dy + dz * dz;
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
      dist[i] = sqrtf(best[k]);
      if (idx) idx[i] = arg[k];
    }
  }
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
  size_t tb = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tb, (const unsigned long long*)nullptr, (unsigned long long*)nullptr,
                                  (const int*)nullptr, (int*)nullptr, (int64_t)n, 0, 63);
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
  k_nn<<<(unsigned)blocks, kNNThreads, 0, static_cast<cudaStream_t>(stream)>>>(q, n, r, m, dist, idx);
  sgr::count_launches(1);
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
  size_t tb = L.temp_bytes;
  if (cub::DeviceRadixSort::SortPairs(sp + L.temp, tb, keys, keys_sorted, ids, ids_sorted, (int64_t)n, 0, 63, st) !=
      cudaSuccess)
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
