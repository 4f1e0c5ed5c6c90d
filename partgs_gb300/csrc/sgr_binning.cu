// Per-tile surfel lists by a stable counting sort over tiles.
//
// The reference emits one 64-bit key (tile << 32 | depth bits) per (surfel,
// tile) pair in surfel order and radix-sorts them (cuda_rasterizer/
// rasterizer_impl.cu:70-111, 288-318); a tile's list is then its surfels by
// (depth bits, index).  Here the records are already in (view, depth bits,
// index) order (the depth order of the geometry phase), so the same lists
// come from a stable distribution of that sequence into tiles, with no key
// array and no sort:
//
//  1. the depth-ordered records are cut into chunks of C (inside a view);
//     each chunk's per-tile counts come from a 2-D difference array of its
//     records' tile rectangles in shared memory (four updates per record);
//  2. per tile, an exclusive scan over the chunks gives each chunk's first
//     slot inside the tile's list, and the per-tile totals are scanned into
//     the tile ranges;
//  3. each chunk writes its records: every warp first counts its own slice
//     of the chunk per tile, the block turns the counts into per-warp bases,
//     then each warp walks its slice record by record (the lanes cover the
//     record's tiles, which are distinct) and places the record id at its
//     tile's next slot.
//
// The result is bit-identical to the sort: within a tile, records appear in
// chunk order, then warp order, then record order, i.e. depth order.
#include <cub/device/device_scan.cuh>

#include "sgr_kernels.cuh"

namespace sgr {

namespace {

constexpr int kRecsPerWarp = 256;

struct BinArgs {
  const uint32_t* depth_order;       // [R]
  const uint32_t* tiles_touched;     // [R]
  const int* radii;                  // [R]
  const float4* records;             // [R][kRecF4]
  const sgr_view_desc* views;        // [V]
  const sgr_scene_desc* scenes;
  uint32_t* chunk_offset;            // [V+1] first chunk of each view
  uint32_t* chunk_counts;            // [chunks][tpv] counts, then bases
  uint32_t* tile_count;              // [V*tpv]
  uint32_t* tile_start;              // [V*tpv]
  uint32_t* point_list;
  uint2* ranges;
  Status* status;
  long long capacity;
  int V, gx, gy, chunk;              // chunk = records per chunk
  int warps;                         // warps per chunk-writing CTA (chunk / kRecsPerWarp)
};

__device__ __forceinline__ int view_count(const BinArgs& a, int v) {
  return a.scenes[a.views[v].scene].surfel_count;
}

// (view, first record position, end position) of a global chunk; false past the last.
__device__ __forceinline__ bool chunk_span(const BinArgs& a, int c, int& v, int& p0, int& p1) {
  if ((uint32_t)c >= a.chunk_offset[a.V]) return false;
  int lo = 0, hi = a.V - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (a.chunk_offset[mid] <= (uint32_t)c) lo = mid; else hi = mid - 1;
  }
  v = lo;
  const int base = a.views[v].record_offset;
  const int cv = c - (int)a.chunk_offset[v];
  p0 = base + cv * a.chunk;
  p1 = min(base + view_count(a, v), p0 + a.chunk);
  return true;
}

__global__ void k_chunk_table(BinArgs a) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  uint32_t acc = 0;
  for (int v = 0; v < a.V; ++v) {
    a.chunk_offset[v] = acc;
    acc += (uint32_t)((view_count(a, v) + a.chunk - 1) / a.chunk);
  }
  a.chunk_offset[a.V] = acc;
}

// 1. per-chunk tile histogram via a 2-D difference array
__global__ void __launch_bounds__(256) k_chunk_hist(BinArgs a) {
  extern __shared__ int s_diff[];                  // [(gy + 1) * (gx + 1)]
  int v, p0, p1;
  if (!chunk_span(a, blockIdx.x, v, p0, p1)) return;
  const int W1 = a.gx + 1, H1 = a.gy + 1;
  for (int i = threadIdx.x; i < W1 * H1; i += blockDim.x) s_diff[i] = 0;
  __syncthreads();
  for (int p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
    const uint32_t r = a.depth_order[p];
    if (a.tiles_touched[r] == 0) continue;
    const float4 r2 = a.records[(size_t)r * kRecF4 + 2];
    int x0, y0, x1, y1;
    tile_rect(r2.y, r2.z, a.radii[r], a.gx, a.gy, x0, y0, x1, y1);
    atomicAdd(&s_diff[y0 * W1 + x0], 1);
    atomicAdd(&s_diff[y0 * W1 + x1], -1);
    atomicAdd(&s_diff[y1 * W1 + x0], -1);
    atomicAdd(&s_diff[y1 * W1 + x1], 1);
  }
  __syncthreads();
  for (int y = threadIdx.x; y < H1; y += blockDim.x) {       // prefix along x
    int run = 0;
    for (int x = 0; x < W1; ++x) {
      run += s_diff[y * W1 + x];
      s_diff[y * W1 + x] = run;
    }
  }
  __syncthreads();
  for (int x = threadIdx.x; x < W1; x += blockDim.x) {       // prefix along y
    int run = 0;
    for (int y = 0; y < H1; ++y) {
      run += s_diff[y * W1 + x];
      s_diff[y * W1 + x] = run;
    }
  }
  __syncthreads();
  const int tpv = a.gx * a.gy;
  uint32_t* out = a.chunk_counts + (size_t)blockIdx.x * tpv;
  for (int t = threadIdx.x; t < tpv; t += blockDim.x) {
    const int ty = t / a.gx, tx = t - ty * a.gx;
    out[t] = (uint32_t)s_diff[ty * W1 + tx];
  }
}

// 2a. per (view, tile): exclusive scan of the counts over the view's chunks
__global__ void k_chunk_scan(BinArgs a) {
  const int tpv = a.gx * a.gy;
  const long long gt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gt >= (long long)a.V * tpv) return;
  const int v = (int)(gt / tpv), t = (int)(gt - (long long)v * tpv);
  const uint32_t c0 = a.chunk_offset[v], c1 = a.chunk_offset[v + 1];
  uint32_t run = 0;
  for (uint32_t c = c0; c < c1; ++c) {
    uint32_t* cell = a.chunk_counts + (size_t)c * tpv + t;
    const uint32_t n = *cell;
    *cell = run;
    run += n;
  }
  a.tile_count[gt] = run;
}

// 2b. tile ranges from the scanned starts (clamped to the list capacity)
__global__ void k_tile_ranges_from_counts(BinArgs a) {
  const long long n = (long long)a.V * a.gx * a.gy;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const unsigned long long s = a.tile_start[t], e = s + a.tile_count[t];
  const unsigned long long cap = (unsigned long long)a.capacity;
  a.ranges[t] = make_uint2((uint32_t)min(s, cap), (uint32_t)min(e, cap));
  if (t == n - 1 && e > cap) atomicOr(&a.status->flags, SGR_FLAG_KEY_OVERFLOW);
}

// 3. stable scatter of each chunk's records into the tile lists
__global__ void __launch_bounds__(256) k_chunk_write(BinArgs a) {
  extern __shared__ uint32_t s_cnt[];              // [warps][tpv]
  int v, p0, p1;
  if (!chunk_span(a, blockIdx.x, v, p0, p1)) return;
  const int tpv = a.gx * a.gy;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint32_t* cnt = s_cnt + (size_t)warp * tpv;
  for (int i = threadIdx.x; i < a.warps * tpv; i += blockDim.x) s_cnt[i] = 0;
  __syncthreads();
  const int w0 = p0 + warp * kRecsPerWarp, w1 = min(p1, w0 + kRecsPerWarp);

  // walks this warp's records in order; for each, the lanes cover its tiles
  auto walk = [&](bool place) {
    for (int g = w0; g < w1; g += 32) {
      const int p = g + lane;
      uint32_t r = 0xffffffffu;
      int x0 = 0, y0 = 0, x1 = 0, y1 = 0;
      if (p < w1) {
        r = a.depth_order[p];
        if (a.tiles_touched[r] != 0) {
          const float4 r2 = a.records[(size_t)r * kRecF4 + 2];
          tile_rect(r2.y, r2.z, a.radii[r], a.gx, a.gy, x0, y0, x1, y1);
        }
      }
      const int m = min(32, w1 - g);
      for (int k = 0; k < m; ++k) {
        const uint32_t rk = __shfl_sync(0xffffffffu, r, k);
        const int ax = __shfl_sync(0xffffffffu, x0, k), ay = __shfl_sync(0xffffffffu, y0, k);
        const int bx = __shfl_sync(0xffffffffu, x1, k), by = __shfl_sync(0xffffffffu, y1, k);
        const int w = bx - ax, n = w * (by - ay);
        for (int q = lane; q < n; q += 32) {
          const int ty = ay + q / w, tx = ax + q - (q / w) * w;
          const int t = ty * a.gx + tx;
          if (!place) {
            cnt[t] += 1;
          } else {
            const uint32_t pos = cnt[t]++;
            if ((long long)pos < a.capacity) a.point_list[pos] = rk;
          }
        }
        __syncwarp();
      }
    }
  };
  walk(false);
  __syncthreads();
  const uint32_t* cbase = a.chunk_counts + (size_t)blockIdx.x * tpv;
  const uint32_t* tstart = a.tile_start + (size_t)v * tpv;
  for (int t = threadIdx.x; t < tpv; t += blockDim.x) {
    uint32_t run = tstart[t] + cbase[t];
    for (int w = 0; w < a.warps; ++w) {
      const uint32_t n = s_cnt[(size_t)w * tpv + t];
      s_cnt[(size_t)w * tpv + t] = run;
      run += n;
    }
  }
  __syncthreads();
  walk(true);
}

}  // namespace

// Layout of the binning scratch for R records, V views and a tpv-tile grid.
size_t binning_scratch_bytes(long long R, int V, int gx, int gy, int* chunk_out, int* warps_out,
                             size_t* off_counts, size_t* off_tiles, size_t* off_temp, size_t* temp_bytes) {
  const int tpv = gx * gy;
  // per-warp counters of the chunk-writing CTA must fit in shared memory
  int warps = (int)std::min<long long>(8, (200 * 1024) / (4LL * std::max(1, tpv)));
  if (warps < 1) return 0;
  const int chunk = warps * kRecsPerWarp;
  const long long chunks = (R + chunk - 1) / chunk + V;
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  size_t o = 0;
  const size_t off_table = o;
  (void)off_table;
  o = al(o + (size_t)(V + 1) * 4);
  *off_counts = o;
  o = al(o + (size_t)chunks * tpv * 4);
  *off_tiles = o;                       // tile_count then tile_start
  o = al(o + (size_t)2 * V * tpv * 4);
  size_t tb = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tb, (uint32_t*)nullptr, (uint32_t*)nullptr, (int64_t)V * tpv);
  *off_temp = o;
  *temp_bytes = tb;
  o = al(o + tb);
  *chunk_out = chunk;
  *warps_out = warps;
  return o;
}

int launch_binning(const sgr_batch& b, const GeomView& g, uint32_t* point_list, long long capacity, void* scratch,
                   cudaStream_t st) {
  int chunk, warps;
  size_t off_counts, off_tiles, off_temp, temp_bytes;
  const size_t need = binning_scratch_bytes(b.num_records, b.num_views, g.tiles_x, g.tiles_y, &chunk, &warps,
                                            &off_counts, &off_tiles, &off_temp, &temp_bytes);
  if (need == 0) return SGR_ERR_UNSUPPORTED;
  char* sp = static_cast<char*>(scratch);
  const int tpv = g.tiles_x * g.tiles_y;
  BinArgs a;
  a.depth_order = g.depth_order;
  a.tiles_touched = g.tiles_touched;
  a.radii = g.radii;
  a.records = g.records;
  a.views = b.views;
  a.scenes = b.scenes;
  a.chunk_offset = reinterpret_cast<uint32_t*>(sp);
  a.chunk_counts = reinterpret_cast<uint32_t*>(sp + off_counts);
  a.tile_count = reinterpret_cast<uint32_t*>(sp + off_tiles);
  a.tile_start = a.tile_count + (size_t)b.num_views * tpv;
  a.point_list = point_list;
  a.ranges = g.ranges;
  a.status = g.status;
  a.capacity = capacity;
  a.V = b.num_views;
  a.gx = g.tiles_x;
  a.gy = g.tiles_y;
  a.chunk = chunk;
  a.warps = warps;
  const long long max_chunks = ((long long)b.num_records + chunk - 1) / chunk + b.num_views;
  k_chunk_table<<<1, 32, 0, st>>>(a);
  const size_t hist_smem = (size_t)(g.tiles_x + 1) * (g.tiles_y + 1) * 4;
  const size_t write_smem = (size_t)warps * tpv * 4;
  if (hist_smem > 220 * 1024) return SGR_ERR_UNSUPPORTED;
  // per-function attributes apply to the current device; set them every call
  if (cudaFuncSetAttribute(k_chunk_hist, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024) != cudaSuccess ||
      cudaFuncSetAttribute(k_chunk_write, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024) != cudaSuccess)
    return SGR_ERR_CUDA;
  k_chunk_hist<<<(unsigned)max_chunks, 256, hist_smem, st>>>(a);
  const long long ntiles = (long long)b.num_views * tpv;
  k_chunk_scan<<<(unsigned)((ntiles + 255) / 256), 256, 0, st>>>(a);
  size_t tb = temp_bytes;
  if (cub::DeviceScan::ExclusiveSum(sp + off_temp, tb, a.tile_count, a.tile_start, (int64_t)ntiles, st) != cudaSuccess)
    return SGR_ERR_CUDA;
  k_tile_ranges_from_counts<<<(unsigned)((ntiles + 255) / 256), 256, 0, st>>>(a);
  k_chunk_write<<<(unsigned)max_chunks, warps * 32, write_smem, st>>>(a);
  return cudaGetLastError() == cudaSuccess ? SGR_OK : SGR_ERR_CUDA;
}

}  // namespace sgr
