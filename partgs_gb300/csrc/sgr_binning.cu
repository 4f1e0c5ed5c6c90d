// Cell lists: the records of each view binned into square cells of B x B
// tiles (the batch's cell_tiles), each cell's list in depth order.
//
// The reference emits one 64-bit key (tile << 32 | depth bits) per (surfel,
// tile) pair in surfel order and radix-sorts them (cuda_rasterizer/
// rasterizer_impl.cu:70-111, 288-318); a tile's list is then its surfels by
// (depth bits, index).  Here the records are already in (view, depth bits,
// index) order after the geometry phase, so a tile's list is the
// subsequence of that order whose tile rectangle holds the tile, and any
// depth-ordered superset of it can stand in for it: a blend CTA streams its
// cell's list and keeps the entries whose rectangle holds its tile
// (sgr_blend.cu).  A record touches ~4 cells instead of ~60 tiles, so the
// lists are a small fraction of the reference's keys, and front-to-back
// termination means a tile reads only a short prefix of its cell's list.
//
// Construction, a stable counting sort over cells with no sort and no keys:
//  0. (geometry phase) each record's tile rectangle is gathered into depth
//     order, 8 bytes per record, and the (record, cell) pairs are counted
//     (k_gather_rects);
//  1. the depth-ordered records of a view are cut into chunks of kChunk;
//     each chunk's per-cell counts come from a 2-D difference array of its
//     records' cell rectangles in shared memory (four updates per record);
//  2. per cell, an exclusive scan over the view's chunks gives each chunk's
//     first position in the cell's list and the cell's total; the totals are
//     scanned into each cell's start in one concatenated array;
//  3. per chunk, every warp counts its own slice of records per cell (a
//     2-D difference array of the slice's cell rectangles in shared memory,
//     then prefix sums along x and y), the block turns the counts into
//     per-warp bases, then each warp walks its slice record by record (the
//     lanes cover the record's cells, which are distinct) and writes the
//     entry at its cell's next slot.  Within a cell, entries come in chunk
//     order, then warp order, then record order: depth order.
// Cell-list entries are depth-order positions (the blend reads the
// rectangle and the record id from them).
//
// With one-tile cells and record ids as entries, the same kernels write the
// reference's exact per-tile lists and [start, end) ranges; that form is
// kept for inspection and tests (sgr_tile_lists).

#include "sgr_kernels.cuh"

namespace sgr {

namespace {

struct CellArgs {
  const uint32_t* depth_order;       // [R]
  const uint2* rects;                // [R] packed tile rectangles, depth order
  const sgr_view_desc* views;        // [V]
  const sgr_scene_desc* scenes;
  uint32_t* chunk_offset;            // [V+1] first chunk of each view
  uint32_t* chunk_base;              // [chunks][cells per view] counts, then list positions
  uint32_t* cell_count;              // [V*cells]
  uint32_t* cell_start;              // [V*cells] exclusive scan of cell_count
  uint32_t* out;                     // the lists
  uint2* ranges;                     // [V*cells] [start, end) clamped to the capacity, or null
  Status* status;
  long long capacity;                // entries `out` holds
  unsigned int overflow_flag;        // status flag raised when the lists exceed the capacity
  int V;
  int B;                             // cell edge in tiles (a power of two)
  int lb;                            // log2(B)
  int cx, cy;                        // cells per view along x and y
  int warps;                         // warps of the list-writing CTA
  int stage;                         // entries a list-writing CTA can stage in shared memory
  bool ids;                          // write record ids (else depth-order positions)
};

__device__ __forceinline__ int view_count(const CellArgs& a, int v) {
  return a.scenes[a.views[v].scene].surfel_count;
}

// (view, first depth-order position, end position) of a global chunk; false past the last.
__device__ __forceinline__ bool chunk_span(const CellArgs& a, int c, int& v, int& p0, int& p1) {
  if ((uint32_t)c >= a.chunk_offset[a.V]) return false;
  int lo = 0, hi = a.V - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (a.chunk_offset[mid] <= (uint32_t)c) lo = mid; else hi = mid - 1;
  }
  v = lo;
  const int base = a.views[v].record_offset;
  p0 = base + (c - (int)a.chunk_offset[v]) * kChunk;
  p1 = min(base + view_count(a, v), p0 + kChunk);
  return true;
}

// Cell rectangle [x0, x1) x [y0, y1) of a packed tile rectangle, for cells
// of 2^lb tiles; empty for an empty one.
__device__ __forceinline__ void cell_rect(uint2 r, int lb, int& x0, int& y0, int& x1, int& y1) {
  unpack_rect(r, x0, y0, x1, y1);
  if (x0 >= x1 || y0 >= y1) {
    x0 = y0 = x1 = y1 = 0;
    return;
  }
  const int m = (1 << lb) - 1;
  x0 >>= lb;
  y0 >>= lb;
  x1 = (x1 + m) >> lb;
  y1 = (y1 + m) >> lb;
}

__host__ __device__ __forceinline__ int log2_of(int B) { return B >= 16 ? 4 : B >= 8 ? 3 : B >= 4 ? 2 : B >= 2 ? 1 : 0; }

// 0. tile rectangles and key counts in depth order; (record, cell) pair count
__global__ void __launch_bounds__(256) k_gather_rects(const uint32_t* __restrict__ order,
                                                      const uint32_t* __restrict__ touched,
                                                      const float4* __restrict__ records,
                                                      const int* __restrict__ radii,
                                                      unsigned long long* __restrict__ counts,
                                                      uint2* __restrict__ rects, Status* status, long long R,
                                                      int gx, int gy, int B) {
  __shared__ unsigned long long s_sum[8];
  const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned int cells = 0;
  if (j < R) {
    const uint32_t r = order[j];
    const uint32_t n = touched[r];
    counts[j] = n;
    uint2 out = make_uint2(0u, 0u);
    if (n != 0) {
      const float4 r2 = records[(size_t)r * kRecF4 + 2];
      int x0, y0, x1, y1;
      tile_rect(r2.y, r2.z, radii[r], gx, gy, x0, y0, x1, y1);
      out = pack_rect(x0, y0, x1, y1);
      int cx0, cy0, cx1, cy1;
      cell_rect(out, log2_of(B), cx0, cy0, cx1, cy1);
      cells = (unsigned int)((cx1 - cx0) * (cy1 - cy0));
    }
    rects[j] = out;
  }
  unsigned long long sum = cells;
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if ((threadIdx.x & 31) == 0) s_sum[threadIdx.x >> 5] = sum;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_sum[w];
    if (t) atomicAdd(&status->num_bin_entries, t);
  }
}

__global__ void k_chunk_table(CellArgs a) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  uint32_t acc = 0;
  for (int v = 0; v < a.V; ++v) {
    a.chunk_offset[v] = acc;
    acc += (uint32_t)((view_count(a, v) + kChunk - 1) / kChunk);
  }
  a.chunk_offset[a.V] = acc;
}

// 1. per-chunk cell histogram via a 2-D difference array
__global__ void __launch_bounds__(256) k_cell_hist(CellArgs a) {
  extern __shared__ int s_diff[];                  // [(cy + 1) * (cx + 1)]
  int v, p0, p1;
  if (!chunk_span(a, blockIdx.x, v, p0, p1)) return;
  const int W1 = a.cx + 1, H1 = a.cy + 1;
  for (int i = threadIdx.x; i < W1 * H1; i += blockDim.x) s_diff[i] = 0;
  __syncthreads();
  for (int p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
    int x0, y0, x1, y1;
    cell_rect(a.rects[p], a.lb, x0, y0, x1, y1);
    if (x0 >= x1) continue;
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
  const int ncell = a.cx * a.cy;
  uint32_t* out = a.chunk_base + (size_t)blockIdx.x * ncell;
  for (int t = threadIdx.x; t < ncell; t += blockDim.x) {
    const int ty = t / a.cx, tx = t - ty * a.cx;
    out[t] = (uint32_t)s_diff[ty * W1 + tx];
  }
}

// 2a. per (view, cell): exclusive scan of the counts over the view's chunks
__global__ void k_cell_scan(CellArgs a) {
  const int ncell = a.cx * a.cy;
  const long long gt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gt >= (long long)a.V * ncell) return;
  const int v = (int)(gt / ncell), t = (int)(gt - (long long)v * ncell);
  const uint32_t c0 = a.chunk_offset[v], c1 = a.chunk_offset[v + 1];
  uint32_t run = 0;
  constexpr int kStep = 8;                         // loads in flight per thread
  for (uint32_t c = c0; c < c1; c += kStep) {
    uint32_t n[kStep];
#pragma unroll
    for (int k = 0; k < kStep; ++k) n[k] = (c + k < c1) ? a.chunk_base[(size_t)(c + k) * ncell + t] : 0u;
#pragma unroll
    for (int k = 0; k < kStep; ++k) {
      if (c + k < c1) a.chunk_base[(size_t)(c + k) * ncell + t] = run;
      run += n[k];
    }
  }
  a.cell_count[gt] = run;
}

// 2b. ranges (when asked for) and the capacity check
__global__ void k_cell_ranges(CellArgs a) {
  const long long n = (long long)a.V * a.cx * a.cy;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const unsigned long long s = a.cell_start[t], e = s + a.cell_count[t];
  const unsigned long long cap = (unsigned long long)a.capacity;
  if (a.ranges) a.ranges[t] = make_uint2((uint32_t)min(s, cap), (uint32_t)min(e, cap));
  // the 32-bit scan wraps past 2^32 entries: also test the exact 64-bit total
  // the geometry phase counted
  if (t == n - 1) {
    const unsigned long long total =
        a.overflow_flag == SGR_FLAG_KEY_OVERFLOW ? a.status->num_keys : a.status->num_bin_entries;
    if (e > cap || total > cap) atomicOr(&a.status->flags, a.overflow_flag);
  }
}

// 3. stable scatter of each chunk's records into the cell lists
__global__ void __launch_bounds__(256) k_cell_write(CellArgs a) {
  // [warps][cells per view] positions, then [cells + 1] chunk-run starts,
  // [cells] list positions of those runs, then the staging area
  extern __shared__ uint32_t s_cnt[];
  int v, p0, p1;
  if (!chunk_span(a, blockIdx.x, v, p0, p1)) return;
  const int ncell = a.cx * a.cy;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint32_t* cnt = s_cnt + (size_t)warp * ncell;
  for (int i = threadIdx.x; i < a.warps * ncell; i += blockDim.x) s_cnt[i] = 0;
  __syncthreads();
  const int per_warp = kChunk / a.warps;
  const int w0 = p0 + warp * per_warp, w1 = min(p1, w0 + per_warp);
  const int cx = a.cx, cy = a.cy;

  // this warp's count per cell: difference array of its records' cell
  // rectangles (updates past the last column or row have no effect inside
  // the grid and are dropped), then prefix sums along x and along y
  for (int p = w0 + lane; p < w1; p += 32) {
    int x0, y0, x1, y1;
    cell_rect(a.rects[p], a.lb, x0, y0, x1, y1);
    if (x0 >= x1) continue;
    atomicAdd(&cnt[y0 * cx + x0], 1u);
    if (x1 < cx) atomicAdd(&cnt[y0 * cx + x1], 0xffffffffu);
    if (y1 < cy) {
      atomicAdd(&cnt[y1 * cx + x0], 0xffffffffu);
      if (x1 < cx) atomicAdd(&cnt[y1 * cx + x1], 1u);
    }
  }
  __syncwarp();
  for (int y = lane; y < cy; y += 32) {
    uint32_t run = 0;
    for (int x = 0; x < cx; ++x) {
      run += cnt[y * cx + x];
      cnt[y * cx + x] = run;
    }
  }
  __syncwarp();
  for (int x = lane; x < cx; x += 32) {
    uint32_t run = 0;
    for (int y = 0; y < cy; ++y) {
      run += cnt[y * cx + x];
      cnt[y * cx + x] = run;
    }
  }
  __syncthreads();
  const uint32_t* cbase = a.chunk_base + (size_t)blockIdx.x * ncell;
  const uint32_t* cstart = a.cell_start + (size_t)v * ncell;
  uint32_t* s_run = s_cnt + (size_t)a.warps * ncell;      // [ncell + 1]: this chunk's run starts, staged order
  uint32_t* s_dst = s_run + ncell + 1;                    // [ncell]: where each run goes in the lists
  uint32_t* s_stage = s_dst + ncell;                      // [a.stage]
  __shared__ uint32_t s_part[8];
  // Each cell's entries from this chunk form one run in the cell's list.
  // When the chunk's entries fit the staging area, they are placed there
  // (cell-major) and each run is then written out contiguously; otherwise
  // straight into the lists.  Runs: exclusive scan of the chunk's per-cell
  // counts, each thread a contiguous range of cells.
  const int per_t = (ncell + blockDim.x - 1) / blockDim.x;
  const int c0 = min(ncell, (int)threadIdx.x * per_t), c1 = min(ncell, c0 + per_t);
  uint32_t mine = 0;
  for (int t = c0; t < c1; ++t)
    for (int w = 0; w < a.warps; ++w) mine += s_cnt[(size_t)w * ncell + t];
  uint32_t incl = mine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) s_part[warp] = incl;
  __syncthreads();
  uint32_t before = 0, total = 0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
    if (w < warp) before += s_part[w];
    total += s_part[w];
  }
  const bool staged = total <= (uint32_t)a.stage;                 // CTA-uniform
  uint32_t run = before + incl - mine;
  for (int t = c0; t < c1; ++t) {
    s_run[t] = run;
    s_dst[t] = cstart[t] + cbase[t];
    uint32_t at = staged ? run : cstart[t] + cbase[t];
    for (int w = 0; w < a.warps; ++w) {
      const uint32_t n = s_cnt[(size_t)w * ncell + t];
      s_cnt[(size_t)w * ncell + t] = at;
      at += n;
      run += n;
    }
  }
  if (threadIdx.x == 0) s_run[ncell] = total;
  __syncthreads();
  // walk this warp's records in order; for each, the lanes cover its cells
  for (int g = w0; g < w1; g += 32) {
    const int p = g + lane;
    uint2 r = make_uint2(0u, 0u);
    uint32_t e = 0;
    if (p < w1) {
      r = a.rects[p];
      e = a.ids ? a.depth_order[p] : (uint32_t)p;
    }
    const int m = min(32, w1 - g);
    for (int k = 0; k < m; ++k) {
      const uint32_t ek = __shfl_sync(0xffffffffu, e, k);
      uint2 rk;
      rk.x = __shfl_sync(0xffffffffu, r.x, k);
      rk.y = __shfl_sync(0xffffffffu, r.y, k);
      int ax, ay, bx, by;
      cell_rect(rk, a.lb, ax, ay, bx, by);
      const int w = bx - ax, n = w * (by - ay);
      for (int q = lane; q < n; q += 32) {
        const int qy = q / w;
        const int t = (ay + qy) * cx + ax + (q - qy * w);
        const uint32_t pos = cnt[t]++;
        if (staged) s_stage[pos] = ek;
        else if ((long long)pos < a.capacity) a.out[pos] = ek;
      }
      __syncwarp();
    }
  }
  if (!staged) return;                               // CTA-uniform
  __syncthreads();
  // each warp writes whole runs, lanes over consecutive entries
  for (int t = warp; t < ncell; t += blockDim.x >> 5) {
    const uint32_t r0 = s_run[t], n = s_run[t + 1] - r0, d = s_dst[t];
    for (uint32_t k = lane; k < n; k += 32)
      if ((long long)(d + k) < a.capacity) a.out[d + k] = s_stage[r0 + k];
  }
}

constexpr size_t kMaxDynSmem = 220 * 1024;
constexpr size_t kAlignB = 256;
size_t al(size_t x) { return (x + kAlignB - 1) & ~(kAlignB - 1); }

// Staging area of the list writer, in entries (6,144: 24 KB), less where
// the per-warp counts leave less room.
#ifndef SGR_CELL_STAGE
#define SGR_CELL_STAGE 6144
#endif
constexpr long long kStageEntries = SGR_CELL_STAGE;

size_t writer_smem(int warps, int ncell, int stage) {
  return ((size_t)warps * ncell + 2 * (size_t)ncell + 1 + (size_t)stage) * 4;
}

int writer_stage(int warps, int ncell) {
  const long long room = (long long)(kMaxDynSmem / 4) - (long long)warps * ncell - 2LL * ncell - 1;
  return (int)std::max(0LL, std::min(kStageEntries, room));
}

int writer_warps(int ncell) {
  // per-warp counts, plus the run starts and destinations, within 200 KB
  const long long fit = ((long long)(200 * 1024) / 4 - 2LL * ncell - 1) / std::max(1, ncell);
  return fit >= 8 ? 8 : fit >= 4 ? 4 : fit >= 2 ? 2 : fit >= 1 ? 1 : 0;
}

// Scratch of one cell-list construction: chunk table, per-chunk bases, and
// (when the counts and starts are not given) counts, starts, and the scan's
// temporary storage.
struct CellScratch {
  size_t chunk_offset, chunk_base, count, start, temp, temp_bytes, end;
};

CellScratch cell_scratch(long long R, int V, int ncell, bool own_counts) {
  CellScratch s;
  const long long chunks = (R + kChunk - 1) / kChunk + V;
  const size_t cells = (size_t)V * ncell;
  size_t o = 0;
  s.chunk_offset = o; o = al(o + (size_t)(V + 1) * 4);
  s.chunk_base = o; o = al(o + (size_t)chunks * ncell * 4);
  s.count = s.start = 0;
  if (own_counts) {
    s.count = o; o = al(o + cells * 4);
    s.start = o; o = al(o + cells * 4);
  }
  const size_t tb = scan_temp_bytes<uint32_t>((long long)cells);
  s.temp = o;
  s.temp_bytes = tb;
  o = al(o + tb);
  s.end = o;
  return s;
}

int run_cells(const sgr_batch& b, const GeomView& g, int B, bool ids, uint32_t* out, long long capacity,
              unsigned int overflow_flag, uint32_t* count, uint32_t* start, uint2* ranges, void* scratch,
              cudaStream_t st) {
  const int cx = (g.tiles_x + B - 1) / B, cy = (g.tiles_y + B - 1) / B;
  const int ncell = cx * cy;
  const size_t hist_smem = (size_t)(cx + 1) * (cy + 1) * 4;
  const int warps = writer_warps(ncell);
  if (hist_smem > kMaxDynSmem || warps == 0) return SGR_ERR_UNSUPPORTED;
  const CellScratch L = cell_scratch(b.num_records, b.num_views, ncell, count == nullptr);
  char* sp = static_cast<char*>(scratch);
  CellArgs a;
  a.depth_order = g.depth_order;
  a.rects = g.rects;
  a.views = b.views;
  a.scenes = b.scenes;
  a.chunk_offset = reinterpret_cast<uint32_t*>(sp + L.chunk_offset);
  a.chunk_base = reinterpret_cast<uint32_t*>(sp + L.chunk_base);
  a.cell_count = count ? count : reinterpret_cast<uint32_t*>(sp + L.count);
  a.cell_start = start ? start : reinterpret_cast<uint32_t*>(sp + L.start);
  a.out = out;
  a.ranges = ranges;
  a.status = g.status;
  a.capacity = capacity;
  a.overflow_flag = overflow_flag;
  a.V = b.num_views;
  a.B = B;
  a.lb = log2_of(B);
  a.cx = cx;
  a.cy = cy;
  a.warps = warps;
  a.stage = writer_stage(warps, ncell);
  a.ids = ids;
  const long long chunks = (b.num_records + kChunk - 1) / kChunk + b.num_views;
  const long long ncells = (long long)b.num_views * ncell;
  k_chunk_table<<<1, 32, 0, st>>>(a);
  count_launches();
  // per-function attributes apply to the current device; set them every call
  if (cudaFuncSetAttribute(k_cell_hist, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxDynSmem) != cudaSuccess ||
      cudaFuncSetAttribute(k_cell_write, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxDynSmem) != cudaSuccess)
    return SGR_ERR_CUDA;
  k_cell_hist<<<(unsigned)chunks, 256, hist_smem, st>>>(a);
  count_launches();
  k_cell_scan<<<(unsigned)((ncells + 255) / 256), 256, 0, st>>>(a);
  count_launches();
  if (prefix_sum<uint32_t, false>(a.cell_count, a.cell_start, ncells, sp + L.temp, L.temp_bytes, st) != SGR_OK)
    return SGR_ERR_CUDA;
  k_cell_ranges<<<(unsigned)((ncells + 255) / 256), 256, 0, st>>>(a);
  count_launches();
  k_cell_write<<<(unsigned)chunks, warps * 32, writer_smem(warps, ncell, a.stage), st>>>(a);
  count_launches();
  return cudaGetLastError() == cudaSuccess ? SGR_OK : SGR_ERR_CUDA;
}

}  // namespace

bool binning_supported(int gx, int gy, int B) {
  if (B != 1 && B != 2 && B != 4 && B != 8 && B != 16) return false;
  const int cx = bin_cells(gx, B), cy = bin_cells(gy, B);
  return gx < 65536 && gy < 65536 && (size_t)(cx + 1) * (cy + 1) * 4 <= kMaxDynSmem && writer_warps(cx * cy) > 0;
}

size_t bin_scratch_bytes(long long R, int V, int gx, int gy, int B) {
  return cell_scratch(R, V, bin_cells(gx, B) * bin_cells(gy, B), false).end;
}

size_t tile_list_scratch_bytes(long long R, int V, int gx, int gy) {
  return cell_scratch(R, V, gx * gy, true).end;
}

void launch_gather_rects(const GeomView& g, long long R, cudaStream_t st) {
  k_gather_rects<<<(unsigned)((R + 255) / 256), 256, 0, st>>>(g.depth_order, g.tiles_touched, g.records, g.radii,
                                                               g.offsets, g.rects, g.status, R, g.tiles_x, g.tiles_y,
                                                               g.cell_tiles);
  count_launches();
}

int launch_binning(const sgr_batch& b, const GeomView& g, void* scratch, cudaStream_t st) {
  return run_cells(b, g, g.cell_tiles, false, const_cast<uint32_t*>(g.bins), g.bin_capacity, SGR_FLAG_BIN_OVERFLOW,
                   g.bin_count, g.bin_start, nullptr, scratch, st);
}

int launch_tile_lists(const sgr_batch& b, const GeomView& g, uint32_t* lists, long long capacity, void* scratch,
                      cudaStream_t st) {
  return run_cells(b, g, 1, true, lists, capacity, SGR_FLAG_KEY_OVERFLOW, nullptr, nullptr, g.ranges, scratch, st);
}

}  // namespace sgr
