// C ABI of the surfel rasteriser: argument checks, workspace layout and the
// launch sequence of each phase.

#include <atomic>
#include <cstdio>
#include <cstring>
#include <string>

#include "sgr_kernels.cuh"
#include "sgr_profile.cuh"

namespace sgr {
namespace {

thread_local std::string g_last_error;
std::atomic<unsigned long long> g_launches{0};

int cuda_fail(cudaError_t e, const char* what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  return SGR_ERR_CUDA;
}

#define SGR_CUDA(call)                                  \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

constexpr size_t kAlign = 256;
size_t align_up(size_t x) { return (x + kAlign - 1) & ~(kAlign - 1); }

int bit_length(unsigned long long n) {
  int b = 0;
  while (n) {
    ++b;
    n >>= 1;
  }
  return b;
}

// Byte layout of the forward scratch.
struct ScratchLayout {
  size_t depth_keys, depth_vals, depth_keys_sorted, temp_a, temp_a_bytes;
  size_t bin;          // list-index scratch (sgr_binning.cu)
  size_t end_a, end;
};

int check_batch(const sgr_batch* b) {
  if (!b) return SGR_ERR_INVALID_ARGUMENT;
  if (b->variant != SGR_VARIANT_PLAIN && b->variant != SGR_VARIANT_PART) return SGR_ERR_INVALID_ARGUMENT;
  if (b->num_scenes < 1 || b->num_views < 1 || b->height < 1 || b->width < 1) return SGR_ERR_INVALID_ARGUMENT;
  if (b->num_surfels < 0 || b->num_records < 0) return SGR_ERR_INVALID_ARGUMENT;
  if (b->semantic_channels < 0) return SGR_ERR_INVALID_ARGUMENT;
  if (b->cell_tiles != 0 && b->cell_tiles != 1 && b->cell_tiles != 2 && b->cell_tiles != 4 && b->cell_tiles != 8 &&
      b->cell_tiles != 16)
    return SGR_ERR_INVALID_ARGUMENT;
  if (b->semantic_channels > SGR_MAX_SEMANTICS) return SGR_ERR_SEMANTIC_CHANNELS;
  if (b->variant == SGR_VARIANT_PLAIN && b->semantic_channels != 0) return SGR_ERR_INVALID_ARGUMENT;
  if (b->blend_shape != SGR_BLEND_STRIP16 && b->blend_shape != SGR_BLEND_PATCH8) return SGR_ERR_INVALID_ARGUMENT;
  if (b->tile_schedule != SGR_SCHEDULE_GRID && b->tile_schedule != SGR_SCHEDULE_QUEUE) return SGR_ERR_INVALID_ARGUMENT;
  if (b->stage_entries != 0 && b->stage_entries != SGR_STAGE_DEFAULT && b->stage_entries != SGR_STAGE_SMALL &&
      b->stage_entries != SGR_STAGE_TINY)
    return SGR_ERR_INVALID_ARGUMENT;
  if (!b->scenes || !b->views || !b->viewmatrix || !b->projmatrix || !b->campos || !b->background)
    return SGR_ERR_INVALID_ARGUMENT;
  if (b->num_surfels > 0) {
    if (!b->means3D || !b->opacities) return SGR_ERR_INVALID_ARGUMENT;
    if ((b->shs == nullptr) == (b->colors_precomp == nullptr)) return SGR_ERR_INVALID_ARGUMENT;
    if (b->transmat_precomp == nullptr && (!b->scales || !b->rotations)) return SGR_ERR_INVALID_ARGUMENT;
    if (b->transmat_precomp != nullptr && b->num_views != 1) return SGR_ERR_UNSUPPORTED;
    if (b->shs != nullptr && (b->sh_coeffs < 1 || b->sh_coeffs > kMaxShCoeffs)) return SGR_ERR_UNSUPPORTED;
    if (b->shs != nullptr && (b->sh_degree < 0 || b->sh_degree > 3 || (b->sh_degree + 1) * (b->sh_degree + 1) > b->sh_coeffs))
      return SGR_ERR_UNSUPPORTED;
    if (b->semantic_channels > 0 && !b->semantics) return SGR_ERR_INVALID_ARGUMENT;
    if ((size_t)reinterpret_cast<uintptr_t>(b->rotations) % 16 != 0) return SGR_ERR_INVALID_ARGUMENT;
  }
  return SGR_OK;
}

void tile_grid(const sgr_batch* b, int& gx, int& gy) {
  gx = (b->width + kTile - 1) / kTile;
  gy = (b->height + kTile - 1) / kTile;
}

int tile_key_bits(const sgr_batch* b) {
  int gx, gy;
  tile_grid(b, gx, gy);
  return bit_length((unsigned long long)gx * gy * b->num_views);
}

int depth_key_bits(const sgr_batch* b) { return 32 + bit_length((unsigned long long)(b->num_views - 1)); }

int scratch_layout(const sgr_batch* b, long long cap, ScratchLayout& L) {
  const size_t R = (size_t)b->num_records;
  size_t o = 0;
  L.depth_keys = o; o = align_up(o + R * 8);
  L.depth_vals = o; o = align_up(o + R * 4);
  L.depth_keys_sorted = o; o = align_up(o + R * 8);
  const size_t sort_a = radix_sort_temp_bytes<unsigned long long>((long long)R);
  const size_t scan_a = scan_temp_bytes<unsigned long long>((long long)R);
  L.temp_a = o;
  L.temp_a_bytes = std::max(sort_a, scan_a);
  o = align_up(o + L.temp_a_bytes);
  L.end_a = o;
  (void)cap;
  int gx, gy;
  tile_grid(b, gx, gy);
  const int B = cell_tiles_of(*b);
  if (!binning_supported(gx, gy, B)) return SGR_ERR_UNSUPPORTED;   // cell size, or a grid too large for it
  const size_t bin = bin_scratch_bytes((long long)R, b->num_views, gx, gy, B);
  L.bin = o;
  o = align_up(o + bin);
  L.end = o;
  return SGR_OK;
}

int sizes_impl(const sgr_batch* b, long long cap, sgr_sizes* s) {
  int gx, gy;
  tile_grid(b, gx, gy);
  const size_t R = (size_t)b->num_records;
  const size_t V = (size_t)b->num_views;
  const size_t HW = (size_t)b->height * b->width;
  size_t o = 0;
  s->off_records = o; o = align_up(o + R * kRecF4 * 16);
  s->off_radii = o; o = align_up(o + R * 4);
  s->off_tiles_touched = o; o = align_up(o + R * 4);
  s->off_depth_order = o; o = align_up(o + R * 4);
  s->off_offsets = o; o = align_up(o + R * 8);
  s->off_ranges = o; o = align_up(o + V * gx * gy * 8);
  s->off_final_T = o; o = align_up(o + V * 3 * HW * 4);
  s->off_n_contrib = o; o = align_up(o + V * 2 * HW * 4);
  s->off_status = o; o = align_up(o + sizeof(Status));
  s->off_rects = o; o = align_up(o + R * 8);
  const int B = cell_tiles_of(*b);
  const size_t cells = V * (size_t)bin_cells(gx, B) * bin_cells(gy, B);
  s->off_bin_start = o; o = align_up(o + cells * 4);
  s->off_bin_count = o; o = align_up(o + cells * 4);
  s->off_tile_resume = o; o = align_up(o + V * gx * gy * 8);
  s->off_tile_queue = o; o = align_up(o + (V * gx * gy + 1) * 4);
  s->cell_tiles = B;
  s->geom_bytes = o;
  s->list_bytes = align_up((size_t)std::max(0LL, cap) * 4);
  ScratchLayout L;
  int rc = scratch_layout(b, cap, L);
  if (rc) return rc;
  s->fwd_scratch_bytes = L.end;
  s->bwd_scratch_bytes = align_up(R * kGradF * 4);
  s->tile_list_scratch_bytes = tile_list_scratch_bytes((long long)R, (int)V, gx, gy);
  s->tiles_x = gx;
  s->tiles_y = gy;
  s->tile_key_bits = tile_key_bits(b);
  return SGR_OK;
}

GeomView geom_view(const sgr_batch* b, const sgr_sizes& s, void* geom, void* scratch, const ScratchLayout* L) {
  char* gp = static_cast<char*>(geom);
  char* sp = static_cast<char*>(scratch);
  GeomView g;
  g.records = reinterpret_cast<float4*>(gp + s.off_records);
  g.radii = reinterpret_cast<int*>(gp + s.off_radii);
  g.tiles_touched = reinterpret_cast<uint32_t*>(gp + s.off_tiles_touched);
  g.depth_order = reinterpret_cast<uint32_t*>(gp + s.off_depth_order);
  g.offsets = reinterpret_cast<unsigned long long*>(gp + s.off_offsets);
  g.ranges = reinterpret_cast<uint2*>(gp + s.off_ranges);
  g.final_T = reinterpret_cast<float*>(gp + s.off_final_T);
  g.n_contrib = reinterpret_cast<uint32_t*>(gp + s.off_n_contrib);
  g.status = reinterpret_cast<Status*>(gp + s.off_status);
  g.rects = reinterpret_cast<uint2*>(gp + s.off_rects);
  g.bin_start = reinterpret_cast<uint32_t*>(gp + s.off_bin_start);
  g.bin_count = reinterpret_cast<uint32_t*>(gp + s.off_bin_count);
  g.tile_resume = reinterpret_cast<uint2*>(gp + s.off_tile_resume);
  g.tile_queue = reinterpret_cast<uint32_t*>(gp + s.off_tile_queue);
  g.bins = nullptr;
  g.bin_capacity = 0;
  g.depth_keys = (sp && L) ? reinterpret_cast<unsigned long long*>(sp + L->depth_keys) : nullptr;
  g.depth_vals = (sp && L) ? reinterpret_cast<uint32_t*>(sp + L->depth_vals) : nullptr;
  g.depth_keys_sorted = (sp && L) ? reinterpret_cast<unsigned long long*>(sp + L->depth_keys_sorted) : nullptr;
  g.tiles_x = s.tiles_x;
  g.tiles_y = s.tiles_y;
  g.cell_tiles = s.cell_tiles;
  return g;
}

int check_cap(long long cap) {
  if (cap < 0 || cap > 0x7fffffffLL) return SGR_ERR_KEY_CAPACITY;
  return SGR_OK;
}

__global__ void k_status_accumulate(const Status* status, long long* sticky) {
  sticky[0] |= (long long)status->flags;
  const long long n = (long long)status->num_bin_entries;
  if (n > sticky[1]) sticky[1] = n;
}

}  // namespace

void count_launches(int n) { g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed); }

void set_last_error(const std::string& message) { g_last_error = message; }

}  // namespace sgr

using namespace sgr;

extern "C" {

int sgr_abi_version(void) { return SGR_ABI_VERSION; }

const char* sgr_status_string(int status) {
  switch (status) {
    case SGR_OK: return "ok";
    case SGR_ERR_INVALID_ARGUMENT: return "invalid argument";
    case SGR_ERR_UNSUPPORTED: return "unsupported combination of inputs";
    case SGR_ERR_SEMANTIC_CHANNELS: return "more than 16 semantic channels";
    case SGR_ERR_WORKSPACE: return "workspace smaller than sgr_query_sizes requires";
    case SGR_ERR_KEY_CAPACITY: return "key capacity out of range";
    case SGR_ERR_CUDA: return "CUDA runtime error";
    default: return "unknown status";
  }
}

const char* sgr_last_error_message(void) { return g_last_error.c_str(); }

int sgr_query_sizes(const sgr_batch* batch, int64_t key_capacity, sgr_sizes* out) {
  int rc = check_batch(batch);
  if (rc) return rc;
  if ((rc = check_cap(key_capacity))) return rc;
  if (!out) return SGR_ERR_INVALID_ARGUMENT;
  std::memset(out, 0, sizeof(*out));
  return sizes_impl(batch, key_capacity, out);
}

int sgr_forward_geometry(const sgr_batch* batch, void* geom, void* fwd_scratch, size_t fwd_scratch_bytes,
                         void* status_host, void* stream) {
  int rc = check_batch(batch);
  if (rc) return rc;
  if (!geom) return SGR_ERR_INVALID_ARGUMENT;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  sgr_sizes s;
  if ((rc = sizes_impl(batch, 0, &s))) return rc;
  ScratchLayout L;
  if ((rc = scratch_layout(batch, 0, L))) return rc;
  if (fwd_scratch_bytes < L.end_a || (!fwd_scratch && L.end_a > 0)) return SGR_ERR_WORKSPACE;
  GeomView g = geom_view(batch, s, geom, fwd_scratch, &L);
  SGR_CUDA(cudaMemsetAsync(g.status, 0, sizeof(Status), st));
  const long long R = batch->num_records;
  if (R > 0) {
    {
      PhaseScope ph(SGR_PHASE_PREPROCESS, st);
      launch_preprocess(*batch, g, st);
    }
    SGR_CUDA(cudaGetLastError());
    PhaseScope ph(SGR_PHASE_DEPTH_ORDER, st);
    char* sp = static_cast<char*>(fwd_scratch);
    if ((rc = radix_sort_pairs<unsigned long long>(g.depth_keys, g.depth_keys_sorted, g.depth_vals, g.depth_order, R,
                                                   depth_key_bits(batch), sp + L.temp_a, L.temp_a_bytes, st)))
      return rc == SGR_ERR_CUDA ? cuda_fail(cudaGetLastError(), "depth sort") : rc;
    launch_gather_rects(g, R, st);
    SGR_CUDA(cudaGetLastError());
    if ((rc = prefix_sum<unsigned long long, true>(g.offsets, g.offsets, R, sp + L.temp_a, L.temp_a_bytes, st)))
      return rc == SGR_ERR_CUDA ? cuda_fail(cudaGetLastError(), "key offsets") : rc;
    launch_store_key_count(g, R, st);
    SGR_CUDA(cudaGetLastError());
  }
  if (status_host) SGR_CUDA(cudaMemcpyAsync(status_host, g.status, sizeof(Status), cudaMemcpyDeviceToHost, st));
  return SGR_OK;
}

int sgr_forward_raster(const sgr_batch* batch, void* geom, void* bins, int64_t bin_capacity, void* fwd_scratch,
                       size_t fwd_scratch_bytes, const sgr_fwd_outputs* out, void* stream) {
  int rc = check_batch(batch);
  if (rc) return rc;
  if ((rc = check_cap(bin_capacity))) return rc;
  if (!geom || !out || !out->color || !out->others) return SGR_ERR_INVALID_ARGUMENT;
  if (batch->variant == SGR_VARIANT_PART && batch->semantic_channels > 0 && !out->semantic)
    return SGR_ERR_INVALID_ARGUMENT;
  if (bin_capacity > 0 && !bins) return SGR_ERR_INVALID_ARGUMENT;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  sgr_sizes s;
  if ((rc = sizes_impl(batch, bin_capacity, &s))) return rc;
  ScratchLayout L;
  if ((rc = scratch_layout(batch, bin_capacity, L))) return rc;
  if (fwd_scratch_bytes < L.end || (!fwd_scratch && L.end > 0)) return SGR_ERR_WORKSPACE;
  GeomView g = geom_view(batch, s, geom, fwd_scratch, &L);
  g.bins = static_cast<const uint32_t*>(bins);
  g.bin_capacity = bin_capacity;
  char* sp = static_cast<char*>(fwd_scratch);
  const int NO = batch->variant == SGR_VARIANT_PLAIN ? 7 : 8;
  const size_t HW = (size_t)batch->height * batch->width;
  if (batch->num_surfels == 0) {
    // the reference returns zero-filled images when there is nothing to draw
    // (submodules/diff-surfel-rasterization/rasterize_points.cu:85-99)
    SGR_CUDA(cudaMemsetAsync(out->color, 0, (size_t)batch->num_views * 3 * HW * 4, st));
    SGR_CUDA(cudaMemsetAsync(out->others, 0, (size_t)batch->num_views * NO * HW * 4, st));
    if (out->semantic && batch->semantic_channels > 0)
      SGR_CUDA(cudaMemsetAsync(out->semantic, 0, (size_t)batch->num_views * batch->semantic_channels * HW * 4, st));
    return SGR_OK;
  }
  {
    PhaseScope ph(SGR_PHASE_BINNING, st);
    rc = launch_binning(*batch, g, sp + L.bin, st);
    if (rc == SGR_ERR_CUDA) return cuda_fail(cudaGetLastError(), "cell lists");
    if (rc) return rc;
  }
  {
    PhaseScope ph(SGR_PHASE_BLEND_FWD, st);
    launch_render_fwd(*batch, g, *out, st);
  }
  SGR_CUDA(cudaGetLastError());
  if (out->radii)
    SGR_CUDA(cudaMemcpyAsync(out->radii, g.radii, (size_t)batch->num_records * 4, cudaMemcpyDeviceToDevice, st));
  return SGR_OK;
}

int sgr_backward(const sgr_batch* batch, const void* geom, const void* bins, int64_t bin_capacity, void* bwd_scratch,
                 size_t bwd_scratch_bytes, const sgr_bwd_inputs* in, const sgr_bwd_outputs* out, void* stream) {
  int rc = check_batch(batch);
  if (rc) return rc;
  if ((rc = check_cap(bin_capacity))) return rc;
  if (bin_capacity > 0 && !bins) return SGR_ERR_INVALID_ARGUMENT;
  if (!geom || !in || !out || !in->dL_dcolor || !in->dL_dothers) return SGR_ERR_INVALID_ARGUMENT;
  const int S = batch->variant == SGR_VARIANT_PART ? batch->semantic_channels : 0;
  if (S > 0 && !in->dL_dsemantic) return SGR_ERR_INVALID_ARGUMENT;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  sgr_sizes s;
  if ((rc = sizes_impl(batch, 0, &s))) return rc;
  if (bwd_scratch_bytes < s.bwd_scratch_bytes || (!bwd_scratch && s.bwd_scratch_bytes > 0)) return SGR_ERR_WORKSPACE;
  GeomView g = geom_view(batch, s, const_cast<void*>(geom), nullptr, nullptr);
  g.bins = static_cast<const uint32_t*>(bins);
  g.bin_capacity = bin_capacity;
  float* grads = static_cast<float*>(bwd_scratch);
  const size_t P = (size_t)batch->num_surfels;
  if (out->dL_dsemantics && S > 0) SGR_CUDA(cudaMemsetAsync(out->dL_dsemantics, 0, P * S * 4, st));
  if (batch->num_records == 0) return SGR_OK;
  float* dsem = (S > 0) ? out->dL_dsemantics : nullptr;
  if (S > 0 && !dsem) return SGR_ERR_INVALID_ARGUMENT;
  {
    PhaseScope ph(SGR_PHASE_BLEND_BWD, st);
    SGR_CUDA(cudaMemsetAsync(grads, 0, (size_t)batch->num_records * kGradF * 4, st));
    launch_render_bwd(*batch, g, *in, grads, dsem, st);
  }
  SGR_CUDA(cudaGetLastError());
  {
    PhaseScope ph(SGR_PHASE_PREPROCESS_BWD, st);
    launch_preprocess_bwd(*batch, g, grads, *out, st);
  }
  SGR_CUDA(cudaGetLastError());
  return SGR_OK;
}

int sgr_tile_lists(const sgr_batch* batch, void* geom, int32_t* lists, int64_t key_capacity, void* scratch,
                   size_t scratch_bytes, void* stream) {
  int rc = check_batch(batch);
  if (rc) return rc;
  if ((rc = check_cap(key_capacity))) return rc;
  if (!geom || (key_capacity > 0 && !lists)) return SGR_ERR_INVALID_ARGUMENT;
  sgr_sizes s;
  if ((rc = sizes_impl(batch, 0, &s))) return rc;
  if (scratch_bytes < s.tile_list_scratch_bytes || !scratch) return SGR_ERR_WORKSPACE;
  if (batch->num_records == 0) return SGR_OK;
  GeomView g = geom_view(batch, s, geom, nullptr, nullptr);
  rc = launch_tile_lists(*batch, g, reinterpret_cast<uint32_t*>(lists), key_capacity, scratch,
                         static_cast<cudaStream_t>(stream));
  if (rc == SGR_ERR_CUDA) return cuda_fail(cudaGetLastError(), "tile lists");
  return rc;
}

uint64_t sgr_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

int sgr_profile_enable(int enable) {
  PhaseTimer::get().enable(enable != 0);
  return SGR_OK;
}

int sgr_profile_read(float* ms, int32_t* count) { return PhaseTimer::get().read(ms, count); }

int sgr_status_accumulate(const void* status, int64_t* sticky, void* stream) {
  if (!status || !sticky) return SGR_ERR_INVALID_ARGUMENT;
  k_status_accumulate<<<1, 1, 0, static_cast<cudaStream_t>(stream)>>>(static_cast<const sgr::Status*>(status),
                                                                       reinterpret_cast<long long*>(sticky));
  sgr::count_launches(1);
  SGR_CUDA(cudaGetLastError());
  return SGR_OK;
}

int sgr_mark_visible(int32_t P, const float* means3D, const float* viewmatrix, const float* projmatrix,
                     uint8_t* present, void* stream) {
  (void)projmatrix;
  if (P < 0) return SGR_ERR_INVALID_ARGUMENT;
  if (P == 0) return SGR_OK;
  if (!means3D || !viewmatrix || !present) return SGR_ERR_INVALID_ARGUMENT;
  launch_mark_visible(P, means3D, viewmatrix, present, static_cast<cudaStream_t>(stream));
  SGR_CUDA(cudaGetLastError());
  return SGR_OK;
}

}  // extern "C"
