/*
 * sgr.h - C ABI of the GB300 surfel rasteriser (libsgr.so).
 *
 * The library implements the differentiable 2D-Gaussian surfel rasteriser
 * of PartGS in both of its variants ("plain": submodules/diff-surfel-
 * rasterization, "part": submodules/diff-surfel-rasterization_part) and the
 * superquadric-to-surfel binding that feeds it.  No C++ or torch type crosses
 * this boundary: every argument is a plain pointer, an integer, a float or a
 * struct of those.  Device pointers are CUDA global-memory addresses; every
 * call enqueues its work on the caller's stream and never synchronises the
 * host, so whole steps can be captured in a CUDA graph.
 *
 * Reference interfaces replaced (paths relative to the PartGS repository):
 *   sgr_forward_geometry + sgr_forward_raster
 *       -> _C.rasterize_gaussians           submodules/diff-surfel-rasterization/ext.cpp:16,
 *          RasterizeGaussiansCUDA           submodules/diff-surfel-rasterization/rasterize_points.cu:39-134
 *          (part variant: submodules/diff-surfel-rasterization_part/rasterize_points.cu:39-145)
 *   sgr_backward
 *       -> _C.rasterize_gaussians_backward  submodules/diff-surfel-rasterization/ext.cpp:17,
 *          RasterizeGaussiansBackwardCUDA   submodules/diff-surfel-rasterization/rasterize_points.cu:136-233
 *          (part variant: submodules/diff-surfel-rasterization_part/rasterize_points.cu:148-252)
 *   sgr_mark_visible
 *       -> _C.mark_visible                  submodules/diff-surfel-rasterization/ext.cpp:18,
 *          markVisible                      submodules/diff-surfel-rasterization/rasterize_points.cu:235-254
 *   sgr_bind_forward / sgr_bind_backward
 *       -> BlockGaussianModel.prepare_scaling_rot and its autograd backward
 *          games/block_mesh_splatting/scene/block_gaussian_model.py:178-256
 *
 * The reference forward sizes its scratch buffers from the number of
 * (surfel, tile) keys, which it learns with a blocking device-to-host copy
 * (cuda_rasterizer/rasterizer_impl.cu:282), and writes and sorts every key.
 * Here the records are put in depth order once and binned into cells of
 * B x B tiles (sgr_batch.cell_tiles); each tile's list is streamed out of its cell's list by the
 * blend kernels, so no per-tile list is written.  The forward is split in
 * two calls: sgr_forward_geometry counts, on the device, the keys (the
 * reference's num_rendered) and the (record, cell) entries the cell lists
 * need (and, if asked, copies the status word to pinned host memory); the
 * caller sizes the cell-list buffer from that count, or passes a capacity
 * it chose earlier, to sgr_forward_raster.  A count above the capacity is
 * reported through the device status word (SGR_FLAG_BIN_OVERFLOW), never by
 * faulting.  The reference's exact per-tile lists and ranges can still be
 * written out with sgr_tile_lists, for inspection.
 */
#ifndef SGR_H_INCLUDED
#define SGR_H_INCLUDED

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SGR_ABI_VERSION 4

/* status codes returned by every entry point */
#define SGR_OK 0
#define SGR_ERR_INVALID_ARGUMENT 1   /* a null pointer, a negative size or inconsistent tables */
#define SGR_ERR_UNSUPPORTED 2        /* a combination the path does not define */
#define SGR_ERR_SEMANTIC_CHANNELS 3  /* more than SGR_MAX_SEMANTICS semantic channels */
#define SGR_ERR_WORKSPACE 4          /* a workspace smaller than sgr_query_sizes asked for */
#define SGR_ERR_KEY_CAPACITY 5       /* key capacity above 2^31 - 1 or below zero */
#define SGR_ERR_CUDA 6               /* a CUDA runtime call failed; see sgr_last_error_message */

/* Byte offsets in the 32-byte device status word (sgr_sizes.off_status).
 * SGR_STATUS_FRAGMENTS counts the (pixel, list entry) pairs the reference's
 * forward blend would visit: per pixel, the list entries up to and including
 * the one that ends it (or the whole tile list), summed over the batch; the
 * blend's algorithmic work unit (about 77 FP32 operations each). */
#define SGR_STATUS_KEYS 0
#define SGR_STATUS_FLAGS 8
#define SGR_STATUS_BIN_ENTRIES 16
#define SGR_STATUS_FRAGMENTS 24

/* bits of the device status word (sgr_sizes.off_status), set by kernels */
#define SGR_FLAG_KEY_OVERFLOW 1u     /* sgr_tile_lists: more (surfel, tile) keys than its capacity */
#define SGR_FLAG_PREFILTERED 2u      /* prefiltered was set but a surfel failed the near test
                                        (the reference traps here, cuda_rasterizer/auxiliary.h:200-206) */
#define SGR_FLAG_BIN_OVERFLOW 4u     /* more (record, cell) entries than the cell-list capacity */
#define SGR_FLAG_LIST_INCONSISTENT 8u /* sgr_backward: a tile's cell list held fewer entries than its
                                         forward blended (the workspace or the lists changed between the
                                         calls); that tile's gradients are incomplete */

/* sgr_batch.blend_shape: the part of a 16x16 tile each warp of the blend
 * kernels owns.  STRIP16: 16-pixel-wide rows (16x4 at two pixels per
 * thread); PATCH8: 8-pixel-wide patches (8x8).  Only the grouping of pixels
 * into warps changes: every pixel still walks its 16x16 tile's list, so
 * images and gradients are the same. */
#define SGR_BLEND_STRIP16 0
#define SGR_BLEND_PATCH8 1
/* sgr_batch.tile_schedule */
#define SGR_SCHEDULE_GRID 0
#define SGR_SCHEDULE_QUEUE 1
/* sgr_batch.stage_entries: tile-list entries the blends stage in shared
 * memory per batch.  0 lets the library choose: SGR_STAGE_DEFAULT, or
 * SGR_STAGE_SMALL for the part variant above 12 semantic channels (the
 * smaller batch keeps its forward at 4 CTAs per SM).  Every pixel still walks
 * the same entries in the same order, so images and gradients are the same. */
#define SGR_STAGE_DEFAULT 256
#define SGR_STAGE_SMALL 128
#define SGR_STAGE_TINY 64

#define SGR_VARIANT_PLAIN 0
#define SGR_VARIANT_PART 1
#define SGR_MAX_SEMANTICS 16         /* the part variant's fixed register array, P1 forward.cu:317 */
#define SGR_TILE 16                  /* tile edge in pixels, cuda_rasterizer/config.h:15-16 */
#define SGR_DEFAULT_CELL_TILES 8     /* cell edge in tiles when sgr_batch.cell_tiles is 0 */

/* One scene: a contiguous range of surfels seen by a contiguous range of views. */
typedef struct sgr_scene_desc {
    int32_t surfel_offset;
    int32_t surfel_count;
    int32_t view_begin;
    int32_t view_count;
} sgr_scene_desc;

/* One view.  record_offset is the first of this view's surfel_count per-view
 * records; records of all views are packed back to back. */
typedef struct sgr_view_desc {
    int32_t scene;
    int32_t record_offset;
    float tanfovx;
    float tanfovy;
} sgr_view_desc;

/* A batch of views over one or more scenes.  With one scene and one view
 * this is exactly the reference's single-view call. */
typedef struct sgr_batch {
    int32_t variant;             /* SGR_VARIANT_PLAIN or SGR_VARIANT_PART */
    int32_t num_scenes;
    int32_t num_views;
    int32_t height;              /* image size, shared by every view */
    int32_t width;
    int32_t num_surfels;         /* P: surfels of all scenes */
    int32_t num_records;         /* R: sum over views of their scene's surfel count */
    int32_t sh_degree;           /* active SH degree D */
    int32_t sh_coeffs;           /* M coefficients per surfel; 0 when colors_precomp is given */
    int32_t semantic_channels;   /* S, part variant only, 0..SGR_MAX_SEMANTICS */
    int32_t prefiltered;
    float scale_modifier;
    /* device tables */
    const sgr_scene_desc* scenes;    /* [num_scenes] */
    const sgr_view_desc* views;      /* [num_views] */
    const float* viewmatrix;         /* [V,16] world_view_transform, row-major as torch stores it */
    const float* projmatrix;         /* [V,16] full_proj_transform */
    const float* campos;             /* [V,3] */
    const float* background;         /* [3] */
    /* device surfel attributes, contiguous float32 */
    const float* means3D;            /* [P,3] */
    const float* scales;             /* [P,2] or NULL with transmat_precomp */
    const float* rotations;          /* [P,4] (w,x,y,z) or NULL with transmat_precomp */
    const float* opacities;          /* [P] */
    const float* shs;                /* [P,M,3] or NULL */
    const float* colors_precomp;     /* [P,3] or NULL */
    const float* transmat_precomp;   /* [P,9] or NULL (single-view batches only) */
    const float* semantics;          /* [P,S] or NULL */
    int32_t cell_tiles;              /* edge, in tiles, of the cells records are binned into: 1, 2, 4, 8 or 16;
                                        0 for the default (SGR_DEFAULT_CELL_TILES) */
    int32_t blend_shape;             /* pixels of a tile each warp of the blends owns: SGR_BLEND_STRIP16 or
                                        SGR_BLEND_PATCH8 (results identical; speed depends on splat sizes) */
    int32_t tile_schedule;           /* SGR_SCHEDULE_GRID (one CTA per tile) or SGR_SCHEDULE_QUEUE (persistent
                                        CTAs take tiles from a device queue, longest estimated first) */
    int32_t stage_entries;           /* 0 (the library's choice), SGR_STAGE_DEFAULT, SGR_STAGE_SMALL or
                                        SGR_STAGE_TINY: list entries per staged batch of the blends (results
                                        identical) */
} sgr_batch;

/* Workspace sizes and the layout of the geometry workspace. */
typedef struct sgr_sizes {
    size_t geom_bytes;           /* kept from the forward to the backward */
    size_t list_bytes;           /* kept: the cell lists, bin_capacity entries */
    size_t fwd_scratch_bytes;    /* forward only */
    size_t bwd_scratch_bytes;    /* backward only */
    size_t tile_list_scratch_bytes;  /* sgr_tile_lists only */
    /* byte offsets inside the geometry workspace */
    size_t off_records;          /* float4[R][6] per-view surfel records */
    size_t off_radii;            /* int32[R] */
    size_t off_tiles_touched;    /* uint32[R] */
    size_t off_depth_order;      /* uint32[R] record ids in (view, depth, id) order */
    size_t off_offsets;          /* uint64[R] inclusive scan of tiles_touched in that order */
    size_t off_ranges;           /* uint32[V*tiles][2] per-tile [start, end), written by sgr_tile_lists */
    size_t off_final_T;          /* float[V][3][H][W]: T, M1, M2 */
    size_t off_n_contrib;        /* uint32[V][2][H][W]: last contributor, median contributor */
    size_t off_status;           /* uint64 key count, uint32 flags, uint32 pad, uint64 cell-list entries,
                                    uint64 fragments the forward blend visited (see SGR_STATUS_FRAGMENTS) */
    size_t off_rects;            /* uint32[R][2] tile rectangle of each record in depth order */
    size_t off_bin_start;        /* uint32[V*cells] start of each cell list */
    size_t off_bin_count;        /* uint32[V*cells] length of each cell list */
    size_t off_tile_resume;      /* uint32[V*tiles][2] cell-list entries the forward scanned, tile entries found */
    size_t off_tile_queue;       /* uint32[V*tiles + 1]: tile order and head of the SGR_SCHEDULE_QUEUE queue */
    int32_t tiles_x, tiles_y;
    int32_t tile_key_bits;
    int32_t cell_tiles;          /* cell edge in tiles */
} sgr_sizes;

/* Per-view outputs of the forward.  color [V,3,H,W], others [V,7,H,W]
 * (plain: expected depth, alpha, normal xyz, median depth, distortion) or
 * [V,8,H,W] (part: the same plus median weight), semantic [V,S,H,W] (part),
 * radii [R]. */
typedef struct sgr_fwd_outputs {
    float* color;
    float* others;
    float* semantic;
    int32_t* radii;
} sgr_fwd_outputs;

/* Upstream gradients, same shapes as the forward outputs. */
typedef struct sgr_bwd_inputs {
    const float* dL_dcolor;
    const float* dL_dothers;
    const float* dL_dsemantic;   /* part variant, or NULL */
} sgr_bwd_inputs;

/* Gradients.  Per-surfel tensors are summed over the views of the surfel's
 * scene; dL_dmeans2D and dL_dtransmat are per view record.  Every element
 * is written (no zero-fill needed); NULL skips an output. */
typedef struct sgr_bwd_outputs {
    float* dL_dmeans2D;          /* [R,3] densification proxy (P0 backward.cu:626-629) */
    float* dL_dcolors;           /* [P,3] */
    float* dL_dopacity;          /* [P] */
    float* dL_dmeans3D;          /* [P,3] */
    float* dL_dtransmat;         /* [R,9] */
    float* dL_dsh;               /* [P,M,3] */
    float* dL_dscales;           /* [P,2] */
    float* dL_drotations;        /* [P,4] */
    float* dL_dsemantics;        /* [P,S] */
} sgr_bwd_outputs;

/* Library identity. */
int sgr_abi_version(void);
const char* sgr_status_string(int status);
/* Message of the last failing CUDA call on this host thread ("" if none). */
const char* sgr_last_error_message(void);

/* Workspace sizes for a batch and a cell-list capacity in entries (0 when
 * only the geometry phase will run).  Replaces the sizing in
 * required<GeometryState> / required<ImageState> / required<BinningState>,
 * cuda_rasterizer/rasterizer_impl.cu:155-194. */
int sgr_query_sizes(const sgr_batch* batch, int64_t bin_capacity, sgr_sizes* out);

/* Phase 1 of the forward: per-view preprocess (transform, screen bounds,
 * SH colour), depth order, the key count and the cell-list entry count.  If
 * status_host is not NULL it must be pinned host memory of 32 bytes; the
 * status word is copied there asynchronously on the stream. */
int sgr_forward_geometry(const sgr_batch* batch, void* geom, void* fwd_scratch, size_t fwd_scratch_bytes,
                         void* status_host, void* stream);

/* Phase 2: the cell lists (bin_capacity entries in `bins`) and the blend
 * (replaces duplicateWithKeys, the tile sort, identifyTileRanges and
 * renderCUDA, cuda_rasterizer/rasterizer_impl.cu:288-342). */
int sgr_forward_raster(const sgr_batch* batch, void* geom, void* bins, int64_t bin_capacity,
                       void* fwd_scratch, size_t fwd_scratch_bytes, const sgr_fwd_outputs* out, void* stream);

/* Backward of both phases, from the geometry workspace and the cell lists
 * of the forward. */
int sgr_backward(const sgr_batch* batch, const void* geom, const void* bins, int64_t bin_capacity,
                 void* bwd_scratch, size_t bwd_scratch_bytes, const sgr_bwd_inputs* in,
                 const sgr_bwd_outputs* out, void* stream);

/* Writes out, after a forward, the reference's per-tile lists (record ids,
 * at most key_capacity of them, in the binning buffer's layout) and their
 * [start, end) ranges at sizes.off_ranges of the geometry workspace.  For
 * inspection; the blend never reads them. */
int sgr_tile_lists(const sgr_batch* batch, void* geom, int32_t* lists, int64_t key_capacity, void* scratch,
                   size_t scratch_bytes, void* stream);

/* ---- phase timing ------------------------------------------------------ */

/* Phases the entry points bracket with CUDA events while profiling is on. */
#define SGR_PHASE_PREPROCESS 0      /* per-view preprocess */
#define SGR_PHASE_DEPTH_ORDER 1     /* depth order and key offsets */
#define SGR_PHASE_BINNING 2         /* per-(chunk, tile) list index and ranges */
#define SGR_PHASE_BLEND_FWD 3
#define SGR_PHASE_BLEND_BWD 4
#define SGR_PHASE_PREPROCESS_BWD 5
#define SGR_NUM_PHASES 6

/* Turns event recording on (1) or off (0) for calls made afterwards from
 * any thread.  Events are recorded on the caller's stream. */
int sgr_profile_enable(int enable);
/* Waits for the recorded events, writes the summed milliseconds and the
 * number of recordings of each phase since the last read (arrays of
 * SGR_NUM_PHASES), and forgets them. */
int sgr_profile_read(float* ms, int32_t* count);
/* Number of kernels this library has launched (or recorded into a stream
 * capture) since it was loaded, over all threads.  Instrumentation with no
 * counterpart in the reference. */
uint64_t sgr_kernel_launches(void);

/* Folds the status word at `status` (sgr_sizes.off_status of a geometry
 * workspace) into a device record of two int64: sticky[0] |= its flags,
 * sticky[1] = max(sticky[1], its cell-list entry count).  One one-thread
 * kernel on `stream`, so a captured training step keeps the flags of every
 * forward and backward it replays.  No counterpart in the reference (whose
 * calls synchronise the host instead). */
int sgr_status_accumulate(const void* status, int64_t* sticky, void* stream);

/* ---- the sort and scans the forward uses -------------------------------- */

/* Stable LSD radix sort of n (key, value) pairs on key bits [0, end_bit),
 * 8 bits per pass: keys_out / vals_out in ascending key order, equal keys in
 * input order.  Replaces the reference's cub::DeviceRadixSort::SortPairs
 * (cuda_rasterizer/rasterizer_impl.cu:304-309), which sorts the same way;
 * the forward calls it on (view << 32 | depth bits, record) pairs.  The
 * inputs are not modified; temp must hold sgr_radix_sort_temp_bytes(n, key
 * bytes) bytes.  key_bytes is 8 (uint64 keys) or 4 (uint32 keys). */
size_t sgr_radix_sort_temp_bytes(int64_t n, int key_bytes);
int sgr_radix_sort_pairs(const void* keys_in, void* keys_out, const uint32_t* vals_in, uint32_t* vals_out, int64_t n,
                         int key_bytes, int end_bit, void* temp, size_t temp_bytes, void* stream);
/* Prefix sums the forward uses: inclusive over uint64 (key offsets, the
 * reference's cub::DeviceScan::InclusiveSum, rasterizer_impl.cu:278) and
 * exclusive over uint32 (cell-list starts).  `in` may equal `out`; temp
 * must hold sgr_prefix_sum_temp_bytes(n, element bytes) bytes. */
size_t sgr_prefix_sum_temp_bytes(int64_t n, int elem_bytes);
int sgr_inclusive_sum_u64(const uint64_t* in, uint64_t* out, int64_t n, void* temp, size_t temp_bytes, void* stream);
int sgr_exclusive_sum_u32(const uint32_t* in, uint32_t* out, int64_t n, void* temp, size_t temp_bytes, void* stream);

/* Near-plane visibility of P points in one view (present: uint8[P]). */
int sgr_mark_visible(int32_t P, const float* means3D, const float* viewmatrix, const float* projmatrix,
                     uint8_t* present, void* stream);

/* ---- point-level training loss ------------------------------------------ */

/* The per-view loss of the reference's point-stage step (train.py:229-250,
 * utils/loss_utils.py:8-54, utils/point_utils.py:4-33), averaged over V views:
 *   L = (1 - ls) mean|c - t| + ls (1 - mean SSIM11(c, t))
 *     + ld mean(distortion) + ln mean(1 - n_render . n_surface)
 * n_render is the rendered normal rotated to world space; n_surface is the
 * normal of the surface depth (median depth weighted by depth_ratio, the
 * expected depth by 1 - depth_ratio) times the detached alpha. */
typedef struct sgr_loss_args {
    int32_t V, H, W;
    float lambda_dssim;
    float lambda_dist;
    float lambda_normal;
    float depth_ratio;
    const float* color;          /* [V,3,H,W] rendered */
    const float* target;         /* [V,3,H,W] */
    const float* others;         /* [V,7,H,W] rendered aux maps (plain layout) */
    const float* view_to_world;  /* [V,3,3] rotation taking view normals to world: n_w[d] = sum_c n_v[c] R[c][d] */
    const float* ray_basis;      /* [V,3,3] rows a0, a1, a2: ray(x, y) = x a0 + y a1 + a2 */
    const float* ray_origin;     /* [V,3] */
} sgr_loss_args;

size_t sgr_loss_scratch_bytes(const sgr_loss_args* a);
/* Loss value (device float) and its gradients w.r.t. color and others (every
 * element written). */
int sgr_loss_forward_backward(const sgr_loss_args* a, float* loss, float* dL_dcolor, float* dL_dothers, void* scratch,
                              void* stream);

/* ---- superquadric binding ---------------------------------------------- */

/* Shapes of the binding: B superquadrics, each with V vertices on an
 * (eta, omega) parameter set, F triangles, N surfels per triangle. */
typedef struct sgr_bind_args {
    int32_t B, V, F, N;
    float ratio_block_scene;     /* vertex scale of the unit superquadric */
    float scale_block_min;       /* added to exp(sq_s) */
    const float* sq_s;           /* [B,3] log semi-axes */
    const float* sq_r;           /* [B,4] unnormalised quaternion (w,x,y,z) */
    const float* sq_t;           /* [B,3] translation */
    const float* sq_eps;         /* [B,2] exponent logits */
    const float* eta;            /* [B,V] */
    const float* omega;          /* [B,V] */
    const int32_t* faces;        /* [B,F,3] vertex ids */
    const float* sq_occ;         /* [B] occupancy logits */
    const float* alpha;          /* [B*F,N,3] raw barycentric weights (relu + normalise inside) */
    const float* scale;          /* [B,F*N] surfel scale factors */
} sgr_bind_args;

/* Forward: xyz [B*F*N,3], log_scaling [B*F*N,2], rotation [B*F*N,4]
 * (the tensors prepare_scaling_rot stores in _xyz, _scaling, _rotation,
 * block_gaussian_model.py:198-256) and opacity [B*F*N] (get_opacity,
 * block_gaussian_model.py:107-109).  NULL skips an output. */
int sgr_bind_forward(const sgr_bind_args* a, float* xyz, float* log_scaling, float* rotation, float* opacity,
                     void* stream);

/* Backward: from dL/d_xyz, dL/d_scaling (of the log scaling), dL/d_rotation
 * and dL/d_opacity (each may be NULL for zero) to dL/dsq_s, dL/dsq_r,
 * dL/dsq_t, dL/dsq_eps and dL/dsq_occ, which are overwritten.  scratch must
 * hold sgr_bind_scratch_bytes(a) bytes. */
size_t sgr_bind_scratch_bytes(const sgr_bind_args* a);
int sgr_bind_backward(const sgr_bind_args* a, const float* d_xyz, const float* d_log_scaling,
                      const float* d_rotation, const float* d_opacity, float* d_sq_s, float* d_sq_r,
                      float* d_sq_t, float* d_sq_eps, float* d_sq_occ, void* scratch, void* stream);

/* sgr_bind_backward without a scratch argument: the scratch is a fixed
 * 4 MiB device array inside the library, so the call allocates nothing.
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory at the call (no device allocator of their own, or a loop that must
 * not enter cudaMalloc).  Shapes needing more than 4 MiB of scratch
 * (sgr_bind_scratch_bytes) return SGR_ERR_WORKSPACE; calls that overlap on
 * one device race on the array; the first call on a device sets it up and
 * should come before any stream capture. */
int sgr_bind_backward_static(const sgr_bind_args* a, const float* d_xyz, const float* d_log_scaling,
                             const float* d_rotation, const float* d_opacity, float* d_sq_s, float* d_sq_r,
                             float* d_sq_t, float* d_sq_eps, float* d_sq_occ, void* stream);

/* ---- optimiser ---------------------------------------------------------- */

/* One parameter tensor of an Adam step: numel floats each of param, grad and
 * the two moment buffers (device pointers), and its learning rate. */
#define SGR_ADAM_MAX_TENSORS 16
typedef struct sgr_adam_tensor {
    float* param;
    float* grad;
    float* exp_avg;
    float* exp_avg_sq;
    int64_t numel;
    float lr;
} sgr_adam_tensor;

typedef struct sgr_adam_args {
    sgr_adam_tensor tensors[SGR_ADAM_MAX_TENSORS];
    int32_t count;
    float beta1, beta2, eps;
    int32_t zero_grad;           /* 1: clear each gradient after its update */
} sgr_adam_args;

/* Adam update of up to SGR_ADAM_MAX_TENSORS tensors in one launch, the
 * surfel optimiser of scene/gaussian_model.py:266 (torch.optim.Adam, one
 * learning rate per group, eps 1e-15).  `step` is a device float holding the
 * step count; the call increments it first.  Never synchronises. */
int sgr_adam_step(const sgr_adam_args* args, float* step, void* stream);

/* ---- point-level parameter activations ---------------------------------- */

/* The training step's parameter getters (scene/gaussian_model.py:198-218):
 * scales = exp(log_scaling), rotations = F.normalize(rotation),
 * opacities = sigmoid(opacity_logit), shs = cat(features_dc, features_rest),
 * and their adjoints.  Device pointers; P surfels, M = sh_coeffs. */
typedef struct sgr_activate_args {
    int64_t P;
    int32_t sh_coeffs;           /* M, 1..16 */
    const float* log_scaling;    /* [P,2] */
    const float* rotation;       /* [P,4] */
    const float* opacity_logit;  /* [P] */
    const float* features_dc;    /* [P,1,3] */
    const float* features_rest;  /* [P,M-1,3] */
    float* scales;               /* forward outputs: [P,2], [P,4], [P], [P,M,3] */
    float* rotations;
    float* opacities;
    float* shs;
    float* d_log_scaling;        /* backward outputs, the inputs' shapes */
    float* d_rotation;
    float* d_opacity_logit;
    float* d_features_dc;
    float* d_features_rest;
} sgr_activate_args;

int sgr_activate_forward(const sgr_activate_args* args, void* stream);
/* Upstream gradients may be NULL (zero). */
int sgr_activate_backward(const sgr_activate_args* args, const float* d_scales, const float* d_rotations,
                          const float* d_opacities, const float* d_shs, void* stream);

/* ---- densification statistics (train.py:293-297) ------------------------- */

/* For every surfel and each of its scene's views (device scene / view tables
 * of the batch) where radii[record] > 0: max_radii2D = max(max_radii2D,
 * radius), grad_accum += grad_scale * |dmeans2D[record][0:2]|, denom += 1
 * (scene/gaussian_model.py:515-517), views in order.  radii [R] int32 and
 * dmeans2D [R,3] as the forward and backward wrote them; max_radii2D,
 * grad_accum, denom [num_surfels] updated in place. */
int sgr_densify_stats(const sgr_scene_desc* scenes, int32_t num_scenes, const sgr_view_desc* views,
                      int32_t num_surfels, const int32_t* radii, const float* dmeans2D, float grad_scale,
                      float* max_radii2D, float* grad_accum, float* denom, void* stream);

/* ---- block-stage superquadric losses -------------------------------------
 * games/block_mesh_splatting/scene/block_gaussian_model.py:522-582: the ray
 * coverage (ray_in_mask), uncoverage (ray_out_mask) and occupancy
 * (primitive_opacity) losses over a view's ray samples, and the overlap loss
 * over random points of every block, with the SDF of
 * games/block_mesh_splatting/utils/superquadric.py:25-46 (as_sdf=2). */

#define SGR_SQ_MAX_BLOCKS 64

typedef struct sgr_sq_loss_args {
    int32_t n_blocks;            /* 1 .. SGR_SQ_MAX_BLOCKS */
    float ratio;                 /* ratio_block_scene */
    const float* S;              /* [n,3] block scales (get_mesh_scaling) */
    const float* R;              /* [n,3,3] row-major rotation matrices */
    const float* T;              /* [n,3] translations */
    const float* eps1;           /* [n] */
    const float* eps2;           /* [n] */
    const float* occ_logit;      /* [n] sq_occ (alpha = sigmoid); NULL: 0 */
    /* ray losses (n_rays = 0: none; losses[0..2] = 0) */
    int32_t n_rays, n_samples;
    const float* ray_origin;     /* [n_rays,3] camera centre per ray */
    const float* ray_dir;        /* [n_rays,3] pixel point minus centre */
    const float* ray_jitter;     /* [n_rays,n_samples] uniform [0,1) */
    const float* ray_label;      /* [n_rays] mask value at the ray's pixel */
    float near, far;
    /* overlap loss (n_overlap = 0: none; losses[3] = 0) */
    int32_t n_overlap;           /* points per block (OVERLAP_N_POINTS) */
    const float* overlap_unit;   /* [n_blocks,n_overlap,3] uniform in [-1,1] */
    const float* overlap_noise;  /* [n_blocks] N(0,1) added to occ_logit; NULL: 0 */
    float overlap_temperature;   /* OVERLAP_TEMPERATURE */
    float overlap_max_blocks;    /* OVERLAP_N_BLOCKS */
    /* workspace (sgr_sq_scratch_bytes), outputs and gradients */
    void* scratch;
    size_t scratch_bytes;
    float* losses;               /* [4] device: ray_in_mask, ray_out_mask, primitive_opacity, overlap */
    float *d_S, *d_R, *d_T, *d_eps1, *d_eps2, *d_occ_logit;   /* written (not accumulated) by the backward */
} sgr_sq_loss_args;

size_t sgr_sq_scratch_bytes(const sgr_sq_loss_args* args);
/* Forward: losses[4]; keeps each ray's minimum and occupancy choice in the
 * scratch for the backward.  Two launches. */
int sgr_sq_losses_forward(const sgr_sq_loss_args* args, void* stream);
/* Backward from d_losses[4] (device) to the block parameters, after the
 * forward with the same arguments and scratch.  Two launches. */
int sgr_sq_losses_backward(const sgr_sq_loss_args* args, const float* d_losses, void* stream);
/* The SDF (implicit_sq, as_sdf=2) of points [m,3] to every block: out [n,m]. */
int sgr_sq_sdf(const sgr_sq_loss_args* args, const float* points, int64_t n_points, float* out, void* stream);

/* ---- Chamfer evaluation (utils/blender_eval.py:25-111) ------------------- */

/* Exact nearest neighbour in r (m points, xyz float) of each of the n points
 * of q: dist [n] (Euclidean) and, unless NULL, idx [n] (first minimum). */
int sgr_nn_search(const float* q, int64_t n, const float* r, int64_t m, float* dist, int32_t* idx, void* stream);

/* The same search through a uniform cell grid over r (about two cells per
 * point): the same distances and indices as sgr_nn_search, bit for bit, at
 * a cost that grows with n + m instead of n m for surface-like point sets.
 * lo / hi (host, 3 floats): a box holding every point of r, e.g. its
 * bounding box.  Queries far from every point of r fall back to the
 * brute-force scan inside the call.  Seven launches plus a CUB scan and
 * sort; no host synchronisation. */
size_t sgr_nn_grid_scratch_bytes(int64_t n, int64_t m, const float* lo, const float* hi);
int sgr_nn_search_grid(const float* q, int64_t n, const float* r, int64_t m, const float* lo, const float* hi,
                       float* dist, int32_t* idx, void* scratch, size_t scratch_bytes, void* stream);

/* The reference's radius downsample: in index order, point i is kept unless
 * an earlier kept point lies within `radius` (distance <= radius, fp64 like
 * the reference).  pts [n,3] float64 on the device, lo / hi their bounding
 * box on the host; state [n] receives 1 (kept) or 2 (removed); rounds (host,
 * may be NULL) the number of parallel rounds.  Synchronises the host once
 * per round. */
size_t sgr_downsample_scratch_bytes(int64_t n);
int sgr_radius_downsample(const double* pts, int64_t n, const double* lo, const double* hi, double radius,
                          uint8_t* state, void* scratch, size_t scratch_bytes, int32_t* rounds, void* stream);

/* ---- proposal network: BF16 tensor-core GEMM --------------------------- */

/* Epilogues of sgr_mlp_gemm (x = accumulator + bias) */
#define SGR_GEMM_STORE_F32 0   /* out[m,n] = x (fp32) */
#define SGR_GEMM_ADD_F32 1     /* out[m,n] += x (fp32, atomic; with split_k) */
#define SGR_GEMM_RELU_BF16 2   /* out[m,n] = bf16(max(x, 0)) */
#define SGR_GEMM_MASK_BF16 3   /* out[m,n] = bf16(mask[m,n] > 0 ? x : 0): a ReLU's backward */
#define SGR_MLP_TIMEOUT 1u     /* status bit: a wait for the tensor cores or a copy ran out (1 s) */

/* C[M,N] = A[M,K] . B[N,K]^T with bf16 operands, fp32 accumulation.  A is
 * row-major with K contiguous (lda elements per row) or, with a_trans, its
 * transpose (K rows of M contiguous values); likewise B (a_trans and b_trans
 * must agree).  Strides are multiples of 8 and bases 16-byte aligned. */
typedef struct sgr_gemm_args {
    int64_t M, N, K;
    const void* A;               /* bf16 */
    int64_t lda;
    int32_t a_trans;
    const void* B;               /* bf16 */
    int64_t ldb;
    int32_t b_trans;
    const float* bias;           /* [N] or NULL */
    int32_t epilogue;            /* SGR_GEMM_* */
    void* out;
    int64_t ldo;
    const void* mask;            /* bf16 [M, ldmask], SGR_GEMM_MASK_BF16 only */
    int64_t ldmask;
    int64_t split_k;             /* 0, or K per CTA (a multiple of 64; SGR_GEMM_ADD_F32) */
    uint32_t* status;            /* device word, OR-ed with SGR_MLP_TIMEOUT */
    int32_t skip_loads;          /* 0.  Nonzero (tests of the timeout path only): the TMA producer issues no
                                    loads, so the MMA issuer's bounded wait runs out with nothing in flight
                                    and the call reports SGR_MLP_TIMEOUT after about one second */
} sgr_gemm_args;

/* The GEMM of the point-set proposal network's layers and their backward
 * (no counterpart in the reference: the network is new).  tcgen05 MMA with
 * tensor-memory accumulators; never synchronises. */
int sgr_mlp_gemm(const sgr_gemm_args* args, void* stream);

/* Max-pool of a bf16 [sets*P, C] activation over each set's P rows: g
 * [sets, C] fp32 (and bf16 into g_bf16 unless NULL) and arg [sets, C], the
 * row of each maximum. */
int sgr_mlp_maxpool(const void* h, int32_t sets, int32_t P, int32_t C, float* g, void* g_bf16, int32_t* arg,
                    void* stream);
/* Its backward through the ReLU below it: dh (bf16 [sets*P, C], cleared
 * here) gets dg[s, c] at row arg[s, c] where g[s, c] > 0. */
int sgr_mlp_maxpool_backward(const float* dg, const float* g, const int32_t* arg, int32_t sets, int32_t P,
                             int32_t C, void* dh, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SGR_H_INCLUDED */
