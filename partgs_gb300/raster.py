"""Host side of the surfel rasteriser: tensors -> sgr_batch -> libsgr.so.

``forward`` / ``backward`` are the functional core both drop-in packages
(``diff_surfel_rasterization`` and ``diff_surfel_rasterization_part``) and
the batched multi-view path use.  Memory comes from PyTorch's caching
allocator; every device byte the library touches is a tensor held here, so
the forward state lives exactly as long as the autograd graph needs it (as
the reference's three byte buffers do,
submodules/diff-surfel-rasterization/diff_surfel_rasterization/__init__.py:97).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import torch

from . import _lib as L

_PINNED: dict = {}


def _ptr(t: torch.Tensor | None) -> int | None:
    if t is None or t.numel() == 0:
        return None
    return t.data_ptr()


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def _f32(t: torch.Tensor | None, align16: bool = False) -> torch.Tensor | None:
    if t is None or t.numel() == 0:
        return None
    if not t.is_cuda:
        raise ValueError("rasteriser inputs must be CUDA tensors")
    t = t.detach()
    if t.dtype != torch.float32:
        t = t.float()
    t = t.contiguous()
    if align16 and t.data_ptr() % 16 != 0:
        t = t.clone()
    return t


def _pinned(device, nbytes=L.STATUS_BYTES):
    key = (device, nbytes)
    buf = _PINNED.get(key)
    if buf is None:
        buf = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
        _PINNED[key] = buf
    return buf


@dataclass
class ViewSet:
    """Views of a batch.  One scene by default; ``scene_sizes`` /
    ``scene_views`` describe several scenes packed back to back."""
    viewmatrix: torch.Tensor      # [V,16] (or [V,4,4])
    projmatrix: torch.Tensor      # [V,16]
    campos: torch.Tensor          # [V,3]
    tanfov: list                  # [(tanfovx, tanfovy)] * V
    height: int
    width: int
    scene_sizes: list | None = None   # surfels per scene
    scene_views: list | None = None   # views per scene (views are grouped by scene)


@dataclass
class RasterState:
    variant: int
    batch: L.Batch
    keep: list
    geom: torch.Tensor
    bins: torch.Tensor            # cell lists
    bin_capacity: int             # entries they hold
    sizes: L.Sizes
    num_surfels: int
    num_records: int
    num_views: int
    sh_coeffs: int
    semantic_channels: int
    extra: dict = field(default_factory=dict)


def _tables(variant, P, vs: ViewSet, device):
    V = int(vs.viewmatrix.shape[0])
    sizes = vs.scene_sizes or [P]
    sviews = vs.scene_views or [V]
    if sum(sizes) != P or sum(sviews) != V or len(sizes) != len(sviews):
        raise ValueError("scene table does not cover the surfels / views")
    scenes, views = [], []
    so, vo, ro = 0, 0, 0
    for s, (n, nv) in enumerate(zip(sizes, sviews)):
        scenes.append((so, n, vo, nv))
        for _ in range(nv):
            tx, ty = vs.tanfov[vo]
            views.append((s, ro, float(tx), float(ty)))
            ro += n
            vo += 1
        so += n
    if ro >= 2 ** 31:
        raise ValueError("more than 2^31 per-view surfel records")
    sc = (L.SceneDesc * len(scenes))(*[L.SceneDesc(*x) for x in scenes])
    vw = (L.ViewDesc * len(views))(*[L.ViewDesc(*x) for x in views])
    sct = torch.frombuffer(bytearray(bytes(sc)), dtype=torch.uint8).to(device)
    vwt = torch.frombuffer(bytearray(bytes(vw)), dtype=torch.uint8).to(device)
    return sct, vwt, len(scenes), ro


def make_batch(variant, means3D, opacities, shs, colors_precomp, scales, rotations, transmat_precomp, semantics,
               vs: ViewSet, bg, sh_degree, scale_modifier, prefiltered, tables=None, cell_tiles=0, blend_shape=0,
               tile_schedule=0, stage_entries=0):
    if means3D.dim() != 2 or means3D.shape[1] != 3:
        raise ValueError("means3D must have dimensions (num_points, 3)")
    if variant == L.SGR_VARIANT_PART and semantics is not None and semantics.dim() == 2 and \
            int(semantics.shape[1]) > L.SGR_MAX_SEMANTICS:
        raise ValueError(f"at most {L.SGR_MAX_SEMANTICS} semantic channels are supported, "
                         f"got {int(semantics.shape[1])}")
    if shs is not None and shs.numel() and (shs.dim() != 3 or shs.shape[2] != 3 or shs.shape[1] > 16):
        raise ValueError("shs must have dimensions (num_points, M <= 16, 3)")
    device = means3D.device
    P = int(means3D.shape[0])
    keep = []
    t = {}
    t["means3D"] = _f32(means3D)
    t["opacities"] = _f32(opacities.reshape(-1)) if opacities is not None else None
    t["shs"] = _f32(shs)
    t["colors_precomp"] = _f32(colors_precomp)
    t["scales"] = _f32(scales)
    t["rotations"] = _f32(rotations, align16=True)
    t["transmat_precomp"] = _f32(transmat_precomp)
    t["semantics"] = _f32(semantics)
    t["viewmatrix"] = _f32(vs.viewmatrix.reshape(-1, 16))
    t["projmatrix"] = _f32(vs.projmatrix.reshape(-1, 16))
    t["campos"] = _f32(vs.campos.reshape(-1, 3))
    t["background"] = _f32(bg)
    if variant == L.SGR_VARIANT_PART and t["scales"] is not None:
        if scales.dim() != 2 or scales.shape[1] != 2:
            raise ValueError("scales must have dimensions (num_points, 2)")
        if rotations.dim() != 2 or rotations.shape[1] != 4:
            raise ValueError("rotations must have dimensions (num_points, 4)")
    S = 0
    if variant == L.SGR_VARIANT_PART:
        S = int(semantics.shape[1]) if semantics is not None and semantics.dim() == 2 else 0
        if S > L.SGR_MAX_SEMANTICS:
            raise ValueError(f"at most {L.SGR_MAX_SEMANTICS} semantic channels are supported, got {S}")
    M = int(shs.shape[1]) if t["shs"] is not None else 0
    sct, vwt, nscenes, R = tables if tables is not None else _tables(variant, P, vs, device)
    keep += list(t.values()) + [sct, vwt]
    b = L.Batch()
    b.variant = variant
    b.num_scenes = nscenes
    b.num_views = int(t["viewmatrix"].shape[0])
    b.height = int(vs.height)
    b.width = int(vs.width)
    b.num_surfels = P
    b.num_records = R
    b.sh_degree = int(sh_degree)
    b.sh_coeffs = M
    b.semantic_channels = S
    b.prefiltered = int(bool(prefiltered))
    b.cell_tiles = int(cell_tiles)
    b.blend_shape = int(blend_shape)
    b.tile_schedule = int(tile_schedule)
    b.stage_entries = int(stage_entries)
    b.scale_modifier = float(scale_modifier)
    b.scenes = sct.data_ptr()
    b.views = vwt.data_ptr()
    for k in ("viewmatrix", "projmatrix", "campos", "background", "means3D", "scales", "rotations", "opacities",
              "shs", "colors_precomp", "transmat_precomp", "semantics"):
        setattr(b, k, _ptr(t[k]))
    return b, keep, t


def forward(variant, means3D, opacities, shs, colors_precomp, scales, rotations, transmat_precomp, semantics,
            vs: ViewSet, bg, sh_degree=0, scale_modifier=1.0, prefiltered=False, bin_capacity=None, tables=None,
            status_host=None, cell_tiles=0, blend_shape=0, tile_schedule=0, stage_entries=0):
    """Rasterises every view of ``vs``.  Returns (color [V,3,H,W], others
    [V,7|8,H,W], semantic [V,S,H,W] or None, radii [R] int32, state).

    Without ``bin_capacity`` the cell-list entry count is read back (one
    host synchronisation, where the reference reads its key count back,
    cuda_rasterizer/rasterizer_impl.cu:282) and the cell lists are sized
    exactly.  With it nothing synchronises: the lists hold ``bin_capacity``
    entries, and the device status word (key count, flags, entry count) is
    copied into the pinned ``status_host`` tensor (32 bytes) for the caller
    to inspect once the stream has reached it.  ``cell_tiles`` is the edge,
    in tiles, of the cells the lists are binned into (0: the library's
    default; ``autotune.tune_cells`` picks one per workload).  ``blend_shape``
    (SGR_BLEND_STRIP16 / SGR_BLEND_PATCH8) and ``tile_schedule``
    (SGR_SCHEDULE_GRID / SGR_SCHEDULE_QUEUE) choose how the blends group
    pixels into warps and hand tiles to CTAs, ``stage_entries`` (0 /
    SGR_STAGE_DEFAULT / SGR_STAGE_SMALL) how many list entries they stage in
    shared memory at a time; results do not depend on them
    (``autotune.tune_blend`` picks them per workload)."""
    lib = L.load()
    b, keep, t = make_batch(variant, means3D, opacities, shs, colors_precomp, scales, rotations, transmat_precomp,
                            semantics, vs, bg, sh_degree, scale_modifier, prefiltered, tables, cell_tiles,
                            blend_shape, tile_schedule, stage_entries)
    device = means3D.device
    s0 = L.Sizes()
    L.check(lib.sgr_query_sizes(C.byref(b), 0, C.byref(s0)), "sgr_query_sizes")
    geom = torch.empty(max(1, s0.geom_bytes), dtype=torch.uint8, device=device)
    scratch = torch.empty(max(1, s0.fwd_scratch_bytes), dtype=torch.uint8, device=device)
    st = _stream()
    L.check(lib.sgr_forward_geometry(C.byref(b), geom.data_ptr(), scratch.data_ptr(), s0.fwd_scratch_bytes, None,
                                     st), "sgr_forward_geometry")
    if bin_capacity is None:
        pin = _pinned(device)
        pin.copy_(geom[s0.off_status:s0.off_status + L.STATUS_BYTES], non_blocking=True)
        ev = torch.cuda.Event()
        ev.record()
        ev.synchronize()
        _, flags, nbins = read_status(pin)
        if flags & L.SGR_FLAG_PREFILTERED:
            raise RuntimeError("Point is filtered although prefiltered is set. This shouldn't happen!")
        if nbins >= 2 ** 31:
            raise RuntimeError(f"{nbins} (surfel, cell) entries exceed the 2^31 - 1 list limit")
        cap = nbins
    else:
        cap = int(bin_capacity)
    bins = torch.empty(max(1, cap), dtype=torch.int32, device=device)
    V, H, W = b.num_views, b.height, b.width
    NO = 7 if variant == L.SGR_VARIANT_PLAIN else 8
    color = torch.empty((V, 3, H, W), dtype=torch.float32, device=device)
    others = torch.empty((V, NO, H, W), dtype=torch.float32, device=device)
    semantic = None
    if variant == L.SGR_VARIANT_PART:
        semantic = torch.empty((V, b.semantic_channels, H, W), dtype=torch.float32, device=device)
    radii = torch.empty(b.num_records, dtype=torch.int32, device=device)     # the library writes every record
    out = L.FwdOutputs(color.data_ptr(), others.data_ptr(), _ptr(semantic), radii.data_ptr())
    L.check(lib.sgr_forward_raster(C.byref(b), geom.data_ptr(), bins.data_ptr(), cap, scratch.data_ptr(),
                                   s0.fwd_scratch_bytes, C.byref(out), st), "sgr_forward_raster")
    if status_host is not None:
        status_host.copy_(geom[s0.off_status:s0.off_status + L.STATUS_BYTES], non_blocking=True)
    state = RasterState(variant, b, keep, geom, bins, cap, s0, b.num_surfels, b.num_records, V, b.sh_coeffs,
                        b.semantic_channels)
    return color, others, semantic, radii, state


def read_fragments(status_host: torch.Tensor) -> int:
    """(pixel, list entry) pairs the forward blend visited, summed over the
    batch, from a status copy taken after the forward."""
    return int(status_host[24:32].view(torch.int64)[0])


def read_status(status_host: torch.Tensor):
    """(key count, flags, cell-list entry count) from a status copy."""
    w = status_host[:L.STATUS_BYTES].view(torch.int64)
    return int(w[0]), int(status_host[8:12].view(torch.int32)[0]), int(w[2])


def backward(state: RasterState, dL_dcolor, dL_dothers, dL_dsemantic=None, need=None, out=None):
    """Gradients of every surfel input.  Returns a dict of tensors shaped as
    the reference's backward returns them; ``out`` may name buffers (float32,
    contiguous, of those sizes) to write some of them into instead."""
    lib = L.load()
    b = state.batch
    device = state.geom.device
    P, R, M, S = state.num_surfels, state.num_records, state.sh_coeffs, state.semantic_channels
    st = _stream()
    dL_dcolor = _f32(dL_dcolor)
    dL_dothers = _f32(dL_dothers)
    dL_dsemantic = _f32(dL_dsemantic) if S > 0 else None
    scratch = torch.empty(max(1, state.sizes.bwd_scratch_bytes), dtype=torch.uint8, device=device)
    e = lambda *shape: torch.empty(shape, dtype=torch.float32, device=device)  # noqa: E731
    g = dict(
        dL_dmeans2D=e(R, 3), dL_dcolors=e(P, 3), dL_dopacity=e(P, 1), dL_dmeans3D=e(P, 3), dL_dtransmat=e(R, 9),
        dL_dsh=e(P, M, 3) if M > 0 else e(0), dL_dscales=e(P, 2), dL_drotations=e(P, 4),
        dL_dsemantics=e(P, S) if S > 0 else e(0))
    for k, t in (out or {}).items():
        if t.dtype != torch.float32 or not t.is_contiguous() or t.numel() != g[k].numel():
            raise ValueError(f"output buffer for {k}: float32, contiguous, {g[k].numel()} elements")
        g[k] = t
    inp = L.BwdInputs(dL_dcolor.data_ptr(), dL_dothers.data_ptr(), _ptr(dL_dsemantic))
    out = L.BwdOutputs(*(_ptr(g[k]) for k in ("dL_dmeans2D", "dL_dcolors", "dL_dopacity", "dL_dmeans3D",
                                               "dL_dtransmat", "dL_dsh", "dL_dscales", "dL_drotations",
                                               "dL_dsemantics")))
    L.check(lib.sgr_backward(C.byref(b), state.geom.data_ptr(), state.bins.data_ptr(), state.bin_capacity,
                             scratch.data_ptr(), state.sizes.bwd_scratch_bytes, C.byref(inp), C.byref(out), st),
            "sgr_backward")
    return g


def mark_visible(positions: torch.Tensor, viewmatrix: torch.Tensor, projmatrix: torch.Tensor) -> torch.Tensor:
    lib = L.load()
    pos = _f32(positions)
    P = int(positions.shape[0])
    present = torch.zeros(P, dtype=torch.bool, device=positions.device)
    if P == 0:
        return present
    vm = _f32(viewmatrix.reshape(-1))
    pm = _f32(projmatrix.reshape(-1))
    L.check(lib.sgr_mark_visible(P, pos.data_ptr(), vm.data_ptr(), pm.data_ptr(), present.data_ptr(), _stream()),
            "sgr_mark_visible")
    return present


def tile_lists(state: RasterState):
    """The reference's per-tile lists of the last forward, written out from
    the depth order: (ranges [V*tiles, 2], point_list [K] record ids, K).
    Synchronises the host (the key count sizes the list)."""
    lib = L.load()
    s = state.sizes
    device = state.geom.device
    pin = _pinned(device)
    pin.copy_(state.geom[s.off_status:s.off_status + L.STATUS_BYTES], non_blocking=True)
    torch.cuda.current_stream().synchronize()
    K = read_status(pin)[0]
    lists = torch.empty(max(1, K), dtype=torch.int32, device=device)
    scratch = torch.empty(max(1, s.tile_list_scratch_bytes), dtype=torch.uint8, device=device)
    L.check(lib.sgr_tile_lists(C.byref(state.batch), state.geom.data_ptr(), lists.data_ptr(), K, scratch.data_ptr(),
                               s.tile_list_scratch_bytes, _stream()), "sgr_tile_lists")
    ntiles = state.num_views * s.tiles_x * s.tiles_y
    ranges = state.geom[s.off_ranges:s.off_ranges + ntiles * 8].view(torch.int32).reshape(ntiles, 2).clone()
    return ranges, lists[:K].clone(), K


def debug_state(state: RasterState) -> dict:
    """Copies of the internal per-view state (for tests and inspection)."""
    s = state.sizes
    g = state.geom
    R, V = state.num_records, state.num_views
    H, W = state.batch.height, state.batch.width

    def sl(off, n, dtype):
        nbytes = n * torch.tensor([], dtype=dtype).element_size()
        return g[off:off + nbytes].view(dtype).clone()

    ranges, point_list, K = tile_lists(state)
    return dict(
        records=sl(s.off_records, R * 24, torch.float32).reshape(R, 24),
        radii=sl(s.off_radii, R, torch.int32),
        tiles_touched=sl(s.off_tiles_touched, R, torch.int32),
        depth_order=sl(s.off_depth_order, R, torch.int32),
        ranges=ranges,
        point_list=point_list,
        num_keys=K,
        final_T=sl(s.off_final_T, V * 3 * H * W, torch.float32).reshape(V, 3, H, W),
        n_contrib=sl(s.off_n_contrib, V * 2 * H * W, torch.int32).reshape(V, 2, H, W),
    )
