"""Many views (and many scenes) in one launch sequence.

``MultiViewRasterizer`` rasterises every camera of a set in one call of the
library: one preprocess over all (surfel, view) records, one depth order,
one set of cell lists over all views and one blend launch over all tiles
of all views; the backward sums each surfel's per-view gradients on the
device.  With ``bin_capacity`` set, no call synchronises the host, so a
whole training step built on it can be captured in a CUDA graph
(``torch.cuda.graph``); the counts and overflow flag of the last forward
are then read from ``status`` after the step.

Scenes of different sizes are batched the same way: pass ``scene_sizes``
(surfels per scene, surfels concatenated) and ``scene_views`` (cameras per
scene, cameras grouped by scene).
"""
from __future__ import annotations

import torch

from . import _lib as L
from . import raster as _r


class _MultiViewFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, means3D, opacities, shs, scales, rotations, colors_precomp, semantics, cfg):
        color, others, semantic, radii, state = cfg.forward_state(means3D, opacities, shs, scales, rotations,
                                                                  colors_precomp, semantics)
        ctx.state = state
        ctx.cfg = cfg
        ctx.op_shape = opacities.shape
        ctx.has = (shs is not None, colors_precomp is not None, semantics is not None)
        ctx.mark_non_differentiable(radii)
        if semantic is None:
            semantic = torch.empty(0, device=means3D.device)
        return color, others, semantic, radii

    @staticmethod
    def backward(ctx, d_color, d_others, d_semantic, d_radii):
        g = ctx.cfg.backward_state(ctx.state, d_color, d_others, d_semantic if ctx.has[2] else None)
        return (g["dL_dmeans3D"], g["dL_dopacity"].reshape(ctx.op_shape),
                g["dL_dsh"] if ctx.has[0] else None, g["dL_dscales"], g["dL_drotations"],
                g["dL_dcolors"] if ctx.has[1] else None,
                g["dL_dsemantics"] if ctx.has[2] else None, None)


class MultiViewRasterizer:
    """Rasterises a fixed set of cameras; tables and camera tensors are built
    once, so calls make no host-to-device copies."""

    def __init__(self, cameras, bg, sh_degree=3, variant=L.SGR_VARIANT_PLAIN, bin_capacity=None,
                 scene_sizes=None, scene_views=None, num_surfels=None, device="cuda", cell_tiles=0, blend_shape=0,
                 tile_schedule=0, stage_entries=0):
        dev = torch.device(device)
        self.cameras = list(cameras)
        self.variant = variant
        self.sh_degree = sh_degree
        self.bin_capacity = bin_capacity
        self.cell_tiles = cell_tiles
        self.blend_shape = blend_shape          # L.SGR_BLEND_*
        self.tile_schedule = tile_schedule      # L.SGR_SCHEDULE_*
        self.stage_entries = stage_entries      # 0 or L.SGR_STAGE_*
        self.bg = torch.as_tensor(bg, dtype=torch.float32, device=dev)
        vm = torch.stack([torch.as_tensor(c.world_view_transform, dtype=torch.float32) for c in cameras])
        pm = torch.stack([torch.as_tensor(c.full_proj_transform, dtype=torch.float32) for c in cameras])
        cp = torch.stack([torch.as_tensor(c.camera_center, dtype=torch.float32) for c in cameras])
        H = {c.height for c in cameras}
        W = {c.width for c in cameras}
        if len(H) != 1 or len(W) != 1:
            raise ValueError("all cameras of a batch share one image size")
        self.viewset = _r.ViewSet(vm.reshape(-1, 16).to(dev), pm.reshape(-1, 16).to(dev), cp.to(dev),
                                  [(c.tanfovx, c.tanfovy) for c in cameras], H.pop(), W.pop(),
                                  scene_sizes, scene_views)
        P = num_surfels if num_surfels is not None else (sum(scene_sizes) if scene_sizes else None)
        self.tables = _r._tables(variant, P, self.viewset, dev) if P is not None else None
        self.status = torch.zeros(L.STATUS_BYTES, dtype=torch.uint8).pin_memory()
        self.sticky = torch.zeros(2, dtype=torch.int64, device=dev)   # see sticky_counts()
        self.last_means2D_grad = None
        self.last_state = None

    @property
    def num_views(self):
        return len(self.cameras)

    def set_capacity(self, bin_capacity):
        self.bin_capacity = bin_capacity

    def sticky_counts(self, reset: bool = False):
        """(flags OR-ed over every forward since the last reset, largest
        cell-list entry count among them); synchronises with the device."""
        flags, most = (int(x) for x in self.sticky.tolist())
        if reset:
            self.sticky.zero_()
        return flags, most

    def accumulate_status(self, state):
        """Folds the status word of ``state``'s workspace into ``self.sticky``
        (one library kernel on the current stream)."""
        lib = L.load()
        st = state.geom[state.sizes.off_status:state.sizes.off_status + L.STATUS_BYTES]
        L.check(lib.sgr_status_accumulate(st.data_ptr(), self.sticky.data_ptr(), _r._stream()),
                "sgr_status_accumulate")

    def counts(self):
        """(key count, flags, cell-list entry count) of the last forward;
        valid once the stream has passed that forward."""
        return _r.read_status(self.status)

    def fragments(self):
        """(pixel, list entry) pairs the last forward visited; valid once the
        stream has passed that forward."""
        return _r.read_fragments(self.status)

    def _refresh_tables(self, means3D):
        if self.tables is None or self.tables[3] != int(means3D.shape[0]) * self.num_views and \
                self.viewset.scene_sizes is None:
            self.tables = _r._tables(self.variant, int(means3D.shape[0]), self.viewset, means3D.device)

    def forward_state(self, means3D, opacities, shs=None, scales=None, rotations=None, colors_precomp=None,
                      semantics=None):
        """The forward without autograd: (color, others, semantic, radii,
        state), ``state`` to pass to ``backward_state``."""
        self._refresh_tables(means3D)
        color, others, semantic, radii, state = _r.forward(
            self.variant, means3D, opacities, shs, colors_precomp, scales, rotations, None, semantics, self.viewset,
            self.bg, self.sh_degree, 1.0, False, bin_capacity=self.bin_capacity, tables=self.tables,
            status_host=self.status, cell_tiles=self.cell_tiles, blend_shape=self.blend_shape,
            tile_schedule=self.tile_schedule, stage_entries=self.stage_entries)
        self.last_state = state                   # for inspection (bench counters)
        # sticky record of every forward since the last reset: flags OR-ed,
        # largest cell-list entry count (device side, so captured steps keep it)
        self.accumulate_status(state)
        return color, others, semantic, radii, state

    def backward_state(self, state, d_color, d_others, d_semantic=None, out=None):
        """The backward of a ``forward_state`` call without autograd: the
        gradient dict of ``raster.backward`` (``out``: buffers to write some
        of them into)."""
        g = _r.backward(state, d_color, d_others, d_semantic, out=out)
        self.accumulate_status(state)             # flags the backward raised
        self.last_means2D_grad = g["dL_dmeans2D"]
        return g

    def __call__(self, means3D, opacities, shs=None, scales=None, rotations=None, colors_precomp=None,
                 semantics=None):
        color, others, semantic, radii = _MultiViewFn.apply(means3D, opacities, shs, scales, rotations,
                                                            colors_precomp, semantics, self)
        return color, others, (semantic if semantics is not None else None), radii
