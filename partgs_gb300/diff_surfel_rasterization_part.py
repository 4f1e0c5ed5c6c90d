"""Drop-in for the reference's ``diff_surfel_rasterization_part`` package.

Mirrors submodules/diff-surfel-rasterization_part/diff_surfel_rasterization_part/__init__.py:
``GaussianRasterizer(...)(means3D, means2D, opacities, semantics, shs,
colors_precomp, scales, rotations, cov3D_precomp)`` returns ``(color [3,H,W],
semantic [S,H,W], radii [P] int32, allmap [8,H,W])`` with allmap =
(expected depth, alpha, normal xyz, median depth, distortion, median weight).
At most 16 semantic channels are accepted (the reference's fixed-size
register array, P1/cuda_rasterizer/forward.cu:317, is silently overrun
beyond that; here it is an error).
"""
from __future__ import annotations

import torch
import torch.nn as nn

from . import _lib as L
from . import raster as _r
from .diff_surfel_rasterization import (GaussianRasterizationSettings, _none_if_empty, _viewset,
                                        cpu_deep_copy_tuple)

__all__ = ["GaussianRasterizationSettings", "GaussianRasterizer", "rasterize_gaussians"]


def rasterize_gaussians(means3D, means2D, sh, colors_precomp, opacities, semantics, scales, rotations,
                        cov3Ds_precomp, raster_settings):
    return _RasterizeGaussians.apply(means3D, means2D, sh, colors_precomp, opacities, semantics, scales, rotations,
                                     cov3Ds_precomp, raster_settings)


class _RasterizeGaussians(torch.autograd.Function):
    """Autograd contract of P1/diff_surfel_rasterization_part/__init__.py:44-161."""

    @staticmethod
    def forward(ctx, means3D, means2D, sh, colors_precomp, opacities, semantics, scales, rotations, cov3Ds_precomp,
                raster_settings):
        rs = raster_settings
        if semantics is None or semantics.dim() != 2 or semantics.shape[0] != means3D.shape[0]:
            raise ValueError("semantics must have dimensions (num_points, num_semantic_channels)")
        args = (rs.bg, means3D, colors_precomp, opacities, semantics, scales, rotations, rs.scale_modifier,
                cov3Ds_precomp, rs.viewmatrix, rs.projmatrix, rs.tanfovx, rs.tanfovy, rs.image_height,
                rs.image_width, sh, rs.sh_degree, rs.campos, rs.prefiltered, rs.debug)
        try:
            color, others, semantic, radii, state = _r.forward(
                L.SGR_VARIANT_PART, means3D, opacities, _none_if_empty(sh), _none_if_empty(colors_precomp),
                _none_if_empty(scales), _none_if_empty(rotations), _none_if_empty(cov3Ds_precomp), semantics,
                _viewset(rs), rs.bg, rs.sh_degree, rs.scale_modifier, rs.prefiltered)
        except Exception:
            if rs.debug:
                torch.save(cpu_deep_copy_tuple(args), "snapshot_fw.dump")
                print("\nAn error occured in forward. Please forward snapshot_fw.dump for debugging.")
            raise
        ctx.raster_settings = rs
        ctx.state = state
        ctx.P = means3D.shape[0]
        ctx.save_for_backward(colors_precomp, semantics, means3D, scales, rotations, cov3Ds_precomp, radii, sh)
        return color[0], semantic[0], radii, others[0]

    @staticmethod
    def backward(ctx, grad_out_color, grad_out_semantic, grad_radii, grad_depth):
        rs = ctx.raster_settings
        try:
            g = _r.backward(ctx.state, grad_out_color.unsqueeze(0), grad_depth.unsqueeze(0),
                            grad_out_semantic.unsqueeze(0))
        except Exception:
            if rs.debug:
                torch.save(cpu_deep_copy_tuple((grad_out_color, grad_out_semantic, grad_depth)), "snapshot_bw.dump")
                print("\nAn error occured in backward. Writing snapshot_bw.dump for debugging.\n")
            raise
        P = ctx.P
        grad_sh = g["dL_dsh"] if g["dL_dsh"].numel() else torch.zeros((P, 0, 3), device=g["dL_dcolors"].device)
        grad_sem = g["dL_dsemantics"] if g["dL_dsemantics"].numel() else \
            torch.zeros((P, 0), device=g["dL_dcolors"].device)
        return (g["dL_dmeans3D"], g["dL_dmeans2D"], grad_sh, g["dL_dcolors"], g["dL_dopacity"], grad_sem,
                g["dL_dscales"], g["dL_drotations"], g["dL_dtransmat"], None)


class GaussianRasterizer(nn.Module):
    def __init__(self, raster_settings):
        super().__init__()
        self.raster_settings = raster_settings

    def markVisible(self, positions):
        with torch.no_grad():
            rs = self.raster_settings
            return _r.mark_visible(positions, rs.viewmatrix, rs.projmatrix)

    def forward(self, means3D, means2D, opacities, semantics, shs=None, colors_precomp=None, scales=None,
                rotations=None, cov3D_precomp=None):
        raster_settings = self.raster_settings
        if (shs is None and colors_precomp is None) or (shs is not None and colors_precomp is not None):
            raise Exception('Please provide excatly one of either SHs or precomputed colors!')
        if ((scales is None or rotations is None) and cov3D_precomp is None) or \
                ((scales is not None or rotations is not None) and cov3D_precomp is not None):
            raise Exception('Please provide exactly one of either scale/rotation pair or precomputed 3D covariance!')
        dev = means3D.device
        empty = lambda: torch.empty(0, device=dev)  # noqa: E731
        shs = empty() if shs is None else shs
        colors_precomp = empty() if colors_precomp is None else colors_precomp
        scales = empty() if scales is None else scales
        rotations = empty() if rotations is None else rotations
        cov3D_precomp = empty() if cov3D_precomp is None else cov3D_precomp
        return rasterize_gaussians(means3D, means2D, shs, colors_precomp, opacities, semantics, scales, rotations,
                                   cov3D_precomp, raster_settings)
