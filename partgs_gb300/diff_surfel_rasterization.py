"""Drop-in for the reference's ``diff_surfel_rasterization`` package (plain variant).

Same module-level names, NamedTuple fields, argument names and defaults,
return arity and channel layout as
submodules/diff-surfel-rasterization/diff_surfel_rasterization/__init__.py:
``GaussianRasterizer(...)(means3D, means2D, opacities, shs, colors_precomp,
scales, rotations, cov3D_precomp)`` returns ``(color [3,H,W], radii [P] int32,
allmap [7,H,W])`` with allmap = (expected depth, alpha, normal xyz, median
depth, distortion).  The work runs in libsgr.so on the GB300; there is no
other compute path.
"""
from __future__ import annotations

from typing import NamedTuple

import torch
import torch.nn as nn

from . import _lib as L
from . import raster as _r


def cpu_deep_copy_tuple(input_tuple):
    return tuple(item.cpu().clone() if isinstance(item, torch.Tensor) else item for item in input_tuple)


def _viewset(rs) -> _r.ViewSet:
    return _r.ViewSet(rs.viewmatrix.reshape(1, 16), rs.projmatrix.reshape(1, 16), rs.campos.reshape(1, 3),
                      [(rs.tanfovx, rs.tanfovy)], int(rs.image_height), int(rs.image_width))


def _none_if_empty(t):
    return None if t is None or t.numel() == 0 else t


def rasterize_gaussians(means3D, means2D, sh, colors_precomp, opacities, scales, rotations, cov3Ds_precomp,
                        raster_settings):
    return _RasterizeGaussians.apply(means3D, means2D, sh, colors_precomp, opacities, scales, rotations,
                                     cov3Ds_precomp, raster_settings)


class _RasterizeGaussians(torch.autograd.Function):
    """Autograd contract of P0/diff_surfel_rasterization/__init__.py:44-156."""

    @staticmethod
    def forward(ctx, means3D, means2D, sh, colors_precomp, opacities, scales, rotations, cov3Ds_precomp,
                raster_settings):
        rs = raster_settings
        args = (rs.bg, means3D, colors_precomp, opacities, scales, rotations, rs.scale_modifier, cov3Ds_precomp,
                rs.viewmatrix, rs.projmatrix, rs.tanfovx, rs.tanfovy, rs.image_height, rs.image_width, sh,
                rs.sh_degree, rs.campos, rs.prefiltered, rs.debug)
        try:
            color, others, _, radii, state = _r.forward(
                L.SGR_VARIANT_PLAIN, means3D, opacities, _none_if_empty(sh), _none_if_empty(colors_precomp),
                _none_if_empty(scales), _none_if_empty(rotations), _none_if_empty(cov3Ds_precomp), None,
                _viewset(rs), rs.bg, rs.sh_degree, rs.scale_modifier, rs.prefiltered)
        except Exception:
            if rs.debug:
                torch.save(cpu_deep_copy_tuple(args), "snapshot_fw.dump")
                print("\nAn error occured in forward. Please forward snapshot_fw.dump for debugging.")
            raise
        ctx.raster_settings = rs
        ctx.state = state
        ctx.shapes = (means3D.shape[0], None if sh is None else tuple(sh.shape))
        ctx.save_for_backward(colors_precomp, means3D, scales, rotations, cov3Ds_precomp, radii, sh)
        return color[0], radii, others[0]

    @staticmethod
    def backward(ctx, grad_out_color, grad_radii, grad_depth):
        rs = ctx.raster_settings
        try:
            g = _r.backward(ctx.state, grad_out_color.unsqueeze(0), grad_depth.unsqueeze(0))
        except Exception:
            if rs.debug:
                torch.save(cpu_deep_copy_tuple((grad_out_color, grad_depth)), "snapshot_bw.dump")
                print("\nAn error occured in backward. Writing snapshot_bw.dump for debugging.\n")
            raise
        P = ctx.shapes[0]
        grad_sh = g["dL_dsh"] if g["dL_dsh"].numel() else torch.zeros((P, 0, 3), device=g["dL_dcolors"].device)
        return (g["dL_dmeans3D"], g["dL_dmeans2D"], grad_sh, g["dL_dcolors"], g["dL_dopacity"], g["dL_dscales"],
                g["dL_drotations"], g["dL_dtransmat"], None)


class GaussianRasterizationSettings(NamedTuple):
    image_height: int
    image_width: int
    tanfovx: float
    tanfovy: float
    bg: torch.Tensor
    scale_modifier: float
    viewmatrix: torch.Tensor
    projmatrix: torch.Tensor
    sh_degree: int
    campos: torch.Tensor
    prefiltered: bool
    debug: bool


class GaussianRasterizer(nn.Module):
    def __init__(self, raster_settings):
        super().__init__()
        self.raster_settings = raster_settings

    def markVisible(self, positions):
        with torch.no_grad():
            rs = self.raster_settings
            return _r.mark_visible(positions, rs.viewmatrix, rs.projmatrix)

    def forward(self, means3D, means2D, opacities, shs=None, colors_precomp=None, scales=None, rotations=None,
                cov3D_precomp=None):
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
        return rasterize_gaussians(means3D, means2D, shs, colors_precomp, opacities, scales, rotations,
                                   cov3D_precomp, raster_settings)
