"""Running the reference CUDA rasterisers (built by ``oracle/ref_build.py``)
through their own Python API, and reading their internal per-pixel and
per-tile state back out of the byte buffers they return.

TEST / MEASUREMENT INFRASTRUCTURE ONLY.

The reference's forward returns its work buffers as uint8 tensors
(``rasterize_points.cu:85-134``); their layout is fixed by
``CudaRasterizer::ImageState::fromChunk`` / ``BinningState::fromChunk``
(``cuda_rasterizer/rasterizer_impl.cu:172-194``, both variants):

* image buffer: ``accum_alpha`` float[3·H·W] (final T, M1, M2 planes),
  ``n_contrib`` uint32[2·H·W] (last contributor, median contributor),
  ``ranges`` uint2[H·W] (only the first tiles_x·tiles_y are used), each
  start rounded up to a 128-byte boundary of the absolute address;
* binning buffer: ``point_list`` uint32[num_rendered] first;
* geometry buffer (``GeometryState::fromChunk``, :155-170): depths float[P],
  clamped bool[3P], radii int[P], means2D float2[P], transMat float[9P],
  normal_opacity float4[P], rgb float[3P], tiles_touched uint32[P], ...
"""
from __future__ import annotations

import numpy as np
import torch

from oracle import ref_build

TILE = 16   # BLOCK_X = BLOCK_Y (cuda_rasterizer/config.h:15-16)


class _Capture:
    """Stands in for the reference package's ``_C`` module and keeps the last
    forward's raw return tuple (num_rendered, images, radii, buffers)."""

    def __init__(self, ext):
        self.ext = ext
        self.last = None

    def rasterize_gaussians(self, *args):
        out = self.ext.rasterize_gaussians(*args)
        self.last = out
        return out

    def __getattr__(self, name):
        return getattr(self.ext, name)


def load(variant: str):
    """The reference package (``plain`` or ``part``) with its forward's
    buffers captured; raises ImportError when it was not built."""
    mod = ref_build.load(variant)
    if not isinstance(mod._C, _Capture):
        mod._C = _Capture(mod._C)
    return mod


def available() -> bool:
    return all(ref_build.available(v) for v in ref_build.VARIANTS)


def _aligned(base: int, off: int, align: int = 128) -> int:
    return ((base + off + align - 1) & ~(align - 1)) - base


def image_state(img_buffer: torch.Tensor, H: int, W: int):
    """(final_T [3,H,W] float32, n_contrib [2,H,W] int64, ranges [tiles,2])."""
    N = H * W
    base = img_buffer.data_ptr()
    buf = img_buffer.detach().cpu().numpy()
    o_a = _aligned(base, 0)
    o_n = _aligned(base, o_a + 12 * N)
    o_r = _aligned(base, o_n + 8 * N)
    final_T = buf[o_a:o_a + 12 * N].view(np.float32).reshape(3, H, W).copy()
    n_contrib = buf[o_n:o_n + 8 * N].view(np.uint32).reshape(2, H, W).astype(np.int64)
    tiles = ((W + TILE - 1) // TILE) * ((H + TILE - 1) // TILE)
    ranges = buf[o_r:o_r + 8 * tiles].view(np.uint32).reshape(tiles, 2).astype(np.int64)
    return final_T, n_contrib, ranges


def geometry_state(geom_buffer: torch.Tensor, P: int) -> dict:
    """Per-surfel preprocess outputs of the forward: depths, radii, means2D,
    transMat (row-major 3x3 per surfel), normal_opacity, rgb, tiles_touched."""
    base = geom_buffer.data_ptr()
    buf = geom_buffer.detach().cpu().numpy()
    out, off = {}, 0
    for name, n, dt, shape in (("depths", P, np.float32, (P,)), ("clamped", 3 * P, np.uint8, (P, 3)),
                               ("radii", P, np.int32, (P,)), ("means2D", 2 * P, np.float32, (P, 2)),
                               ("transmat", 9 * P, np.float32, (P, 9)),
                               ("normal_opacity", 4 * P, np.float32, (P, 4)), ("rgb", 3 * P, np.float32, (P, 3)),
                               ("tiles_touched", P, np.uint32, (P,))):
        o = _aligned(base, off)
        nbytes = n * np.dtype(dt).itemsize
        out[name] = buf[o:o + nbytes].view(dt).reshape(shape).copy()
        off = o + nbytes
    return out


def point_list(binning_buffer: torch.Tensor, num_rendered: int) -> np.ndarray:
    base = binning_buffer.data_ptr()
    o = _aligned(base, 0)
    buf = binning_buffer.detach().cpu().numpy()
    return buf[o:o + 4 * num_rendered].view(np.uint32).astype(np.int64).copy()


def settings(mod, cam, bg, sh_degree=3, scale_modifier=1.0, device="cuda"):
    """The reference's GaussianRasterizationSettings for a PinholeCamera."""
    return mod.GaussianRasterizationSettings(
        image_height=cam.height, image_width=cam.width, tanfovx=cam.tanfovx, tanfovy=cam.tanfovy,
        bg=torch.as_tensor(bg, dtype=torch.float32, device=device), scale_modifier=scale_modifier,
        viewmatrix=torch.as_tensor(cam.world_view_transform, dtype=torch.float32, device=device),
        projmatrix=torch.as_tensor(cam.full_proj_transform, dtype=torch.float32, device=device),
        sh_degree=sh_degree, campos=torch.as_tensor(cam.camera_center, dtype=torch.float32, device=device),
        prefiltered=False, debug=False)


def render(variant, cam, bg, means3D, opacities, shs=None, colors_precomp=None, scales=None, rotations=None,
           transmat_precomp=None, semantics=None, sh_degree=3, scale_modifier=1.0, upstream=None):
    """One forward (and, with ``upstream``, one backward) through the
    reference's own ``GaussianRasterizer``.

    ``upstream`` = (dL/dcolor [3,H,W], dL/dallmap [7|8,H,W], dL/dsemantic
    [S,H,W] or None).  Returns a dict of numpy arrays: color, allmap,
    semantic (part), radii, final_T, n_contrib, ranges, point_list,
    num_rendered, and the gradients (dL_d<name>) of the given inputs."""
    mod = load(variant)
    rs = settings(mod, cam, bg, sh_degree, scale_modifier)
    leaf = {}

    def lf(name, t):
        if t is None:
            return None
        t = t.detach().float().cuda().contiguous().requires_grad_(upstream is not None)
        leaf[name] = t
        return t

    m3 = lf("means3D", means3D)
    m2 = torch.zeros_like(m3, requires_grad=upstream is not None)
    leaf["means2D"] = m2
    kw = dict(means3D=m3, means2D=m2, opacities=lf("opacity", opacities), shs=lf("sh", shs),
              colors_precomp=lf("colors", colors_precomp), scales=lf("scales", scales),
              rotations=lf("rotations", rotations), cov3D_precomp=lf("transmat", transmat_precomp))
    rast = mod.GaussianRasterizer(rs)
    if variant == "part":
        kw["semantics"] = lf("semantics", semantics)
        color, semantic, radii, allmap = rast(**kw)
    else:
        color, radii, allmap = rast(**kw)
        semantic = None
    raw = mod._C.last
    num_rendered = int(raw[0])
    img_buf, bin_buf, geom_buf = raw[-1], raw[-2], raw[-3]
    torch.cuda.synchronize()
    final_T, n_contrib, ranges = image_state(img_buf, cam.height, cam.width)
    out = dict(color=color.detach().cpu().numpy(), allmap=allmap.detach().cpu().numpy(),
               radii=radii.cpu().numpy().astype(np.int64), final_T=final_T, n_contrib=n_contrib, ranges=ranges,
               point_list=point_list(bin_buf, num_rendered), num_rendered=num_rendered)
    geo = geometry_state(geom_buf, int(m3.shape[0]))
    out.update({"geom_" + k: v for k, v in geo.items()})
    if semantic is not None:
        out["semantic"] = semantic.detach().cpu().numpy()
    if upstream is not None:
        dcol, doth, dsem = upstream
        loss = (color * torch.as_tensor(dcol, device="cuda")).sum() + \
            (allmap * torch.as_tensor(doth, device="cuda")).sum()
        if semantic is not None and dsem is not None:
            loss = loss + (semantic * torch.as_tensor(dsem, device="cuda")).sum()
        loss.backward()
        torch.cuda.synchronize()
        for k, t in leaf.items():
            if t is not None and t.grad is not None:
                out["dL_d" + k] = t.grad.detach().cpu().numpy()
    return out
