"""Block-stage superquadric losses on the GPU, the regularisers of the
reference's BlockGaussianModel.summarize_losses
(games/block_mesh_splatting/scene/block_gaussian_model.py:514-648):

- ``ray_in_mask`` (ray coverage): rays through the object mask should meet a
  block, mean of clamp(min SDF along the ray - 1e-3, 0);
- ``ray_out_mask`` (ray uncoverage): rays outside it should meet none;
- ``primitive_opacity``: BCE between the highest occupancy alpha among the
  blocks a ray enters and the mask;
- ``overlap``: random points of every block should lie in at most
  OVERLAP_N_BLOCKS blocks (soft occupancy, temperature 0.005);
- ``parsimony`` and ``scale_reg`` are per-block elementwise terms and stay in
  torch.

The four SDF-based losses are one fused forward (``sgr_sq_losses_forward``,
two launches) and one fused backward (two launches) over all rays, samples,
points and blocks.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import torch

from . import _lib as L

OVERLAP_N_POINTS = 2048
OVERLAP_N_BLOCKS = 1.95
OVERLAP_TEMPERATURE = 0.005
MAX_BLOCKS = 64
NEAR_FAR = {"dtu": (0.5, 3.5), "blender": (2.0, 5.0), "blendermvs": (1.0, 3.0)}   # summarize_losses
_p = C.c_void_p


class SQLossArgs(C.Structure):
    _fields_ = [("n_blocks", C.c_int32), ("ratio", C.c_float),
                ("S", _p), ("R", _p), ("T", _p), ("eps1", _p), ("eps2", _p), ("occ_logit", _p),
                ("n_rays", C.c_int32), ("n_samples", C.c_int32),
                ("ray_origin", _p), ("ray_dir", _p), ("ray_jitter", _p), ("ray_label", _p),
                ("near", C.c_float), ("far", C.c_float),
                ("n_overlap", C.c_int32), ("overlap_unit", _p), ("overlap_noise", _p),
                ("overlap_temperature", C.c_float), ("overlap_max_blocks", C.c_float),
                ("scratch", _p), ("scratch_bytes", C.c_size_t), ("losses", _p),
                ("d_S", _p), ("d_R", _p), ("d_T", _p), ("d_eps1", _p), ("d_eps2", _p), ("d_occ_logit", _p)]


def _lib():
    lib = L.load()
    A = C.POINTER(SQLossArgs)
    lib.sgr_sq_scratch_bytes.restype = C.c_size_t
    lib.sgr_sq_scratch_bytes.argtypes = [A]
    lib.sgr_sq_losses_forward.restype = C.c_int
    lib.sgr_sq_losses_forward.argtypes = [A, _p]
    lib.sgr_sq_losses_backward.restype = C.c_int
    lib.sgr_sq_losses_backward.argtypes = [A, _p, _p]
    lib.sgr_sq_sdf.restype = C.c_int
    lib.sgr_sq_sdf.argtypes = [A, _p, C.c_int64, _p, _p]
    return lib


@dataclass
class RaySamples:
    """One view's rays (scene/cameras.py:79-96): per ray its origin, direction
    and uniform jitter of its ``n_samples`` stratified depths in [near, far],
    and the mask value at its pixel."""
    origin: torch.Tensor   # [R, 3]
    dirs: torch.Tensor     # [R, 3]
    jitter: torch.Tensor   # [R, C]
    label: torch.Tensor    # [R]
    near: float
    far: float
    ray_idx: torch.Tensor | None = None


@dataclass
class OverlapSamples:
    unit: torch.Tensor     # [N, P, 3] uniform in [-1, 1]
    noise: torch.Tensor    # [N] N(0, 1), added to the occupancy logits
    temperature: float = OVERLAP_TEMPERATURE
    max_blocks: float = OVERLAP_N_BLOCKS


def intrinsics(height: int, width: int, fovx: float, fovy: float, device="cuda") -> torch.Tensor:
    """The reference camera's K (scene/cameras.py:35-40)."""
    K = torch.zeros(3, 3, dtype=torch.float32)
    K[0, 0] = (width / 2.0) / math.tan(fovx / 2.0)
    K[1, 1] = (height / 2.0) / math.tan(fovy / 2.0)
    K[0, 2] = width / 2.0
    K[1, 2] = height / 2.0
    K[2, 2] = 1.0
    return K.to(device)


def ray_geometry(K, world_view_transform, height: int, width: int, ray_idx):
    """Origins and directions of the rays through pixels ``ray_idx`` (row-major
    index), scene/cameras.py:65-90: pixel centres through K^-1, to the world by
    the inverted world-to-view pose; direction = pixel point - camera centre.
    world_view_transform is the transposed (row-vector) 4x4."""
    xy = torch.stack([ray_idx % width, ray_idx // width], -1).float().add_(0.5)
    pts = torch.cat([xy, torch.ones_like(xy[..., :1])], -1) @ K.inverse().transpose(-1, -2)
    pose = world_view_transform.transpose(-1, -2)[:3, :]
    R_inv = pose[..., :3].transpose(-1, -2)
    t_inv = (-R_inv @ pose[..., 3:])[..., 0]
    pose_inv = torch.cat([R_inv, t_inv[..., None]], -1)

    def cam2world(X):
        return torch.cat([X, torch.ones_like(X[..., :1])], -1) @ pose_inv.transpose(-1, -2)

    grid = cam2world(pts)
    center = cam2world(torch.zeros_like(grid))
    return center, grid - center


def cast_rays(K, world_view_transform, height: int, width: int, mask, near: float, far: float,
              num_samples: int = 128, num_rays: int = 2048, generator=None) -> RaySamples:
    """scene/cameras.py:79-96: ``num_rays`` random pixels, their rays, and the
    jitter of ``num_samples`` stratified depth samples in [near, far]; the
    labels are the mask [H, W] at those pixels."""
    dev = K.device
    ray_idx = torch.randperm(height * width, device=dev, generator=generator)[:num_rays]
    origin, dirs = ray_geometry(K, world_view_transform, height, width, ray_idx)
    jitter = torch.rand(ray_idx.shape[0], num_samples, device=dev, generator=generator)
    label = mask.reshape(-1)[ray_idx].float()
    return RaySamples(origin.contiguous(), dirs.contiguous(), jitter, label, near, far, ray_idx)


def overlap_samples(n_blocks: int, n_points: int = OVERLAP_N_POINTS, device="cuda", generator=None):
    unit = torch.rand(n_blocks, n_points, 3, device=device, generator=generator) * 2 - 1
    noise = torch.randn(n_blocks, device=device, generator=generator)
    return OverlapSamples(unit, noise)


def _args(S, R, T, eps1, eps2, occ, ratio, rays, ovl):
    a = SQLossArgs()
    a.n_blocks = S.shape[0]
    a.ratio = float(ratio)
    a.S, a.R, a.T = S.data_ptr(), R.data_ptr(), T.data_ptr()
    a.eps1, a.eps2, a.occ_logit = eps1.data_ptr(), eps2.data_ptr(), occ.data_ptr()
    if rays is not None:
        a.n_rays, a.n_samples = rays.jitter.shape
        a.ray_origin, a.ray_dir = rays.origin.data_ptr(), rays.dirs.data_ptr()
        a.ray_jitter, a.ray_label = rays.jitter.data_ptr(), rays.label.data_ptr()
        a.near, a.far = float(rays.near), float(rays.far)
    if ovl is not None:
        a.n_overlap = ovl.unit.shape[1]
        a.overlap_unit, a.overlap_noise = ovl.unit.data_ptr(), ovl.noise.data_ptr()
        a.overlap_temperature, a.overlap_max_blocks = float(ovl.temperature), float(ovl.max_blocks)
    return a


def _prep(t, shape):
    t = t.detach().float().contiguous()
    assert tuple(t.shape) == shape, (tuple(t.shape), shape)
    return t


class _SQLosses(torch.autograd.Function):
    @staticmethod
    def forward(ctx, S, R, T, eps1, eps2, occ_logit, ratio, rays, ovl):
        lib = _lib()
        N = S.shape[0]
        if not 1 <= N <= MAX_BLOCKS:
            raise ValueError(f"1..{MAX_BLOCKS} blocks supported, got {N}")
        t = [_prep(S, (N, 3)), _prep(R, (N, 3, 3)), _prep(T, (N, 3)), _prep(eps1.reshape(-1), (N,)),
             _prep(eps2.reshape(-1), (N,)), _prep(occ_logit.reshape(-1), (N,))]
        if rays is not None:
            rays = RaySamples(*(x.float().contiguous() if torch.is_tensor(x) else x
                                for x in (rays.origin, rays.dirs, rays.jitter, rays.label, rays.near, rays.far)))
        if ovl is not None:
            ovl = OverlapSamples(ovl.unit.float().contiguous(), ovl.noise.float().reshape(-1).contiguous(),
                                 ovl.temperature, ovl.max_blocks)
        a = _args(*t, ratio, rays, ovl)
        scratch = torch.empty(lib.sgr_sq_scratch_bytes(C.byref(a)), dtype=torch.uint8, device=S.device)
        losses = torch.empty(4, device=S.device)
        a.scratch, a.scratch_bytes, a.losses = scratch.data_ptr(), scratch.numel(), losses.data_ptr()
        L.check(lib.sgr_sq_losses_forward(C.byref(a), torch.cuda.current_stream().cuda_stream),
                "sgr_sq_losses_forward")
        ctx.keep = (t, rays, ovl, scratch, a, occ_logit.shape, eps1.shape, eps2.shape)
        return losses

    @staticmethod
    def backward(ctx, d_losses):
        lib = _lib()
        t, rays, ovl, scratch, a, occ_shape, e1_shape, e2_shape = ctx.keep
        N = t[0].shape[0]
        dev = t[0].device
        g = [torch.empty(N, 3, device=dev), torch.empty(N, 3, 3, device=dev), torch.empty(N, 3, device=dev),
             torch.empty(N, device=dev), torch.empty(N, device=dev), torch.empty(N, device=dev)]
        a.d_S, a.d_R, a.d_T = g[0].data_ptr(), g[1].data_ptr(), g[2].data_ptr()
        a.d_eps1, a.d_eps2, a.d_occ_logit = g[3].data_ptr(), g[4].data_ptr(), g[5].data_ptr()
        d = d_losses.float().contiguous()
        L.check(lib.sgr_sq_losses_backward(C.byref(a), d.data_ptr(), torch.cuda.current_stream().cuda_stream),
                "sgr_sq_losses_backward")
        return (g[0], g[1], g[2], g[3].reshape(e1_shape), g[4].reshape(e2_shape), g[5].reshape(occ_shape),
                None, None, None)


def sq_losses(S, R, T, eps1, eps2, occ_logit, ratio: float, rays: RaySamples | None = None,
              ovl: OverlapSamples | None = None) -> torch.Tensor:
    """[ray_in_mask, ray_out_mask, primitive_opacity, overlap] (a term whose
    samples are None is 0), differentiable in S, R, T, eps1, eps2, occ_logit."""
    return _SQLosses.apply(S, R, T, eps1, eps2, occ_logit, ratio, rays, ovl)


def quaternion_to_rotation_matrix(q: torch.Tensor) -> torch.Tensor:
    """[N,4] (w, x, y, z) to [N,3,3], the reference's convention
    (games/block_mesh_splatting/utils/superquadric.py:93-101)."""
    w, x, y, z = q.unbind(-1)
    return torch.stack([1 - 2 * y ** 2 - 2 * z ** 2, 2 * x * y - 2 * z * w, 2 * x * z + 2 * y * w,
                        2 * x * y + 2 * z * w, 1 - 2 * x ** 2 - 2 * z ** 2, 2 * y * z - 2 * x * w,
                        2 * x * z - 2 * y * w, 2 * y * z + 2 * x * w, 1 - 2 * x ** 2 - 2 * y ** 2], -1).view(-1, 3, 3)


def block_frames(sq_s, sq_r, sq_t, sq_eps, scale_block_min: float = 0.2):
    """(S, R, T, eps1, eps2) of the block model's raw parameters, as
    BlockGaussianModel builds _blocks_SRT and _blocks_eps
    (block_gaussian_model.py:111-121, 189-192, 220-222); differentiable."""
    S = torch.exp(sq_s) + scale_block_min
    R = quaternion_to_rotation_matrix(torch.nn.functional.normalize(sq_r, dim=-1))
    eps1, eps2 = (torch.sigmoid(sq_eps) * 1.8 + 0.1).unbind(-1)
    return S, R, sq_t, eps1, eps2


def implicit_sq(points, S, R, T, eps1, eps2, ratio: float) -> torch.Tensor:
    """SDF (as_sdf=2) of world points [M, 3] to every block: [N, M] (no gradient)."""
    lib = _lib()
    N = S.shape[0]
    t = [_prep(S, (N, 3)), _prep(R, (N, 3, 3)), _prep(T, (N, 3)), _prep(eps1.reshape(-1), (N,)),
         _prep(eps2.reshape(-1), (N,)), torch.zeros(N, device=S.device)]
    a = _args(*t, ratio, None, None)
    pts = points.detach().float().contiguous()
    out = torch.empty(N, pts.shape[0], device=S.device)
    L.check(lib.sgr_sq_sdf(C.byref(a), pts.data_ptr(), pts.shape[0], out.data_ptr(),
                           torch.cuda.current_stream().cuda_stream), "sgr_sq_sdf")
    return out


def regularisers(sq_occ, get_scaling, weights: dict, losses: torch.Tensor | None = None):
    """The weighted sum summarize_losses adds for the block model: scale
    regulariser (0.1 sum clamp(S - 3, 0)), parsimony (0.002 mean sqrt(alpha)),
    and the fused losses with the reference's weights (coverage 10,
    uncoverage 100, occupancy 0.02, overlap 2)."""
    total = weights.get("primtive_scale_weight", 0.1) * (get_scaling - 3.0).clamp(min=0.0).sum()
    total = total + weights.get("parsimony_weight", 0.002) * torch.sigmoid(sq_occ).clamp(1e-6).pow(0.5).mean()
    if losses is not None:
        w = torch.tensor([weights.get("ray_coverage_weigth", 10.0), weights.get("ray_uncoverage_weigth", 100.0),
                          weights.get("occupancy_weight", 0.02), weights.get("overlap_weight", 2.0)],
                         device=losses.device)
        total = total + (w * losses).sum()
    return total
