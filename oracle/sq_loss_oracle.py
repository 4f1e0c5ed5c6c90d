"""Torch restatement of the reference's block-stage superquadric losses.

TEST INFRASTRUCTURE ONLY: the checker of ``partgs_gb300.sq_losses`` (its
gradients come from torch autograd).  It follows
- games/block_mesh_splatting/utils/pytorch.py (safe_pow, SQRT_EPS 1e-6),
- games/block_mesh_splatting/utils/superquadric.py:25-46 (implicit_sq, safe,
  as_sdf=2),
- games/block_mesh_splatting/scene/block_gaussian_model.py:522-582 (overlap,
  ray_uncoverage, occupancy_opacity, ray_coverage) and :608-622 (the ray
  samples' transform into each block's frame),
- scene/cameras.py:79-96 (cast_rays' depth samples),
in the reference's order of operations, with the random draws passed in.
"""
from __future__ import annotations

import torch
import torch.nn.functional as F

SQRT_EPS = 1e-6


def safe_pow(t, exponent, eps=SQRT_EPS):
    return t.clamp(eps).pow(exponent)


def implicit_sq(points, eps1, eps2):
    """SDF as_sdf=2: points [N, M, 3] in each block's frame, eps [N, 1]."""
    points = points.clamp(-5, 5)
    x2, y2, z2 = [points[..., k].pow(2) for k in range(3)]
    x, y, z = safe_pow(x2, 1 / eps2), safe_pow(y2, 1 / eps1), safe_pow(z2, 1 / eps2)
    res = safe_pow(x + z, eps2 / eps1) + y
    return safe_pow(res, eps1 / 2) - 1


def to_block_frames(points, S, R, T, ratio):
    """[M, 3] world points seen from every block: [N, M, 3]."""
    pts = points[None].expand(S.shape[0], -1, -1)
    return ((pts - T[:, None]) @ R.transpose(1, 2)) / (S[:, None] * ratio)


def ray_points(origin, dirs, jitter, near, far):
    """[rays, C, 3] samples along each ray."""
    C = jitter.shape[1]
    depth = (jitter + torch.arange(C, device=jitter.device, dtype=jitter.dtype)[None, :]) / C * (far - near) + near
    return origin[:, None] + dirs[:, None] * depth[..., None]


def ray_losses(S, R, T, eps1, eps2, occ_logit, ratio, origin, dirs, jitter, label, near, far):
    """(ray_in_mask, ray_out_mask, primitive_opacity)."""
    N, (rays, C) = S.shape[0], jitter.shape
    pts = ray_points(origin, dirs, jitter, near, far).reshape(-1, 3)
    sdf = implicit_sq(to_block_frames(pts, S, R, T, ratio), eps1[:, None], eps2[:, None]).reshape(N, rays, C)
    sdf_rays = sdf.permute(1, 0, 2).flatten(start_dim=1)
    ray_in = torch.clamp(sdf_rays.min(dim=1).values[label > 0.5] - 1e-3, min=0).mean()
    max_values = torch.max(-sdf_rays, dim=1).values * (label < 0.5)
    ray_out = torch.clamp(max_values - 1e-3, min=0).sum() / (label < 0.5).sum()
    alpha = torch.sigmoid(occ_logit)[:, None, None].expand(-1, rays, C)
    alpha = torch.where(sdf <= 1e-8, alpha, 0).permute(1, 0, 2).flatten(start_dim=1).max(dim=1).values
    bce = F.binary_cross_entropy(alpha.clip(1e-3, 1.0 - 1e-3), label).mean()
    return ray_in, ray_out, bce


def overlap_loss(S, R, T, eps1, eps2, occ_logit, ratio, unit, noise, temperature=0.005, max_blocks=1.95):
    """unit [N, P, 3] in [-1, 1]; noise [N]."""
    with torch.no_grad():
        pts = (unit * ratio * S[:, None]) @ R + T[:, None]
    sdf = implicit_sq(to_block_frames(pts.reshape(-1, 3), S, R, T, ratio), eps1[:, None], eps2[:, None])
    occupancy = torch.sigmoid(-sdf / temperature) * torch.sigmoid(occ_logit + noise)[:, None]
    return (occupancy.sum(0) - max_blocks).clamp(0).mean()
