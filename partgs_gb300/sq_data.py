"""Synthetic superquadric scenes for the proposal network.

A scene is a union of K in [1, 8] superquadrics drawn as in the block-level
workload: semi-axes U[0.1, 0.5], exponents U[0.2, 1.8], random unit
quaternions, centres uniform in the unit ball.  Its input is what the
block-level stage starts from: points back-projected from a rendered median
depth map.  Every scene is bound to surfels by the CUDA binding
(``SuperquadricBinding``) and all scenes are rasterised in one multi-scene
launch sequence (one camera each), the median depth back-projected along the
camera rays (utils/point_utils.py:4-20) and 2,048 points sampled from the
covered pixels.

Labels are the generating parameters, slots sorted by the centre's x
coordinate and padded to 8 with ``exist = 0``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import torch

from .batched import MultiViewRasterizer
from .binding import SuperquadricBinding
from .cameras import orbit_cameras
from .surfel_step import DepthNormals

RATIO, SMIN = 0.25, 0.2          # ratio_block_scene, scale_block_min (arguments/__init__.py)
MAX_SQ = 8


def grid_topology(n_eta: int, n_omega: int):
    """(eta, omega) of a half-cell-offset parameter grid and one triangle per
    node: (node, its eta neighbour, its omega neighbour), omega wrapped."""
    eta = -math.pi / 2 + (np.arange(n_eta) + 0.5) * math.pi / n_eta
    omega = -math.pi + (np.arange(n_omega) + 0.25) * 2 * math.pi / n_omega
    E, O_ = np.meshgrid(eta, omega, indexing="ij")
    a, b = np.meshgrid(np.arange(n_eta), np.arange(n_omega), indexing="ij")
    an = np.where(a + 1 < n_eta, a + 1, a - 1)
    faces = np.stack([a * n_omega + b, an * n_omega + b, a * n_omega + (b + 1) % n_omega], -1).reshape(-1, 3)
    return E.reshape(-1), O_.reshape(-1), faces


@dataclass
class SQBatch:
    """Per scene, 8 slots: semi-axes [S,8,3], exponents [S,8,2], unit
    quaternions (w, x, y, z; w >= 0) [S,8,4], centres [S,8,3], exist [S,8]."""
    semi: torch.Tensor
    eps: torch.Tensor
    quat: torch.Tensor
    trans: torch.Tensor
    exist: torch.Tensor

    @property
    def counts(self):
        return self.exist.sum(1).long()


def sample_sq_batch(S: int, g: torch.Generator, kmin: int = 1, kmax: int = MAX_SQ) -> SQBatch:
    K = torch.randint(kmin, kmax + 1, (S,), generator=g)
    semi = torch.rand(S, MAX_SQ, 3, generator=g) * 0.4 + 0.1
    eps = torch.rand(S, MAX_SQ, 2, generator=g) * 1.6 + 0.2
    q = torch.randn(S, MAX_SQ, 4, generator=g)
    q = q / q.norm(dim=-1, keepdim=True)
    q = torch.where(q[..., :1] < 0, -q, q)
    c = torch.randn(S, MAX_SQ, 3, generator=g)
    c = c / c.norm(dim=-1, keepdim=True) * torch.rand(S, MAX_SQ, 1, generator=g) ** (1 / 3)
    exist = (torch.arange(MAX_SQ)[None, :] < K[:, None]).float()
    # canonical slot order: existing superquadrics by centre x, then the padding
    key = torch.where(exist > 0, c[..., 0], torch.full_like(c[..., 0], 1e9))
    order = key.argsort(dim=1)
    take = lambda t: torch.gather(t, 1, order[..., None].expand(-1, -1, t.shape[-1]))  # noqa: E731
    return SQBatch(take(semi), take(eps), take(q), take(c), torch.gather(exist, 1, order))


def to_binding_params(semi, eps, quat, trans):
    """The block model's raw parameters (sq_s, sq_eps, sq_r, sq_t) of given
    semi-axes, exponents, quaternions and centres
    (block_gaussian_model.py:189-193, 207-226)."""
    sq_s = torch.log(semi / RATIO - SMIN)
    sq_eps = torch.logit(((eps - 0.1) / 1.8).clamp(1e-6, 1 - 1e-6))
    return sq_s, sq_eps, quat, trans


class SceneRenderer:
    """Renders batches of superquadric scenes to point sets on the GPU."""

    def __init__(self, n_eta: int = 30, n_omega: int = 30, res: int = 96, fovx_deg: float = 50.0,
                 radius: float = 3.0, device="cuda"):
        self.dev = torch.device(device)
        self.res, self.fovx, self.radius = res, fovx_deg, radius
        eta, omega, faces = grid_topology(n_eta, n_omega)
        self.eta = torch.tensor(eta, dtype=torch.float32)
        self.omega = torch.tensor(omega, dtype=torch.float32)
        self.faces = torch.tensor(faces, dtype=torch.int32)
        self.F = faces.shape[0]

    def points(self, batch: SQBatch, n_points: int = 2048, seed: int = 0):
        """(points [S, n_points, 3], covered pixel count [S])."""
        S = batch.exist.shape[0]
        sel = batch.exist.reshape(-1) > 0
        B = int(sel.sum())
        semi, eps = batch.semi.reshape(-1, 3)[sel], batch.eps.reshape(-1, 2)[sel]
        quat, trans = batch.quat.reshape(-1, 4)[sel], batch.trans.reshape(-1, 3)[sel]
        sq_s, sq_eps, sq_r, sq_t = (t.float().to(self.dev) for t in to_binding_params(semi, eps, quat, trans))
        g = torch.Generator().manual_seed(seed)
        alpha = torch.rand(B * self.F, 1, 3, generator=g)
        bind = SuperquadricBinding(self.eta.expand(B, -1).to(self.dev), self.omega.expand(B, -1).to(self.dev),
                                   self.faces.expand(B, -1, -1).contiguous().to(self.dev), alpha.to(self.dev),
                                   torch.ones(B, self.F, 1, device=self.dev), RATIO, SMIN)
        occ = torch.full((B, 1), 4.6, device=self.dev)               # opacity 0.99
        with torch.no_grad():
            xyz, log_s, rot, op = bind(sq_s, sq_r, sq_t, sq_eps, occ)
        cams = orbit_cameras(S, self.radius, self.res, self.res, self.fovx, seed=seed)
        counts = batch.counts.tolist()
        raster = MultiViewRasterizer(cams, [0.0, 0.0, 0.0], 0, scene_sizes=[k * self.F for k in counts],
                                     scene_views=[1] * S, device=self.dev)
        with torch.no_grad():
            _, others, _, _ = raster(xyz, op, None, torch.exp(log_s), rot,
                                     colors_precomp=torch.ones_like(xyz))
        alpha_map, median = others[:, 1], others[:, 5]
        rays = DepthNormals(cams, self.dev)
        pts = median.reshape(S, -1, 1) * rays.rays_d + rays.rays_o[:, None, :]
        valid = ((alpha_map > 0.5) & (median > 0.2)).reshape(S, -1)
        weight = valid.float() + 1e-12
        idx = torch.multinomial(weight, n_points, replacement=True,
                                generator=torch.Generator(device=self.dev).manual_seed(seed))
        return torch.gather(pts, 1, idx[..., None].expand(-1, -1, 3)), valid.sum(1)


def surface_samples(semi, eps, quat, trans, n: int, g: torch.Generator):
    """n points on each superquadric [..., n, 3], (eta, omega) uniform, the
    binding's row-vector transform (v * S) @ R + t."""
    shape = semi.shape[:-1]
    eta = (torch.rand(*shape, n, generator=g) * 2 - 1) * (math.pi / 2) * 0.999
    omega = (torch.rand(*shape, n, generator=g) * 2 - 1) * math.pi
    sp = lambda t, e: torch.sign(t) * torch.abs(t).pow(e)  # noqa: E731
    e1, e2 = eps[..., 0:1], eps[..., 1:2]
    ce, se = sp(torch.cos(eta), e1), sp(torch.sin(eta), e1)
    co, so = sp(torch.cos(omega), e2), sp(torch.sin(omega), e2)
    v = torch.stack([ce * so, se, ce * co], dim=-1) * semi[..., None, :]
    w, x, y, z = quat.unbind(-1)
    R = torch.stack([
        torch.stack([1 - 2 * y * y - 2 * z * z, 2 * x * y - 2 * z * w, 2 * x * z + 2 * y * w], -1),
        torch.stack([2 * x * y + 2 * z * w, 1 - 2 * x * x - 2 * z * z, 2 * y * z - 2 * x * w], -1),
        torch.stack([2 * x * z - 2 * y * w, 2 * y * z + 2 * x * w, 1 - 2 * x * x - 2 * y * y], -1)], -2)
    return v @ R + trans[..., None, :]
