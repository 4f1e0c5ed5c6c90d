"""Seeded synthetic surfel scenes in the shapes of the benchmark workloads.

The reference trains on DTU / BlendedMVS / ShapeNet renders, none of which is
available here; these generators stand in for them with the sizes and value
distributions the workloads name:

* ``random_surfels``   4,096 surfels, means U[-1,1]^3, tangent scales
  exp(N(-3, 0.5)), quaternions normalize(N(0,1)^4), opacity sigmoid(N(0,1)),
  degree-3 SH with DC ~ N(0, 0.3) and the rest ~ N(0, 0.05).
* ``superquadric_surfels``   means sampled on a seeded union of random
  superquadric surfaces (``parametric_sq``,
  games/block_mesh_splatting/utils/superquadric.py:10-14) plus N(0, 0.01)
  jitter, other attributes as above (500k surfels for the batched-view step).

Everything is drawn from a CPU ``torch.Generator`` so the same seed gives the
same scene on every machine.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import torch

from .cameras import orbit_cameras


@dataclass
class SurfelScene:
    means3D: torch.Tensor      # [P,3]
    scales: torch.Tensor       # [P,2]
    rotations: torch.Tensor    # [P,4]
    opacities: torch.Tensor    # [P,1]
    shs: torch.Tensor          # [P,16,3]
    sh_degree: int = 3

    @property
    def P(self) -> int:
        return int(self.means3D.shape[0])

    def to(self, device):
        return SurfelScene(*(t.to(device) for t in (self.means3D, self.scales, self.rotations,
                                                     self.opacities, self.shs)), self.sh_degree)


def _attributes(P: int, g: torch.Generator):
    scales = torch.exp(torch.randn(P, 2, generator=g) * 0.5 - 3.0)
    q = torch.randn(P, 4, generator=g)
    rotations = q / q.norm(dim=1, keepdim=True)
    opacities = torch.sigmoid(torch.randn(P, 1, generator=g))
    shs = torch.randn(P, 16, 3, generator=g) * 0.05
    shs[:, 0, :] = torch.randn(P, 3, generator=g) * 0.3
    return scales, rotations, opacities, shs


def random_surfels(P: int = 4096, seed: int = 0) -> SurfelScene:
    g = torch.Generator().manual_seed(seed)
    means = torch.rand(P, 3, generator=g) * 2.0 - 1.0
    return SurfelScene(means, *_attributes(P, g))


def _signed_pow(t: torch.Tensor, e):
    return torch.sign(t) * torch.abs(t).pow(e)


def superquadric_points(n: int, scale, eps1, eps2, R, t, g: torch.Generator):
    """Points on one superquadric surface: (eta, omega) uniform, row-vector
    transform ``(v * S) @ R + t`` as the binding does
    (games/block_mesh_splatting/scene/block_gaussian_model.py:225-226)."""
    eta = (torch.rand(n, generator=g) * 2 - 1) * (math.pi / 2) * 0.999
    omega = (torch.rand(n, generator=g) * 2 - 1) * math.pi
    ce, se = _signed_pow(torch.cos(eta), eps1), _signed_pow(torch.sin(eta), eps1)
    co, so = _signed_pow(torch.cos(omega), eps2), _signed_pow(torch.sin(omega), eps2)
    v = torch.stack([ce * so, se, ce * co], dim=-1)
    return (v * scale) @ R + t


def random_rotation(g: torch.Generator) -> torch.Tensor:
    q = torch.randn(4, generator=g)
    q = q / q.norm()
    w, x, y, z = q.tolist()
    return torch.tensor([
        [1 - 2 * y * y - 2 * z * z, 2 * x * y - 2 * z * w, 2 * x * z + 2 * y * w],
        [2 * x * y + 2 * z * w, 1 - 2 * x * x - 2 * z * z, 2 * y * z - 2 * x * w],
        [2 * x * z - 2 * y * w, 2 * y * z + 2 * x * w, 1 - 2 * x * x - 2 * y * y]])


def superquadric_surfels(P: int = 500_000, num_sq: int = 16, seed: int = 0) -> SurfelScene:
    g = torch.Generator().manual_seed(seed)
    counts = [P // num_sq + (1 if i < P % num_sq else 0) for i in range(num_sq)]
    pts = []
    for n in counts:
        scale = torch.rand(3, generator=g) * 0.4 + 0.1
        e1 = float(torch.rand(1, generator=g) * 1.6 + 0.2)
        e2 = float(torch.rand(1, generator=g) * 1.6 + 0.2)
        R = random_rotation(g)
        c = torch.randn(3, generator=g)
        c = c / c.norm() * float(torch.rand(1, generator=g)) ** (1.0 / 3.0)
        pts.append(superquadric_points(n, scale, e1, e2, R, c, g))
    means = torch.cat(pts) + torch.randn(P, 3, generator=g) * 0.01
    return SurfelScene(means, *_attributes(P, g))


def scene_cameras(n: int, height: int, width: int, fovx_deg: float, radius: float = 3.0, seed: int = 0):
    return orbit_cameras(n, radius, height, width, fovx_deg, seed)


def workload(name: str, seed: int = 0):
    """(scene, cameras) of a named workload."""
    if name == "random4k_128":
        return random_surfels(4096, seed), scene_cameras(1, 128, 128, 60.0, seed=seed)
    if name == "sq500k_16x800x600":
        return superquadric_surfels(500_000, 16, seed), scene_cameras(16, 600, 800, 50.0, seed=seed)
    if name == "sq100k_4x800x600":      # a smaller case of the same distribution (profiling)
        return superquadric_surfels(100_000, 16, seed), scene_cameras(4, 600, 800, 50.0, seed=seed)
    raise KeyError(name)
