"""Pins the torch restatement of the block-stage losses (the GPU kernels'
checker) and the ray geometry to the reference's own summarize_losses,
cast_rays and implicit_sq, run in float64 by tests/golden/make_golden.py."""
import os

import numpy as np
import torch

from oracle import sq_loss_oracle as O
from partgs_gb300.sq_losses import ray_geometry

GOLD = os.path.join(os.path.dirname(__file__), "golden", "sq_losses.npz")


def _load():
    d = np.load(GOLD)
    t = {k: torch.from_numpy(np.asarray(d[k])) for k in d.files}
    return d, t


def _rays(d, t):
    origin, dirs = ray_geometry(t["K"], t["world_view"], int(d["height"]), int(d["width"]), t["ray_idx"])
    return origin, dirs


def test_ray_geometry_matches_cast_rays():
    d, t = _load()
    origin, dirs = _rays(d, t)
    pts = O.ray_points(origin, dirs, t["jitter"], float(d["near"]), float(d["far"]))
    np.testing.assert_allclose(pts[:, :8].numpy(), d["points_head"], rtol=0, atol=1e-12)


def test_oracle_losses_and_gradients_match_the_reference():
    d, t = _load()
    origin, dirs = _rays(d, t)
    p = [t[k].clone().requires_grad_(True) for k in ("in_S", "in_R", "in_T")]
    e1 = t["in_eps1"][:, 0].clone().requires_grad_(True)
    e2 = t["in_eps2"][:, 0].clone().requires_grad_(True)
    occ = t["in_sq_occ"][:, 0].clone().requires_grad_(True)
    mask = t["mask"].reshape(-1)[t["ray_idx"]]
    ratio = float(d["ratio"])
    ray = O.ray_losses(*p, e1, e2, occ, ratio, origin, dirs, t["jitter"], mask, float(d["near"]), float(d["far"]))
    ovl = O.overlap_loss(*p, e1, e2, occ, ratio, t["unit01"] * 2 - 1, t["noise"])
    losses = torch.stack([*ray, ovl])
    np.testing.assert_allclose(losses.detach().numpy(), d["losses"], rtol=1e-12)
    (torch.from_numpy(d["weights"]) * losses).sum().backward()
    for name, got in (("S", p[0]), ("R", p[1]), ("T", p[2])):
        np.testing.assert_allclose(got.grad.numpy(), d[f"grad_{name}"], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(e1.grad.numpy(), d["grad_eps1"][:, 0], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(e2.grad.numpy(), d["grad_eps2"][:, 0], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(occ.grad.numpy(), d["grad_sq_occ"][:, 0], rtol=1e-9, atol=1e-12)
    assert all(float(x) > 0 for x in losses.detach()), "every term of the fixture is active"
