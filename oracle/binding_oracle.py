"""CPU oracle for the superquadric -> surfel binding.

TEST INFRASTRUCTURE ONLY (used by tests/ as the checker of the CUDA
binding in libsgr.so; the product path never imports it).

A torch restatement of BlockGaussianModel.update_alpha / get_verts /
prepare_scaling_rot / get_opacity
(games/block_mesh_splatting/scene/block_gaussian_model.py:107-109, 178-256),
parametric_sq (games/block_mesh_splatting/utils/superquadric.py:10-14),
signed_pow (games/block_mesh_splatting/utils/pytorch.py:28-29),
quaternion_to_rotation_matrix (superquadric.py:93-107) and rot_to_quat_batch
(utils/general_utils.py:34-87).  Run in float64 it is the reference for the
CUDA forward and, through autograd, for its hand-written adjoint; it is
pinned to the reference's own code by tests/golden/reference_python.npz.
"""
from __future__ import annotations

import math

import numpy as np
import torch
import torch.nn.functional as F


def signed_pow(t, e):
    return torch.sign(t) * torch.abs(t).pow(e)


def parametric_sq(eta, omega, eps1, eps2):
    ce, se = signed_pow(torch.cos(eta), eps1), signed_pow(torch.sin(eta), eps1)
    co, so = signed_pow(torch.cos(omega), eps2), signed_pow(torch.sin(omega), eps2)
    return torch.stack([ce * so, se, ce * co], dim=-1)


def quat_to_rotmat(q):
    w, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    return torch.stack([
        1 - 2 * y ** 2 - 2 * z ** 2, 2 * x * y - 2 * z * w, 2 * x * z + 2 * y * w,
        2 * x * y + 2 * z * w, 1 - 2 * x ** 2 - 2 * z ** 2, 2 * y * z - 2 * x * w,
        2 * x * z - 2 * y * w, 2 * y * z + 2 * x * w, 1 - 2 * x ** 2 - 2 * y ** 2], dim=-1).view(-1, 3, 3)


def _sqrt_positive_part(x):
    ret = torch.zeros_like(x)
    m = x > 0
    ret[m] = torch.sqrt(x[m])
    return ret


def rot_to_quat(rot):
    m00, m01, m02, m10, m11, m12, m20, m21, m22 = torch.unbind(rot.reshape(-1, 9), dim=-1)
    q_abs = _sqrt_positive_part(torch.stack([1.0 + m00 + m11 + m22, 1.0 + m00 - m11 - m22,
                                             1.0 - m00 + m11 - m22, 1.0 - m00 - m11 + m22], dim=-1))
    rijk = torch.stack([
        torch.stack([q_abs[..., 0] ** 2, m21 - m12, m02 - m20, m10 - m01], dim=-1),
        torch.stack([m21 - m12, q_abs[..., 1] ** 2, m10 + m01, m02 + m20], dim=-1),
        torch.stack([m02 - m20, m10 + m01, q_abs[..., 2] ** 2, m12 + m21], dim=-1),
        torch.stack([m10 - m01, m20 + m02, m21 + m12, q_abs[..., 3] ** 2], dim=-1)], dim=-2)
    flr = torch.tensor(0.1).to(dtype=q_abs.dtype)
    cand = rijk / (2.0 * q_abs[..., None].max(flr))
    out = cand[F.one_hot(q_abs.argmax(dim=-1), num_classes=4) > 0.5, :].reshape(-1, 4)
    return torch.where(out[..., 0:1] < 0, -out, out)


def bind(sq_s, sq_r, sq_t, sq_eps, sq_occ, eta, omega, faces, alpha_raw, scale, ratio_block_scene,
         scale_block_min, eps=1e-8):
    """Returns (xyz [B*F*N,3], log_scaling [..,2], rotation [..,4], opacity [..,1])."""
    B, Fn, _ = faces.shape
    N = alpha_raw.shape[1]
    a = torch.relu(alpha_raw) + 1e-8
    alpha = a / a.sum(dim=-1, keepdim=True)                              # [B*F, N, 3]
    e1, e2 = (sq_eps.sigmoid() * 1.8 + 0.1).split([1, 1], dim=-1)
    verts = parametric_sq(eta, omega, e1, e2) * ratio_block_scene         # [B, V, 3]
    S = torch.exp(sq_s) + scale_block_min
    R = quat_to_rotmat(F.normalize(sq_r))
    v = torch.bmm(verts * S.unsqueeze(1), R) + sq_t.unsqueeze(1)
    tri = v[torch.arange(B)[:, None, None], faces]                       # [B, F, 3, 3]
    xyz = torch.matmul(alpha, tri.reshape(-1, 3, 3))                      # [B*F, N, 3]
    nrm = torch.linalg.cross(tri[:, :, 1] - tri[:, :, 0], tri[:, :, 2] - tri[:, :, 0], dim=2)
    v0 = nrm / (torch.linalg.vector_norm(nrm, dim=-1, keepdim=True) + eps)
    m = torch.mean(tri, dim=2)
    v1 = tri[:, :, 1] - m
    v1n = torch.linalg.vector_norm(v1, dim=-1, keepdim=True) + eps
    v1 = v1 / v1n
    v2i = tri[:, :, 2] - m
    dot = lambda p, q: (p * q).sum(dim=-1, keepdim=True)  # noqa: E731
    v2 = v2i - dot(v2i, v0) * v0 - dot(v2i, v1) * v1
    v2 = v2 / (torch.linalg.vector_norm(v2, dim=-1, keepdim=True) + eps)
    s1 = v1n / 2.0
    s2 = dot(v2i, v2) / 2.0
    scales = torch.cat((s1, s2), dim=2).unsqueeze(2).broadcast_to((B, Fn, N, 2)).flatten(1, 2)
    log_scaling = torch.log(torch.relu(scale.reshape(B, Fn * N, 1) * scales) + eps).reshape(-1, 2)
    rot = torch.stack((v1, v2, v0), dim=2).unsqueeze(2).broadcast_to((B, Fn, N, 3, 3)).flatten(1, 2)
    rotation = rot_to_quat(rot.transpose(-2, -1))
    opacity = torch.sigmoid(sq_occ).reshape(B, 1, 1).expand(-1, Fn * N, -1).reshape(-1, 1)
    return xyz.reshape(-1, 3), log_scaling, rotation, opacity


def grid_topology(n_eta: int, n_omega: int):
    """(eta, omega) on a half-cell-offset grid (no cos(eta) = 0 and no
    sin(omega) = 0 or cos(omega) = 0 node) and one triangle per node:
    (node, its eta neighbour, its omega neighbour), omega wrapped; the last
    eta row uses the row before it."""
    i = np.arange(n_eta)
    j = np.arange(n_omega)
    eta = -math.pi / 2 + (i + 0.5) * math.pi / n_eta
    omega = -math.pi + (j + 0.25) * 2 * math.pi / n_omega
    E, O_ = np.meshgrid(eta, omega, indexing="ij")
    idx = lambda a, b: a * n_omega + b  # noqa: E731
    faces = []
    for a in range(n_eta):
        an = a + 1 if a + 1 < n_eta else a - 1
        for b in range(n_omega):
            faces.append((idx(a, b), idx(an, b), idx(a, (b + 1) % n_omega)))
    return E.reshape(-1), O_.reshape(-1), np.asarray(faces, dtype=np.int64)


def random_binding_inputs(B=8, n_eta=50, n_omega=50, N=1, seed=0, dtype=torch.float64):
    """Block-level inputs in the workload's distributions: semi-axes
    U[0.1, 0.5] (as (exp(sq_s) + 0.2) * 0.25), exponents U[0.2, 1.8], random unit
    quaternions, centres uniform in the unit ball."""
    g = torch.Generator().manual_seed(seed)
    ratio, smin = 0.25, 0.2
    semi = torch.rand(B, 3, generator=g, dtype=dtype) * 0.4 + 0.1
    sq_s = torch.log(semi / ratio - smin)
    epsv = torch.rand(B, 2, generator=g, dtype=dtype) * 1.6 + 0.2
    sq_eps = torch.logit((epsv - 0.1) / 1.8)
    q = torch.randn(B, 4, generator=g, dtype=dtype)
    sq_r = q / q.norm(dim=1, keepdim=True)
    c = torch.randn(B, 3, generator=g, dtype=dtype)
    c = c / c.norm(dim=1, keepdim=True) * torch.rand(B, 1, generator=g, dtype=dtype) ** (1 / 3)
    sq_t = c
    sq_occ = torch.randn(B, 1, generator=g, dtype=dtype)
    eta, omega, faces = grid_topology(n_eta, n_omega)
    Fn = faces.shape[0]
    eta_t = torch.tensor(eta, dtype=dtype).expand(B, -1).contiguous()
    omega_t = torch.tensor(omega, dtype=dtype).expand(B, -1).contiguous()
    faces_t = torch.tensor(faces).expand(B, -1, -1).contiguous()
    alpha_raw = torch.rand(B * Fn, N, 3, generator=g, dtype=dtype)
    scale = torch.full((B, Fn * N, 1), 1.0 / math.sqrt(N), dtype=dtype)
    return dict(sq_s=sq_s, sq_r=sq_r, sq_t=sq_t, sq_eps=sq_eps, sq_occ=sq_occ, eta=eta_t, omega=omega_t,
                faces=faces_t, alpha_raw=alpha_raw, scale=scale, ratio_block_scene=ratio, scale_block_min=smin)
