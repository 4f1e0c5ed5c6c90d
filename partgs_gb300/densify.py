"""Densification of the part-level surfels: the per-step statistics on the
GPU (``sgr_densify_stats``, one launch, capturable in the training graph)
and the periodic clone / split / prune of
games/block_mesh_splatting/scene/two_gaussian_model.py:343-430 with
scene/gaussian_model.py:316-319 and 499-513 (densify_and_prune,
reset_opacity), done with device gathers and carrying the Adam moments the
way the reference's optimiser surgery does (new points start with zero
moments, pruned points drop theirs).

Parameters are the reference's raw tensors, keyed by its optimiser group
names: ``xyz`` [P,3], ``f_dc`` [P,1,3], ``f_rest`` [P,M-1,3], ``opacity``
[P,1] (logit), ``scaling`` [P,2] (log), ``rotation`` [P,4].
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib as L

NAMES = ("xyz", "f_dc", "f_rest", "opacity", "scaling", "rotation")
_p = C.c_void_p


def _lib():
    lib = L.load()
    lib.sgr_densify_stats.restype = C.c_int
    lib.sgr_densify_stats.argtypes = [_p, C.c_int32, _p, C.c_int32, _p, _p, C.c_float, _p, _p, _p, _p]
    return lib


class DensifyStats:
    """xyz_gradient_accum [P,1], denom [P,1] and max_radii2D [P] of the reference."""

    def __init__(self, num_surfels: int, device="cuda"):
        self.reset(num_surfels, device)

    def reset(self, num_surfels: int, device=None):
        dev = device if device is not None else self.denom.device
        self.grad_accum = torch.zeros(num_surfels, 1, device=dev)
        self.denom = torch.zeros(num_surfels, 1, device=dev)
        self.max_radii2D = torch.zeros(num_surfels, device=dev)

    @property
    def num_surfels(self):
        return self.denom.shape[0]

    def update(self, tables, radii: torch.Tensor, means2D_grad: torch.Tensor, grad_scale: float = 1.0):
        """One step's statistics over every view of a batch: ``tables`` are a
        MultiViewRasterizer's (scene table, view table, scenes, records),
        ``radii`` [R] the forward's, ``means2D_grad`` [R,3] the backward's.
        grad_scale multiplies the gradient norms (the number of views, when
        the batch loss is the mean of the per-view losses)."""
        sct, vwt, n_scenes, R = tables
        if radii.numel() != R or means2D_grad.shape[0] != R:
            raise ValueError("radii / means2D gradient do not match the batch's records")
        L.check(_lib().sgr_densify_stats(sct.data_ptr(), n_scenes, vwt.data_ptr(), self.num_surfels,
                                         radii.data_ptr(), means2D_grad.contiguous().data_ptr(), float(grad_scale),
                                         self.max_radii2D.data_ptr(), self.grad_accum.data_ptr(),
                                         self.denom.data_ptr(), torch.cuda.current_stream().cuda_stream),
                "sgr_densify_stats")


def build_rotation(q: torch.Tensor) -> torch.Tensor:
    """Rotation matrices of quaternions (w, x, y, z), normalised first
    (utils/general_utils.py:149-171)."""
    q = q / torch.sqrt(q[:, 0] * q[:, 0] + q[:, 1] * q[:, 1] + q[:, 2] * q[:, 2] + q[:, 3] * q[:, 3])[:, None]
    r, x, y, z = q.unbind(1)
    return torch.stack([1 - 2 * (y * y + z * z), 2 * (x * y - r * z), 2 * (x * z + r * y),
                        2 * (x * y + r * z), 1 - 2 * (x * x + z * z), 2 * (y * z - r * x),
                        2 * (x * z - r * y), 2 * (y * z + r * x), 1 - 2 * (x * x + y * y)], 1).reshape(-1, 3, 3)


def _cat(params, semantic, adam, new, new_semantic):
    params = {k: torch.cat([params[k], new[k]], 0) for k in NAMES}
    if semantic is not None:
        semantic = torch.cat([semantic, new_semantic], 0)
    if adam is not None:
        adam = {k: tuple(torch.cat([m, torch.zeros_like(new[k])], 0) for m in adam[k]) for k in NAMES}
    return params, semantic, adam


def _keep(params, semantic, adam, keep):
    params = {k: params[k][keep] for k in NAMES}
    semantic = semantic[keep] if semantic is not None else None
    adam = {k: tuple(m[keep] for m in adam[k]) for k in NAMES} if adam is not None else None
    return params, semantic, adam


def densify_and_prune(params: dict, stats: DensifyStats, max_grad: float, min_opacity: float, extent: float,
                      max_screen_size=None, percent_dense: float = 0.01, semantic=None, adam=None,
                      split_samples=None, generator=None, N: int = 2):
    """Clone small surfels with a large mean screen-space gradient, split
    large ones into N, then prune transparent (and, with max_screen_size,
    world-space large) surfels.  Returns (params, semantic, adam, stats) at
    the new size; the statistics restart at zero as in the reference.
    ``split_samples`` [N * n_split, 3] replaces the normal draws of the split
    (for reproducing a run); otherwise they come from ``generator``."""
    grads = stats.grad_accum / stats.denom
    grads[grads.isnan()] = 0.0
    P0 = params["xyz"].shape[0]
    # clone (two_gaussian_model.py:406-422)
    sel = (torch.norm(grads, dim=-1) >= max_grad) & \
        (torch.max(torch.exp(params["scaling"]), dim=1).values <= percent_dense * extent)
    new = {k: params[k][sel] for k in NAMES}
    params, semantic, adam = _cat(params, semantic, adam, new, semantic[sel] if semantic is not None else None)
    # split (two_gaussian_model.py:378-404); cloned surfels have no gradient yet
    n1 = params["xyz"].shape[0]
    padded = torch.zeros(n1, device=grads.device)
    padded[:P0] = grads.reshape(-1)
    scale = torch.exp(params["scaling"])
    sel = (padded >= max_grad) & (torch.max(scale, dim=1).values > percent_dense * extent)
    stds = scale[sel].repeat(N, 1)
    stds = torch.cat([stds, torch.zeros_like(stds[:, :1])], dim=-1)
    if split_samples is None:
        samples = torch.normal(torch.zeros_like(stds), stds, generator=generator)
    else:
        samples = split_samples.to(stds)
        if samples.shape != stds.shape:
            raise ValueError(f"split_samples must be {tuple(stds.shape)}")
    rots = build_rotation(params["rotation"][sel]).repeat(N, 1, 1)
    new = {"xyz": torch.bmm(rots, samples.unsqueeze(-1)).squeeze(-1) + params["xyz"][sel].repeat(N, 1),
           "scaling": torch.log(scale[sel].repeat(N, 1) / (0.8 * N)),
           "rotation": params["rotation"][sel].repeat(N, 1),
           "f_dc": params["f_dc"][sel].repeat(N, 1, 1),
           "f_rest": params["f_rest"][sel].repeat(N, 1, 1),
           "opacity": params["opacity"][sel].repeat(N, 1)}
    params, semantic, adam = _cat(params, semantic, adam, new,
                                  semantic[sel].repeat(N, 1) if semantic is not None else None)
    keep = ~torch.cat([sel, torch.zeros(N * int(sel.sum()), dtype=torch.bool, device=sel.device)])
    params, semantic, adam = _keep(params, semantic, adam, keep)
    # prune (gaussian_model.py:505-511); densification reset max_radii2D to
    # zero, so the screen-size test sees zeros, as in the reference
    prune = (torch.sigmoid(params["opacity"]) < min_opacity).squeeze(-1)
    if max_screen_size:
        big_vs = torch.zeros_like(prune)
        big_ws = torch.exp(params["scaling"]).max(dim=1).values > 0.1 * extent
        prune = prune | big_vs | big_ws
    params, semantic, adam = _keep(params, semantic, adam, ~prune)
    stats = DensifyStats(params["xyz"].shape[0], params["xyz"].device)
    return params, semantic, adam, stats


def reset_opacity(params: dict, adam=None):
    """opacity = logit(min(sigmoid(opacity), 0.01)) with its Adam moments
    cleared (scene/gaussian_model.py:316-319, replace_tensor_to_optimizer)."""
    op = torch.sigmoid(params["opacity"])
    x = torch.min(op, torch.ones_like(op) * 0.01)
    params = dict(params, opacity=torch.log(x / (1 - x)))
    if adam is not None:
        adam = dict(adam, opacity=tuple(torch.zeros_like(m) for m in adam["opacity"]))
    return params, adam
