"""Point-level surfel training step over a batch of views.

The step is the reference's point-stage iteration (train.py:225-257) applied
to every view of a batch at once: rasterise, L1 + D-SSIM photometric loss
(utils/loss_utils.py:8-54), depth-distortion loss, and the normal-consistency
loss between rendered normals and normals from the median depth map
(renderer/gaussian_renderer/__init__.py:111-141, utils/point_utils.py:4-33),
then an Adam update (scene/gaussian_model.py:266, eps 1e-15; one launch,
optim.py).  Parameters use
the reference's activations: exp scales, normalised quaternions, sigmoid
opacity, concatenated SH features (scene/gaussian_model.py:198-218), in one
CUDA kernel each way (activations.py).

``SurfelTrainer.capture()`` records the whole step (forward, losses,
backward, optimiser) in one CUDA graph; ``replay()`` runs it.
"""
from __future__ import annotations

import math

import torch
import torch.nn.functional as F

from . import _lib
from .activations import activate, activate_backward, activate_forward
from .batched import MultiViewRasterizer
from .optim import SurfelAdam


def _gaussian_window(size=11, sigma=1.5, channels=3, device="cuda"):
    g = torch.tensor([math.exp(-(x - size // 2) ** 2 / float(2 * sigma ** 2)) for x in range(size)])
    g = g / g.sum()
    w2 = (g[:, None] @ g[None, :]).float()
    return w2.expand(channels, 1, size, size).contiguous().to(device)


def ssim(img1, img2, window):
    """Mean SSIM of [B,C,H,W] images, utils/loss_utils.py:24-54."""
    C = img1.shape[-3]
    pad = window.shape[-1] // 2
    mu1 = F.conv2d(img1, window, padding=pad, groups=C)
    mu2 = F.conv2d(img2, window, padding=pad, groups=C)
    mu1_sq, mu2_sq, mu1_mu2 = mu1 * mu1, mu2 * mu2, mu1 * mu2
    s1 = F.conv2d(img1 * img1, window, padding=pad, groups=C) - mu1_sq
    s2 = F.conv2d(img2 * img2, window, padding=pad, groups=C) - mu2_sq
    s12 = F.conv2d(img1 * img2, window, padding=pad, groups=C) - mu1_mu2
    C1, C2 = 0.01 ** 2, 0.03 ** 2
    m = ((2 * mu1_mu2 + C1) * (2 * s12 + C2)) / ((mu1_sq + mu2_sq + C1) * (s1 + s2 + C2))
    return m.mean()


class DepthNormals:
    """Per-view ray directions for normals from depth maps
    (utils/point_utils.py:4-33), precomputed once per camera set."""

    def __init__(self, cameras, device="cuda"):
        rays_d, rays_o, rot = [], [], []
        for c in cameras:
            wv = torch.as_tensor(c.world_view_transform, dtype=torch.float32)
            full = torch.as_tensor(c.full_proj_transform, dtype=torch.float32)
            W, H = c.width, c.height
            c2w = wv.T.inverse()
            ndc2pix = torch.tensor([[W / 2, 0, 0, W / 2], [0, H / 2, 0, H / 2], [0, 0, 0, 1]]).float().T
            proj = c2w.T @ full
            intr = (proj @ ndc2pix)[:3, :3].T
            gx, gy = torch.meshgrid(torch.arange(W).float(), torch.arange(H).float(), indexing="xy")
            pts = torch.stack([gx, gy, torch.ones_like(gx)], -1).reshape(-1, 3)
            rays_d.append(pts @ intr.inverse().T @ c2w[:3, :3].T)
            rays_o.append(c2w[:3, 3])
            rot.append(wv[:3, :3].T)
        self.H, self.W = cameras[0].height, cameras[0].width
        self.rays_d = torch.stack(rays_d).to(device)          # [V,HW,3]
        self.rays_o = torch.stack(rays_o).to(device)          # [V,3]
        self.view_to_world = torch.stack(rot).to(device)      # [V,3,3]

    def normals(self, depth):
        """depth [V,1,H,W] -> normals [V,3,H,W] (zero border)."""
        V = depth.shape[0]
        pts = depth.reshape(V, -1, 1) * self.rays_d + self.rays_o[:, None, :]
        pts = pts.reshape(V, self.H, self.W, 3)
        dx = pts[:, 2:, 1:-1] - pts[:, :-2, 1:-1]
        dy = pts[:, 1:-1, 2:] - pts[:, 1:-1, :-2]
        n = F.normalize(torch.cross(dx, dy, dim=-1), dim=-1)
        out = torch.zeros_like(pts)
        out[:, 1:-1, 1:-1] = n
        return out.permute(0, 3, 1, 2)


class SurfelTrainer:
    """Surfel parameters, the batched loss and Adam."""

    def __init__(self, scene, cameras, bin_capacity=None, lambda_dssim=0.2, lambda_dist=1000.0,
                 lambda_normal=0.05, depth_ratio=1.0, bg=(0.0, 0.0, 0.0), device="cuda", extent=3.0,
                 fused_loss=True, densify_stats=False):
        dev = torch.device(device)
        self.xyz = scene.means3D.detach().clone().to(dev).requires_grad_(True)
        self.log_scaling = torch.log(scene.scales).detach().clone().to(dev).requires_grad_(True)
        self.rotation = scene.rotations.detach().clone().to(dev).requires_grad_(True)
        op = scene.opacities.clamp(1e-4, 1 - 1e-4)
        self.opacity_logit = torch.log(op / (1 - op)).detach().clone().to(dev).requires_grad_(True)
        self.features_dc = scene.shs[:, :1].detach().clone().to(dev).requires_grad_(True)
        self.features_rest = scene.shs[:, 1:].detach().clone().to(dev).requires_grad_(True)
        self.sh_degree = scene.sh_degree
        self.raster = MultiViewRasterizer(cameras, bg, scene.sh_degree, bin_capacity=bin_capacity,
                                          num_surfels=scene.P, device=dev)
        self.normals = DepthNormals(cameras, dev)
        self.window = _gaussian_window(device=dev)
        self.lambda_dssim, self.lambda_dist, self.lambda_normal = lambda_dssim, lambda_dist, lambda_normal
        self.depth_ratio = depth_ratio
        self.point_loss = None
        if fused_loss:
            from .losses import PointLoss
            self.point_loss = PointLoss(cameras, lambda_dssim, lambda_dist, lambda_normal, depth_ratio, dev)
        groups = [
            {"params": [self.xyz], "lr": 0.00016 * extent},
            {"params": [self.features_dc], "lr": 0.0025},
            {"params": [self.features_rest], "lr": 0.0025 / 20.0},
            {"params": [self.opacity_logit], "lr": 0.05},
            {"params": [self.log_scaling], "lr": 0.005},
            {"params": [self.rotation], "lr": 0.001},
        ]
        self.opt = SurfelAdam(groups, eps=1e-15)
        self.targets = None
        self.graph = None
        self.loss = None
        self._radii = None
        # densification statistics, updated by every step (and captured with it)
        self.stats = None
        if densify_stats:
            from .densify import DensifyStats
            self.stats = DensifyStats(scene.P, dev)

    def params(self):
        return [self.xyz, self.features_dc, self.features_rest, self.opacity_logit, self.log_scaling, self.rotation]

    def loss_fn(self, targets):
        scales, rots, opac, shs = activate(self.log_scaling, self.rotation, self.opacity_logit, self.features_dc,
                                           self.features_rest)
        color, allmap, _, radii = self.raster(self.xyz, opac, shs, scales, rots)
        self._radii = radii
        if self.point_loss is not None:
            return self.point_loss(color, allmap, targets)
        return self.reference_loss(color, allmap, targets)

    def reference_loss(self, color, allmap, targets):
        """The loss in PyTorch operations (the statement the fused kernels
        follow)."""
        l1 = torch.abs(color - targets).mean()
        loss = (1.0 - self.lambda_dssim) * l1 + self.lambda_dssim * (1.0 - ssim(color, targets, self.window))
        alpha = allmap[:, 1:2]
        rend_normal = torch.einsum("vchw,vcd->vdhw", allmap[:, 2:5], self.normals.view_to_world)
        median = torch.nan_to_num(allmap[:, 5:6], 0, 0)
        expected = torch.nan_to_num(allmap[:, 0:1] / alpha, 0, 0)
        surf_depth = expected * (1 - self.depth_ratio) + self.depth_ratio * median
        surf_normal = self.normals.normals(surf_depth) * alpha.detach()
        normal_loss = self.lambda_normal * (1 - (rend_normal * surf_normal).sum(dim=1)).mean()
        dist_loss = self.lambda_dist * allmap[:, 6:7].mean()
        return loss + dist_loss + normal_loss

    def _fused_step(self, targets):
        """Forward, fused loss and backward without autograd: the loss
        kernels hand dL/dcolor and dL/dmaps to the rasteriser's backward,
        which writes dL/dxyz into xyz.grad; the activation backward writes
        the other parameters' gradients into their .grad buffers (which the
        optimiser consumes and clears).  Only this library's kernels run."""
        ins = [t.detach() for t in (self.log_scaling, self.rotation, self.opacity_logit, self.features_dc,
                                    self.features_rest)]
        scales, rots, opac, shs = activate_forward(ins)
        color, allmap, _, radii, state = self.raster.forward_state(self.xyz.detach(), opac, shs, scales, rots)
        self._radii = radii
        loss, dcol, doth = self.point_loss.forward_backward(color, allmap, targets)
        g = self.raster.backward_state(state, dcol, doth, out={"dL_dmeans3D": self.xyz.grad})
        activate_backward(ins, (g["dL_dscales"], g["dL_drotations"], g["dL_dopacity"], g["dL_dsh"]),
                          [self.log_scaling.grad, self.rotation.grad, self.opacity_logit.grad,
                           self.features_dc.grad, self.features_rest.grad])
        return loss

    def step(self, targets):
        """One eager step; returns the loss tensor.  The optimiser clears the
        gradients it consumes."""
        if self.point_loss is not None:
            with torch.no_grad():
                loss = self._fused_step(targets)
        else:
            loss = self.loss_fn(targets)
            loss.backward()
        if self.stats is not None:
            # the batch loss averages its views: scale the per-view screen-space
            # gradients back to what a single-view iteration sees
            self.stats.update(self.raster.tables, self._radii, self.raster.last_means2D_grad,
                              grad_scale=float(self.raster.num_views))
        self.opt.step()
        return loss

    def capture(self, targets, warmup=3, headroom=1.25, autotune=False):
        """Captures step() into a CUDA graph reading ``self.targets``.

        With ``autotune`` the cell size, then the blends' warp footprint and
        tile schedule, are picked first by timing eager steps
        (``autotune.tune_cells``, ``tune_blend``; parameters restored).  Without a cell-list
        capacity, the eager warm-up steps size it (``headroom`` times the
        largest entry count they saw); after replays, ``self.raster.counts()``
        reports the flags (SGR_FLAG_BIN_OVERFLOW when the parameters have
        drifted past the capacity)."""
        if autotune:
            from .autotune import tune_blend, tune_cells
            tune_cells(self, targets)
            tune_blend(self, targets)
        self.targets = targets.clone()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        most = 0
        with torch.cuda.stream(s):
            for _ in range(max(1, warmup)):
                self.step(self.targets)
                s.synchronize()
                most = max(most, self.raster.counts()[2])
        torch.cuda.current_stream().wait_stream(s)
        if self.raster.bin_capacity is None:
            self.raster.set_capacity(int(most * headroom) + 4096)
        self.graph = torch.cuda.CUDAGraph()
        lib = _lib.load()
        n0 = lib.sgr_kernel_launches()
        with torch.cuda.graph(self.graph):
            self.loss = self.step(self.targets)
        self.launches_per_step = int(lib.sgr_kernel_launches() - n0)   # libsgr kernels in one replay
        return self.graph

    def replay(self):
        self.graph.replay()
        return self.loss

    def train(self, steps: int, check_every: int = 25, headroom: float = 1.25, max_recaptures: int = 4):
        """Replays ``steps`` captured steps, checking every ``check_every``
        steps whether any of them overflowed the cell lists.  If one did, the
        interval is undone (parameters and Adam state restored), the step is
        captured again with room for the largest entry count seen times
        ``headroom``, and the interval runs again.  Returns the last loss."""
        if self.graph is None:
            raise RuntimeError("capture() first")
        done, loss, recaptures = 0, self.loss, 0
        self.raster.sticky_counts(reset=True)
        while done < steps:
            n = min(check_every, steps - done)
            snap = self.snapshot()
            for _ in range(n):
                loss = self.replay()
            flags, most = self.raster.sticky_counts(reset=True)
            if flags & _lib.SGR_FLAG_LIST_INCONSISTENT:
                raise RuntimeError("a backward found a cell list shorter than its forward used "
                                   "(SGR_FLAG_LIST_INCONSISTENT): gradients of that step are incomplete")
            if flags & _lib.SGR_FLAG_BIN_OVERFLOW:
                if recaptures == max_recaptures:
                    raise RuntimeError(f"cell lists still overflow after {recaptures} re-captures")
                recaptures += 1
                self.restore(snap)
                self.raster.set_capacity(int(most * headroom) + 4096)
                self.capture(self.targets, warmup=1)
                self.restore(snap)   # the capture's warm-up step is not part of the run
                self.raster.sticky_counts(reset=True)
                continue
            done += n
        self.recaptures = recaptures
        return loss

    def _state(self):
        return [p.detach() for p in self.params()] + self.opt.state_tensors()

    def densify_and_prune(self, max_grad, min_opacity, extent, max_screen_size=None, percent_dense=0.01,
                          generator=None):
        """The reference's densify_and_prune on this trainer's surfels, from the
        statistics the steps gathered (``densify_stats=True``); parameters and
        Adam moments are replaced, so a captured graph is dropped (capture
        again).  Returns the new surfel count."""
        from .densify import densify_and_prune
        if self.stats is None:
            raise RuntimeError("densification statistics are off (SurfelTrainer(..., densify_stats=True))")
        params = dict(zip(("xyz", "f_dc", "f_rest", "opacity", "scaling", "rotation"),
                          (p.detach() for p in self.params())))
        adam = {k: (m, v) for k, (_, _, m, v) in zip(params, self.opt.entries)}
        params, _, adam, self.stats = densify_and_prune(params, self.stats, max_grad, min_opacity, extent,
                                                        max_screen_size, percent_dense, adam=adam,
                                                        generator=generator)
        self._replace(params, adam)
        return int(self.xyz.shape[0])

    def reset_opacity(self):
        """opacity = logit(min(opacity, 0.01)) with its moments cleared."""
        from .densify import reset_opacity
        with torch.no_grad():
            params, adam = reset_opacity({"opacity": self.opacity_logit.detach()},
                                         {"opacity": (self.opt.entries[3][2], self.opt.entries[3][3])})
            self.opacity_logit.copy_(params["opacity"])
            for dst, src in zip(self.opt.entries[3][2:], adam["opacity"]):
                dst.copy_(src)

    def _replace(self, params, adam):
        new = [params[k].contiguous().requires_grad_(True) for k in params]
        (self.xyz, self.features_dc, self.features_rest, self.opacity_logit, self.log_scaling,
         self.rotation) = new
        self.opt.replace(new, [adam[k] for k in params])
        self.graph = None
        self.loss = None
        self.raster.set_capacity(None)

    def snapshot(self):
        """Copies of the parameters and the optimiser state."""
        return [t.clone() for t in self._state()]

    def restore(self, state):
        """Writes a snapshot back in place (captured graphs keep their
        addresses)."""
        dst = self._state()
        if len(dst) != len(state):
            raise ValueError("snapshot does not match the optimiser state")
        with torch.no_grad():
            for d, s in zip(dst, state):
                d.copy_(s)
