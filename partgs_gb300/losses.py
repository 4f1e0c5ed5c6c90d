"""Fused point-level training loss (libsgr.so) behind torch.autograd.

``PointLoss`` computes, for a batch of views, the loss of the reference's
point stage (photometric L1 + D-SSIM, depth distortion, normal consistency;
train.py:229-250) and its gradients with respect to the rendered colour and
aux maps in one forward pass of three CUDA kernels; the autograd backward
only scales the stored gradients.  ``DepthNormals`` in surfel_step.py is the
PyTorch statement of the same normal term, kept for testing.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib as L


class LossArgs(C.Structure):
    _fields_ = [("V", C.c_int32), ("H", C.c_int32), ("W", C.c_int32), ("lambda_dssim", C.c_float),
                ("lambda_dist", C.c_float), ("lambda_normal", C.c_float), ("depth_ratio", C.c_float),
                ("color", C.c_void_p), ("target", C.c_void_p), ("others", C.c_void_p),
                ("view_to_world", C.c_void_p), ("ray_basis", C.c_void_p), ("ray_origin", C.c_void_p)]


_SIGS = {
    "sgr_loss_scratch_bytes": (C.c_size_t, [C.POINTER(LossArgs)]),
    "sgr_loss_forward_backward": (C.c_int, [C.POINTER(LossArgs), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_void_p]),
}


def _lib():
    lib = L.load()
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype, fn.argtypes = res, args
    return lib


def camera_geometry(cameras, device="cuda"):
    """Per view: the rotation taking view-space normals to world space and the
    affine ray basis of the depth back-projection (utils/point_utils.py:4-20),
    ray(x, y) = x a0 + y a1 + a2, with the ray origin."""
    vw, basis, origin = [], [], []
    for c in cameras:
        wv = torch.as_tensor(c.world_view_transform, dtype=torch.float32)
        full = torch.as_tensor(c.full_proj_transform, dtype=torch.float32)
        W, H = c.width, c.height
        c2w = wv.T.inverse()
        ndc2pix = torch.tensor([[W / 2, 0, 0, W / 2], [0, H / 2, 0, H / 2], [0, 0, 0, 1]]).float().T
        intr = ((c2w.T @ full) @ ndc2pix)[:3, :3].T
        basis.append(intr.inverse().T @ c2w[:3, :3].T)
        origin.append(c2w[:3, 3])
        vw.append(wv[:3, :3].T)
    st = lambda xs: torch.stack(xs).contiguous().to(device)  # noqa: E731
    return st(vw), st(basis), st(origin)


def _loss_and_grads(color, others, target, cfg):
    """The fused loss and its gradients with respect to the rendered maps."""
    lib = _lib()
    color = color.detach().contiguous()
    others = others.detach().contiguous()
    target = target.detach().contiguous()
    V, _, H, W = color.shape
    a = LossArgs(V, H, W, cfg.lambda_dssim, cfg.lambda_dist, cfg.lambda_normal, cfg.depth_ratio,
                 color.data_ptr(), target.data_ptr(), others.data_ptr(), cfg.view_to_world.data_ptr(),
                 cfg.ray_basis.data_ptr(), cfg.ray_origin.data_ptr())
    loss = torch.empty((), dtype=torch.float32, device=color.device)
    dcol = torch.empty_like(color)
    doth = torch.empty_like(others)
    scratch = torch.empty(lib.sgr_loss_scratch_bytes(C.byref(a)), dtype=torch.uint8, device=color.device)
    L.check(lib.sgr_loss_forward_backward(C.byref(a), loss.data_ptr(), dcol.data_ptr(), doth.data_ptr(),
                                          scratch.data_ptr(), torch.cuda.current_stream().cuda_stream),
            "sgr_loss_forward_backward")
    return loss, dcol, doth


class _PointLossFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, color, others, target, cfg):
        loss, dcol, doth = _loss_and_grads(color, others, target, cfg)
        ctx.save_for_backward(dcol, doth)
        return loss

    @staticmethod
    def backward(ctx, g):
        dcol, doth = ctx.saved_tensors
        return dcol * g, doth * g, None, None


class PointLoss:
    """Loss of a fixed camera batch; call with (color [V,3,H,W], others
    [V,7,H,W], target [V,3,H,W])."""

    def __init__(self, cameras, lambda_dssim=0.2, lambda_dist=1000.0, lambda_normal=0.05, depth_ratio=1.0,
                 device="cuda"):
        self.view_to_world, self.ray_basis, self.ray_origin = camera_geometry(cameras, device)
        self.lambda_dssim, self.lambda_dist = float(lambda_dssim), float(lambda_dist)
        self.lambda_normal, self.depth_ratio = float(lambda_normal), float(depth_ratio)

    def __call__(self, color, others, target):
        return _PointLossFn.apply(color, others, target, self)

    def forward_backward(self, color, others, target):
        """(loss, dL/dcolor, dL/dothers) without autograd: the three kernels
        of the fused loss, nothing else."""
        return _loss_and_grads(color, others, target, self)
