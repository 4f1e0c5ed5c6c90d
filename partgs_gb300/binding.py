"""Superquadric -> surfel binding on the GPU with a hand-written adjoint.

``SuperquadricBinding`` replaces BlockGaussianModel.update_alpha /
get_verts / prepare_scaling_rot / get_opacity
(games/block_mesh_splatting/scene/block_gaussian_model.py:107-109, 178-256):
from the block parameters (sq_s, sq_r, sq_t, sq_eps, sq_occ) and the fixed
topology (eta, omega, faces, barycentric alpha, per-surfel scale) it produces
the surfel means, log scales, quaternions and opacities in one kernel, and
its backward returns the block-parameter gradients from libsgr.so's adjoint
kernels instead of ~20 autograd nodes.  ``prepare_scaling_rot(model)``
updates a BlockGaussianModel in place, as the reference method does.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib as L


def _c(t, dtype=torch.float32):
    return t.detach().to(dtype).contiguous()


class _BindFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sq_s, sq_r, sq_t, sq_eps, sq_occ, topo):
        lib = L.load()
        a, keep = topo.args(sq_s, sq_r, sq_t, sq_eps, sq_occ)
        n = topo.num_surfels
        dev = sq_s.device
        xyz = torch.empty(n, 3, device=dev)
        log_scaling = torch.empty(n, 2, device=dev)
        rotation = torch.empty(n, 4, device=dev)
        opacity = torch.empty(n, 1, device=dev)
        st = torch.cuda.current_stream().cuda_stream
        L.check(lib.sgr_bind_forward(C.byref(a), xyz.data_ptr(), log_scaling.data_ptr(), rotation.data_ptr(),
                                     opacity.data_ptr(), st), "sgr_bind_forward")
        ctx.topo = topo
        ctx.save_for_backward(*keep[:5])
        return xyz, log_scaling, rotation, opacity

    @staticmethod
    def backward(ctx, d_xyz, d_log, d_rot, d_op):
        lib = L.load()
        topo = ctx.topo
        sq_s, sq_r, sq_t, sq_eps, sq_occ = ctx.saved_tensors
        a, keep = topo.args(sq_s, sq_r, sq_t, sq_eps, sq_occ)
        dev = sq_s.device
        grads = [torch.empty_like(t) for t in (sq_s, sq_r, sq_t, sq_eps, sq_occ)]
        scratch = torch.empty(max(1, lib.sgr_bind_scratch_bytes(C.byref(a))), dtype=torch.uint8, device=dev)
        ptr = lambda t: None if t is None else _c(t).data_ptr()  # noqa: E731
        ups = [None if t is None else _c(t) for t in (d_xyz, d_log, d_rot, d_op)]
        st = torch.cuda.current_stream().cuda_stream
        L.check(lib.sgr_bind_backward(C.byref(a), *(None if u is None else u.data_ptr() for u in ups),
                                      *(g.data_ptr() for g in grads), scratch.data_ptr(), st), "sgr_bind_backward")
        return (*grads, None)


class SuperquadricBinding:
    """Fixed topology of B superquadrics: ``eta``/``omega`` [B,V] vertex
    parameters, ``faces`` [B,F,3], raw barycentric weights ``alpha``
    [B,F,N,3] (or [B*F,N,3]) and per-surfel scale factors ``scale``
    [B,F*N,1]."""

    def __init__(self, eta, omega, faces, alpha, scale, ratio_block_scene=0.25, scale_block_min=0.2):
        self.eta = _c(eta)
        self.omega = _c(omega)
        self.faces = _c(faces, torch.int32)
        B, F, _ = self.faces.shape
        self.alpha = _c(alpha.reshape(B * F, -1, 3))
        self.scale = _c(scale.reshape(B, -1))
        self.B, self.V, self.F, self.N = B, int(self.eta.shape[1]), F, int(self.alpha.shape[1])
        self.ratio, self.smin = float(ratio_block_scene), float(scale_block_min)

    @property
    def num_surfels(self):
        return self.B * self.F * self.N

    def args(self, sq_s, sq_r, sq_t, sq_eps, sq_occ):
        ts = [_c(t) for t in (sq_s, sq_r, sq_t, sq_eps, sq_occ)]
        a = L.BindArgs(self.B, self.V, self.F, self.N, self.ratio, self.smin, ts[0].data_ptr(), ts[1].data_ptr(),
                       ts[2].data_ptr(), ts[3].data_ptr(), self.eta.data_ptr(), self.omega.data_ptr(),
                       self.faces.data_ptr(), ts[4].data_ptr(), self.alpha.data_ptr(), self.scale.data_ptr())
        return a, ts

    def __call__(self, sq_s, sq_r, sq_t, sq_eps, sq_occ):
        """(xyz [n,3], log_scaling [n,2], rotation [n,4], opacity [n,1])."""
        return _BindFn.apply(sq_s, sq_r, sq_t, sq_eps, sq_occ.reshape(-1, 1), self)


def prepare_scaling_rot(model, binding: SuperquadricBinding | None = None):
    """In-place replacement of BlockGaussianModel.prepare_scaling_rot (and
    update_alpha): sets model._xyz, model._scaling, model._rotation and
    model.bound_opacity from the CUDA binding."""
    if binding is None:
        binding = SuperquadricBinding(model.sq_eta, model.sq_omega, model.faces, model._alpha, model._scale,
                                      model.ratio_block_scene, model.scale_block_min)
    xyz, log_scaling, rotation, opacity = binding(model.sq_s, model.sq_r, model.sq_t, model.sq_eps, model.sq_occ)
    model._xyz, model._scaling, model._rotation = xyz, log_scaling, rotation
    model.bound_opacity = opacity
    return binding
