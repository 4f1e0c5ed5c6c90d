"""The point-level parameter getters of the training step in one CUDA
kernel per direction (libsgr.so ``sgr_activate_forward`` / ``_backward``):
exp scales, normalised rotations, sigmoid opacities and the concatenated SH
coefficients (scene/gaussian_model.py:198-218)."""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib as L

_p = C.c_void_p


class ActivateArgs(C.Structure):
    _fields_ = [("P", C.c_int64), ("sh_coeffs", C.c_int32), ("log_scaling", _p), ("rotation", _p),
                ("opacity_logit", _p), ("features_dc", _p), ("features_rest", _p), ("scales", _p),
                ("rotations", _p), ("opacities", _p), ("shs", _p), ("d_log_scaling", _p), ("d_rotation", _p),
                ("d_opacity_logit", _p), ("d_features_dc", _p), ("d_features_rest", _p)]


def _lib():
    lib = L.load()
    lib.sgr_activate_forward.restype = C.c_int
    lib.sgr_activate_forward.argtypes = [C.POINTER(ActivateArgs), _p]
    lib.sgr_activate_backward.restype = C.c_int
    lib.sgr_activate_backward.argtypes = [C.POINTER(ActivateArgs), _p, _p, _p, _p, _p]
    return lib


def _ptr(t):
    return None if t is None else t.data_ptr()


class _ActivateFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, log_scaling, rotation, opacity_logit, features_dc, features_rest):
        ins = [t.detach().contiguous() for t in (log_scaling, rotation, opacity_logit, features_dc, features_rest)]
        P = ins[0].shape[0]
        M = 1 + ins[4].shape[1]
        dev = ins[0].device
        scales = torch.empty(P, 2, device=dev)
        rots = torch.empty(P, 4, device=dev)
        opac = torch.empty(opacity_logit.shape, device=dev)
        shs = torch.empty(P, M, 3, device=dev)
        a = ActivateArgs(P, M, *(t.data_ptr() for t in ins), scales.data_ptr(), rots.data_ptr(), opac.data_ptr(),
                         shs.data_ptr(), None, None, None, None, None)
        L.check(_lib().sgr_activate_forward(C.byref(a), torch.cuda.current_stream().cuda_stream),
                "sgr_activate_forward")
        ctx.save_for_backward(*ins)
        return scales, rots, opac, shs

    @staticmethod
    def backward(ctx, d_scales, d_rots, d_opac, d_shs):
        ins = ctx.saved_tensors
        P, M = ins[0].shape[0], 1 + ins[4].shape[1]
        grads = [torch.empty_like(t) for t in ins]
        ups = [None if g is None else g.contiguous() for g in (d_scales, d_rots, d_opac, d_shs)]
        a = ActivateArgs(P, M, *(t.data_ptr() for t in ins), None, None, None, None,
                         *(g.data_ptr() for g in grads))
        L.check(_lib().sgr_activate_backward(C.byref(a), *(_ptr(u) for u in ups),
                                             torch.cuda.current_stream().cuda_stream), "sgr_activate_backward")
        return tuple(grads)


def activate(log_scaling, rotation, opacity_logit, features_dc, features_rest):
    """(scales, rotations, opacities, shs) with autograd."""
    return _ActivateFn.apply(log_scaling, rotation, opacity_logit, features_dc, features_rest)


def activate_forward(ins):
    """The forward without autograd: ins = (log_scaling, rotation,
    opacity_logit, features_dc, features_rest), contiguous; returns
    (scales, rotations, opacities, shs)."""
    P, M, dev = ins[0].shape[0], 1 + ins[4].shape[1], ins[0].device
    scales = torch.empty(P, 2, device=dev)
    rots = torch.empty(P, 4, device=dev)
    opac = torch.empty(ins[2].shape, device=dev)
    shs = torch.empty(P, M, 3, device=dev)
    a = ActivateArgs(P, M, *(t.data_ptr() for t in ins), scales.data_ptr(), rots.data_ptr(), opac.data_ptr(),
                     shs.data_ptr(), None, None, None, None, None)
    L.check(_lib().sgr_activate_forward(C.byref(a), torch.cuda.current_stream().cuda_stream), "sgr_activate_forward")
    return scales, rots, opac, shs


def activate_backward(ins, ups, outs):
    """The backward without autograd: gradients of (scales, rotations,
    opacities, shs) in ``ups`` (None for none) written into ``outs``, one
    contiguous buffer per input of ``ins`` (e.g. the parameters' ``.grad``)."""
    P, M = ins[0].shape[0], 1 + ins[4].shape[1]
    a = ActivateArgs(P, M, *(t.data_ptr() for t in ins), None, None, None, None, *(g.data_ptr() for g in outs))
    L.check(_lib().sgr_activate_backward(C.byref(a), *(_ptr(u) for u in ups), torch.cuda.current_stream().cuda_stream),
            "sgr_activate_backward")
