"""Adam for surfel parameters in one CUDA launch (libsgr.so ``sgr_adam_step``).

``SurfelAdam`` is the reference's surfel optimiser (torch.optim.Adam with one
learning rate per parameter group and eps 1e-15, scene/gaussian_model.py:266)
for up to sixteen parameter tensors.  The step count lives on the device and
each gradient is cleared by the update itself, so a step neither
synchronises nor needs a separate ``zero_grad`` launch, and it can be
captured in a CUDA graph.  Gradients are created (zero) up front so that
autograd accumulates into fixed addresses.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib as L

_p = C.c_void_p


class AdamTensor(C.Structure):
    _fields_ = [("param", _p), ("grad", _p), ("exp_avg", _p), ("exp_avg_sq", _p), ("numel", C.c_int64),
                ("lr", C.c_float)]


MAX_TENSORS = 16


class AdamArgs(C.Structure):
    _fields_ = [("tensors", AdamTensor * MAX_TENSORS), ("count", C.c_int32), ("beta1", C.c_float),
                ("beta2", C.c_float), ("eps", C.c_float), ("zero_grad", C.c_int32)]


def _lib():
    lib = L.load()
    fn = lib.sgr_adam_step
    fn.restype, fn.argtypes = C.c_int, [C.POINTER(AdamArgs), _p, _p]
    return lib


class SurfelAdam:
    """``groups``: [{"params": [tensor], "lr": float}, ...] as for torch.optim."""

    def __init__(self, groups, betas=(0.9, 0.999), eps=1e-15):
        self.entries = []
        for g in groups:
            for p in g["params"]:
                if not (p.is_cuda and p.dtype == torch.float32 and p.is_contiguous()):
                    raise ValueError("SurfelAdam takes contiguous float32 CUDA tensors")
                if p.grad is None:
                    p.grad = torch.zeros_like(p)
                self.entries.append((p, float(g["lr"]), torch.zeros_like(p), torch.zeros_like(p)))
        if len(self.entries) > MAX_TENSORS:
            raise ValueError(f"at most {MAX_TENSORS} parameter tensors")
        self.betas, self.eps = betas, float(eps)
        self.step_count = torch.zeros(1, dtype=torch.float32, device=self.entries[0][0].device)

    def _args(self):
        a = AdamArgs()
        for i, (p, lr, m, v) in enumerate(self.entries):
            if p.grad is None or p.grad.data_ptr() == 0:
                raise RuntimeError("parameter without a gradient buffer")
            a.tensors[i] = AdamTensor(p.data_ptr(), p.grad.data_ptr(), m.data_ptr(), v.data_ptr(), p.numel(), lr)
        a.count = len(self.entries)
        a.beta1, a.beta2 = self.betas
        a.eps = self.eps
        a.zero_grad = 1
        return a

    def step(self):
        a = self._args()
        L.check(_lib().sgr_adam_step(C.byref(a), self.step_count.data_ptr(), torch.cuda.current_stream().cuda_stream),
                "sgr_adam_step")

    def zero_grad(self, set_to_none=False):
        """Gradients are already cleared by ``step``; kept for the optimiser
        interface."""

    def replace(self, params, moments):
        """New parameter tensors (same groups, new sizes) with their carried
        (exp_avg, exp_avg_sq); the step count is kept, as torch's Adam keeps
        each parameter's step through the reference's optimiser surgery."""
        if len(params) != len(self.entries):
            raise ValueError("one tensor per parameter group")
        entries = []
        for (_, lr, _, _), p, (m, v) in zip(self.entries, params, moments):
            if p.grad is None:
                p.grad = torch.zeros_like(p)
            entries.append((p, lr, m.contiguous(), v.contiguous()))
        self.entries = entries

    def state_tensors(self):
        """The moment buffers and the step count (for snapshots)."""
        return [t for _, _, m, v in self.entries for t in (m, v)] + [self.step_count]
