"""CPU restatement of the proposal network's forward and backward.

TEST INFRASTRUCTURE ONLY: the checker of ``partgs_gb300.proposal`` (the
network has no counterpart in the reference; its definition is the one the
package documents).  numpy, with the GPU path's rounding points restated:
GEMM operands and ReLU outputs in bfloat16 (round to nearest even), products
summed in float64 here (float32 on the tensor cores), the output layer and
all gradients of weights in full precision.
"""
from __future__ import annotations

import numpy as np

IN_PAD = 16


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    r = ((u >> 16) & 1) + np.uint32(0x7FFF)
    return ((u + r) & np.uint32(0xFFFF0000)).view(np.float32)


def forward(W, b, pts):
    """W, b: lists of float32 arrays ([out, in], [out]); pts [S, P, 3]."""
    S, P, _ = pts.shape
    Wb = [bf16(w).astype(np.float64) for w in W]
    x0 = np.zeros((S * P, IN_PAD), np.float32)
    x0[:, :3] = pts.reshape(-1, 3)
    x0 = bf16(x0).astype(np.float64)
    h = [x0]
    for i in range(3):
        h.append(bf16(np.maximum(h[-1] @ Wb[i].T + b[i], 0.0).astype(np.float32)).astype(np.float64))
    h3 = h[3].reshape(S, P, -1)
    arg = h3.argmax(axis=1)                                   # first maximum
    g = h3.max(axis=1)
    gb = bf16(g.astype(np.float32)).astype(np.float64)
    h4 = bf16(np.maximum(gb @ Wb[3].T + b[3], 0.0).astype(np.float32)).astype(np.float64)
    out = h4 @ Wb[4].T + b[4]
    return out, dict(S=S, P=P, Wb=Wb, h=h, g=g, gb=gb, arg=arg, h4=h4)


def backward(c, dout):
    """Gradients (gW, gb) of sum(out * dout)."""
    S, P, Wb, h, g, gb, arg, h4 = (c[k] for k in ("S", "P", "Wb", "h", "g", "gb", "arg", "h4"))
    q = lambda x: bf16(np.asarray(x, np.float32)).astype(np.float64)  # noqa: E731
    gW, gB = [None] * 5, [None] * 5
    d5 = q(dout)
    gW[4] = d5.T @ h4
    gB[4] = dout.sum(0)
    dz4 = q((d5 @ Wb[4]) * (h4 > 0))
    gW[3] = dz4.T @ gb
    gB[3] = dz4.sum(0)
    dg = dz4 @ Wb[3]
    C = g.shape[1]
    dz3 = np.zeros((S * P, C))
    rows = (np.arange(S)[:, None] * P + arg)                   # [S, C]
    dz3[rows, np.arange(C)[None, :]] = q(np.where(g > 0, dg, 0.0))
    gW[2] = dz3.T @ h[2]
    gB[2] = dz3.sum(0)
    dz2 = q((dz3 @ Wb[2]) * (h[2] > 0))
    gW[1] = dz2.T @ h[1]
    gB[1] = dz2.sum(0)
    dz1 = q((dz2 @ Wb[1]) * (h[1] > 0))
    gW[0] = dz1.T @ h[0]
    gB[0] = dz1.sum(0)
    return gW, gB
