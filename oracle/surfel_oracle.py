"""CPU oracle for the 2D-Gaussian surfel rasteriser (plain and part variants).

TEST INFRASTRUCTURE ONLY.  This module is a numpy restatement of the reference
rasteriser's algorithm, used by ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` as the checker.
The product path (``partgs_gb300``) never imports it.

What it restates (paths relative to the PartGS repository; ``P0`` is
``submodules/diff-surfel-rasterization``, ``P1`` is
``submodules/diff-surfel-rasterization_part``, ``cr`` is ``cuda_rasterizer``):

* preprocess forward     P0/cr/forward.cu:148-251, P1/cr/forward.cu:166-260
  (in_frustum P0/cr/auxiliary.h:185-210, quat_to_rotmat :213-235,
  compute_transmat P0/cr/forward.cu:75-115, compute_aabb :119-145,
  computeTransMat P1/cr/forward.cu:75-128, computeAABB :133-163,
  computeColorFromSH P0/cr/forward.cu:20-71, getRect P0/cr/auxiliary.h:67-77)
* tile binning           P0/cr/rasterizer_impl.cu:70-138, 278-318
  (keys ``tile << 32 | float_bits(depth)``, values surfel index, stable sort)
* blend forward          P0/cr/forward.cu:256-441, P1/cr/forward.cu:265-474
* blend backward         P0/cr/backward.cu:143-440, P1/cr/backward.cu:143-470
* preprocess backward    P0/cr/backward.cu:443-630 (incl. the SH backward
  :20-139 and the means2D densification proxy :626-629),
  P1/cr/backward.cu:473-671 (computeAABB adjoint kernel and proxy :621-671)

Arithmetic runs in ``dtype`` (float64 by default; float32 to mirror the
device's single precision).  Sub-expressions the part variant evaluates in
double precision because its constants are double macros
(P1/cr/auxiliary.h:20-36) are evaluated in float64 and narrowed.

Besides the outputs, the oracle reports *ambiguous* decisions: surfels whose
integer outputs (radius, tile rectangle) and pixels whose discrete decisions
(alpha cut-off, early termination, median crossing, 3D/2D filter branch, near
plane) sit within a relative ``amb_tol`` of their threshold.  A single
precision evaluation may legitimately land on either side of such a
threshold, so tests compare those entities loosely and everything else
exactly.

Parity status: the reference rasteriser's CUDA sources need the glm
header library, which is absent from the reference checkout, and need a GPU;
they cannot be built or run here.  The oracle is pinned by the reference's own
Python code where the path has some (SH evaluation ``utils/sh_utils.py``,
camera matrices ``utils/graphics_utils.py``, depth-to-normal
``utils/point_utils.py``, superquadric binding) through the fixtures under
``tests/golden/``, and by hand-derived known-answer cases; the tile binning
and the blend themselves are parity unpinned by a runnable reference.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

BLOCK_X = 16
BLOCK_Y = 16
BLOCK_SIZE = BLOCK_X * BLOCK_Y

PLAIN = 0
PART = 1

# P0/cr/auxiliary.h:37-60 (float device constants)
NEAR_N = 0.2
FAR_N = 100.0
FILTER_SIZE_P0 = 0.707106
FILTER_INV_SQUARE_P0 = 2.0
# P1/cr/auxiliary.h:20-21, 35-36 (double macros)
FILTER_SIZE_P1 = 0.7071067811865476
FILTER_INV_SQUARE_P1 = 1.0 / (FILTER_SIZE_P1 * FILTER_SIZE_P1)

SH_C0 = 0.28209479177387814
SH_C1 = 0.4886025119029199
SH_C2 = (1.0925484305920792, -1.0925484305920792, 0.31539156525252005,
         -1.0925484305920792, 0.5462742152960396)
SH_C3 = (-0.5900435899266435, 2.890611442640554, -0.4570457994644658,
         0.3731763325901154, -0.4570457994644658, 1.445305721320277,
         -0.5900435899266435)


# --------------------------------------------------------------------------
# inputs
# --------------------------------------------------------------------------
@dataclass
class Camera:
    """One view, in the layout the reference's settings carry
    (P0/diff_surfel_rasterization/__init__.py:158-170)."""
    viewmatrix: np.ndarray      # [16], world_view_transform flattened row-major
    projmatrix: np.ndarray      # [16], full_proj_transform flattened row-major
    campos: np.ndarray          # [3]
    tanfovx: float
    tanfovy: float
    height: int
    width: int


@dataclass
class Surfels:
    means3D: np.ndarray                      # [P,3]
    opacities: np.ndarray                    # [P] or [P,1]
    scales: np.ndarray | None = None         # [P,2]
    rotations: np.ndarray | None = None      # [P,4], real part first
    shs: np.ndarray | None = None            # [P,M,3]
    colors_precomp: np.ndarray | None = None  # [P,3]
    transmat_precomp: np.ndarray | None = None  # [P,9]
    semantics: np.ndarray | None = None      # [P,S] (part variant)
    sh_degree: int = 0
    scale_modifier: float = 1.0

    @property
    def P(self) -> int:
        return int(self.means3D.shape[0])


@dataclass
class ViewState:
    """Everything the forward keeps for the backward, plus diagnostics."""
    radii: np.ndarray
    tiles_touched: np.ndarray
    means2D: np.ndarray
    depths: np.ndarray
    transmat: np.ndarray
    normal_opacity: np.ndarray
    rgb: np.ndarray
    clamped: np.ndarray
    point_list: np.ndarray
    ranges: np.ndarray
    keys: np.ndarray
    final_T: np.ndarray      # [3,H,W]
    n_contrib: np.ndarray    # [2,H,W]
    color: np.ndarray        # [3,H,W]
    others: np.ndarray       # [7|8,H,W]
    semantic: np.ndarray | None
    amb_surfel: np.ndarray   # bool [P]
    amb_pixel: np.ndarray    # bool [H,W]
    fragments: int = 0
    extra: dict = field(default_factory=dict)


# --------------------------------------------------------------------------
# small helpers
# --------------------------------------------------------------------------
def _f(dtype):
    return np.dtype(dtype).type


def focal(width_or_height: int, tanfov: float, dtype) -> float:
    """focal = size / (2 tan) evaluated in single precision as the reference
    does (P0/cr/rasterizer_impl.cu:223-224)."""
    f = _f(dtype)
    if np.dtype(dtype) == np.float32:
        return np.float32(np.float32(width_or_height) / (np.float32(2.0) * np.float32(tanfov)))
    return f(width_or_height) / (f(2.0) * f(tanfov))


def quat_to_rotmat(q: np.ndarray) -> np.ndarray:
    """Rotation from a (w,x,y,z) quaternion after normalisation,
    P0/cr/auxiliary.h:213-235.  Returns R[P,3,3] in (row, col) order."""
    s = 1.0 / np.sqrt(q[:, 3] * q[:, 3] + q[:, 0] * q[:, 0] + q[:, 1] * q[:, 1] + q[:, 2] * q[:, 2])
    w, x, y, z = q[:, 0] * s, q[:, 1] * s, q[:, 2] * s, q[:, 3] * s
    R = np.empty((q.shape[0], 3, 3), dtype=q.dtype)
    R[:, 0, 0] = 1.0 - 2.0 * (y * y + z * z)
    R[:, 1, 0] = 2.0 * (x * y + w * z)
    R[:, 2, 0] = 2.0 * (x * z - w * y)
    R[:, 0, 1] = 2.0 * (x * y - w * z)
    R[:, 1, 1] = 1.0 - 2.0 * (x * x + z * z)
    R[:, 2, 1] = 2.0 * (y * z + w * x)
    R[:, 0, 2] = 2.0 * (x * z + w * y)
    R[:, 1, 2] = 2.0 * (y * z - w * x)
    R[:, 2, 2] = 1.0 - 2.0 * (x * x + y * y)
    return R


def quat_to_rotmat_vjp(q: np.ndarray, vR: np.ndarray) -> np.ndarray:
    """P0/cr/auxiliary.h:238-282.  vR is dL/dR in (row, col) order.  The
    result is the gradient w.r.t. the *normalised* quaternion components
    (the reference applies no normalisation Jacobian)."""
    s = 1.0 / np.sqrt(q[:, 3] * q[:, 3] + q[:, 0] * q[:, 0] + q[:, 1] * q[:, 1] + q[:, 2] * q[:, 2])
    w, x, y, z = q[:, 0] * s, q[:, 1] * s, q[:, 2] * s, q[:, 3] * s
    # glm v_R[c][r] == vR[:, r, c]
    g = lambda c, r: vR[:, r, c]  # noqa: E731
    out = np.empty_like(q)
    out[:, 0] = 2.0 * (x * (g(1, 2) - g(2, 1)) + y * (g(2, 0) - g(0, 2)) + z * (g(0, 1) - g(1, 0)))
    out[:, 1] = 2.0 * (-2.0 * x * (g(1, 1) + g(2, 2)) + y * (g(0, 1) + g(1, 0))
                       + z * (g(0, 2) + g(2, 0)) + w * (g(1, 2) - g(2, 1)))
    out[:, 2] = 2.0 * (x * (g(0, 1) + g(1, 0)) - 2.0 * y * (g(0, 0) + g(2, 2))
                       + z * (g(1, 2) + g(2, 1)) + w * (g(2, 0) - g(0, 2)))
    out[:, 3] = 2.0 * (x * (g(0, 2) + g(2, 0)) + y * (g(1, 2) + g(2, 1))
                       - 2.0 * z * (g(0, 0) + g(1, 1)) + w * (g(0, 1) - g(1, 0)))
    return out


def sh_to_rgb(deg: int, sh: np.ndarray, means: np.ndarray, campos: np.ndarray):
    """computeColorFromSH, P0/cr/forward.cu:20-71.  Returns (rgb, clamped, dir_orig)."""
    dir_orig = means - campos[None, :]
    n = np.sqrt(np.sum(dir_orig * dir_orig, axis=1))
    d = dir_orig / n[:, None]
    x, y, z = d[:, 0:1], d[:, 1:2], d[:, 2:3]
    res = SH_C0 * sh[:, 0]
    if deg > 0:
        res = res - SH_C1 * y * sh[:, 1] + SH_C1 * z * sh[:, 2] - SH_C1 * x * sh[:, 3]
        if deg > 1:
            xx, yy, zz = x * x, y * y, z * z
            xy, yz, xz = x * y, y * z, x * z
            res = (res + SH_C2[0] * xy * sh[:, 4] + SH_C2[1] * yz * sh[:, 5]
                   + SH_C2[2] * (2.0 * zz - xx - yy) * sh[:, 6]
                   + SH_C2[3] * xz * sh[:, 7] + SH_C2[4] * (xx - yy) * sh[:, 8])
            if deg > 2:
                res = (res + SH_C3[0] * y * (3.0 * xx - yy) * sh[:, 9]
                       + SH_C3[1] * xy * z * sh[:, 10]
                       + SH_C3[2] * y * (4.0 * zz - xx - yy) * sh[:, 11]
                       + SH_C3[3] * z * (2.0 * zz - 3.0 * xx - 3.0 * yy) * sh[:, 12]
                       + SH_C3[4] * x * (4.0 * zz - xx - yy) * sh[:, 13]
                       + SH_C3[5] * z * (xx - yy) * sh[:, 14]
                       + SH_C3[6] * x * (xx - 3.0 * yy) * sh[:, 15])
    res = res + 0.5
    clamped = res < 0
    return np.maximum(res, 0.0), clamped, dir_orig


def sh_backward(deg, sh, dir_orig, clamped, dL_dcolor):
    """SH part of the preprocess backward, P0/cr/backward.cu:20-139.
    Returns (dL_dsh [P,M,3], dL_dmean contribution [P,3])."""
    P, M = sh.shape[0], sh.shape[1]
    n = np.sqrt(np.sum(dir_orig * dir_orig, axis=1))
    d = dir_orig / n[:, None]
    x, y, z = d[:, 0:1], d[:, 1:2], d[:, 2:3]
    g = np.where(clamped, 0.0, dL_dcolor).astype(dL_dcolor.dtype)
    dsh = np.zeros_like(sh)
    dsh[:, 0] = SH_C0 * g
    dx = np.zeros_like(g)
    dy = np.zeros_like(g)
    dz = np.zeros_like(g)
    if deg > 0:
        dsh[:, 1] = -SH_C1 * y * g
        dsh[:, 2] = SH_C1 * z * g
        dsh[:, 3] = -SH_C1 * x * g
        dx = -SH_C1 * sh[:, 3]
        dy = -SH_C1 * sh[:, 1]
        dz = SH_C1 * sh[:, 2]
        if deg > 1:
            xx, yy, zz = x * x, y * y, z * z
            xy, yz, xz = x * y, y * z, x * z
            dsh[:, 4] = SH_C2[0] * xy * g
            dsh[:, 5] = SH_C2[1] * yz * g
            dsh[:, 6] = SH_C2[2] * (2.0 * zz - xx - yy) * g
            dsh[:, 7] = SH_C2[3] * xz * g
            dsh[:, 8] = SH_C2[4] * (xx - yy) * g
            dx = dx + SH_C2[0] * y * sh[:, 4] + SH_C2[2] * 2.0 * -x * sh[:, 6] + SH_C2[3] * z * sh[:, 7] + SH_C2[4] * 2.0 * x * sh[:, 8]
            dy = dy + SH_C2[0] * x * sh[:, 4] + SH_C2[1] * z * sh[:, 5] + SH_C2[2] * 2.0 * -y * sh[:, 6] + SH_C2[4] * 2.0 * -y * sh[:, 8]
            dz = dz + SH_C2[1] * y * sh[:, 5] + SH_C2[2] * 2.0 * 2.0 * z * sh[:, 6] + SH_C2[3] * x * sh[:, 7]
            if deg > 2:
                dsh[:, 9] = SH_C3[0] * y * (3.0 * xx - yy) * g
                dsh[:, 10] = SH_C3[1] * xy * z * g
                dsh[:, 11] = SH_C3[2] * y * (4.0 * zz - xx - yy) * g
                dsh[:, 12] = SH_C3[3] * z * (2.0 * zz - 3.0 * xx - 3.0 * yy) * g
                dsh[:, 13] = SH_C3[4] * x * (4.0 * zz - xx - yy) * g
                dsh[:, 14] = SH_C3[5] * z * (xx - yy) * g
                dsh[:, 15] = SH_C3[6] * x * (xx - 3.0 * yy) * g
                dx = dx + (SH_C3[0] * sh[:, 9] * 3.0 * 2.0 * xy + SH_C3[1] * sh[:, 10] * yz
                           + SH_C3[2] * sh[:, 11] * -2.0 * xy + SH_C3[3] * sh[:, 12] * -3.0 * 2.0 * xz
                           + SH_C3[4] * sh[:, 13] * (-3.0 * xx + 4.0 * zz - yy)
                           + SH_C3[5] * sh[:, 14] * 2.0 * xz + SH_C3[6] * sh[:, 15] * 3.0 * (xx - yy))
                dy = dy + (SH_C3[0] * sh[:, 9] * 3.0 * (xx - yy) + SH_C3[1] * sh[:, 10] * xz
                           + SH_C3[2] * sh[:, 11] * (-3.0 * yy + 4.0 * zz - xx)
                           + SH_C3[3] * sh[:, 12] * -3.0 * 2.0 * yz + SH_C3[4] * sh[:, 13] * -2.0 * xy
                           + SH_C3[5] * sh[:, 14] * -2.0 * yz + SH_C3[6] * sh[:, 15] * -3.0 * 2.0 * xy)
                dz = dz + (SH_C3[1] * sh[:, 10] * xy + SH_C3[2] * sh[:, 11] * 4.0 * 2.0 * yz
                           + SH_C3[3] * sh[:, 12] * 3.0 * (2.0 * zz - xx - yy)
                           + SH_C3[4] * sh[:, 13] * 4.0 * 2.0 * xz + SH_C3[5] * sh[:, 14] * (xx - yy))
    dL_ddir = np.stack([np.sum(dx * g, 1), np.sum(dy * g, 1), np.sum(dz * g, 1)], axis=1)
    return dsh, dnormvdv(dir_orig, dL_ddir)


def dnormvdv(v, dv):
    """P0/cr/auxiliary.h:128-138."""
    sum2 = np.sum(v * v, axis=1)
    inv = 1.0 / np.sqrt(sum2 * sum2 * sum2)
    out = np.empty_like(v)
    out[:, 0] = ((sum2 - v[:, 0] * v[:, 0]) * dv[:, 0] - v[:, 1] * v[:, 0] * dv[:, 1] - v[:, 2] * v[:, 0] * dv[:, 2]) * inv
    out[:, 1] = (-v[:, 0] * v[:, 1] * dv[:, 0] + (sum2 - v[:, 1] * v[:, 1]) * dv[:, 1] - v[:, 2] * v[:, 1] * dv[:, 2]) * inv
    out[:, 2] = (-v[:, 0] * v[:, 2] * dv[:, 0] - v[:, 1] * v[:, 2] * dv[:, 1] + (sum2 - v[:, 2] * v[:, 2]) * dv[:, 2]) * inv
    return out


def _near_int(v, tol):
    """True where v lies within a relative tol of an integer (a truncation or
    ceil there may go either way in single precision)."""
    return np.abs(v - np.round(v)) <= tol * np.maximum(1.0, np.abs(v))


EPS32 = 2.0 ** -24       # unit roundoff of float32
FP32_ROUNDINGS = 4       # roundings an FP32 evaluation of a short sum accumulates (a bound)


def _near_int_abs(v, err):
    """True where v lies within an absolute err of an integer."""
    return np.abs(v - np.round(v)) <= err


def _extent_err(h0, mag):
    """Absolute FP32 error bound of sqrt(max(0, h0)) when h0 is a difference
    whose terms sum to ``mag`` in magnitude: the cancellation in h0 leaves
    an error of about FP32_ROUNDINGS * EPS32 * mag there, and the square
    root divides it by 2 sqrt(h0)."""
    dh0 = FP32_ROUNDINGS * EPS32 * mag
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.where(h0 > dh0, dh0 / (2.0 * np.sqrt(np.maximum(h0, dh0))), np.sqrt(dh0))


def _rect(px, py, radius, gx, gy, f):
    """getRect, P0/cr/auxiliary.h:67-77: truncation toward zero, clamped."""
    def trunc_clamp(v, hi):
        t = np.trunc(np.clip(v, -2.0e9, 2.0e9)).astype(np.int64)
        return np.minimum(hi, np.maximum(0, t))
    r = radius.astype(f)
    xmin = trunc_clamp((px - r) / f(BLOCK_X), gx)
    ymin = trunc_clamp((py - r) / f(BLOCK_Y), gy)
    xmax = trunc_clamp((px + r + f(BLOCK_X - 1)) / f(BLOCK_X), gx)
    ymax = trunc_clamp((py + r + f(BLOCK_Y - 1)) / f(BLOCK_Y), gy)
    return xmin, ymin, xmax, ymax


# --------------------------------------------------------------------------
# preprocess forward
# --------------------------------------------------------------------------
def preprocess(s: Surfels, cam: Camera, variant=PLAIN, dtype=np.float64, amb_tol=2e-6):
    f = _f(dtype)
    P = s.P
    W, H = cam.width, cam.height
    gx, gy = (W + BLOCK_X - 1) // BLOCK_X, (H + BLOCK_Y - 1) // BLOCK_Y
    vm = cam.viewmatrix.astype(dtype)
    pm = cam.projmatrix.astype(dtype)
    Vm = vm.reshape(4, 4)
    F = pm.reshape(4, 4)
    p = s.means3D.astype(dtype)
    opac = s.opacities.reshape(-1).astype(dtype)
    fx = focal(W, cam.tanfovx, dtype)
    fy = focal(H, cam.tanfovy, dtype)

    # in_frustum (P0/cr/auxiliary.h:185-210); only the near test culls
    p_view = p @ Vm[:3, :3] + Vm[3, :3]
    alive = p_view[:, 2] > f(np.float32(0.2))
    amb_near = np.abs(p_view[:, 2] - 0.2) <= amb_tol * 0.2
    amb = np.zeros(P, bool)

    transmat = np.zeros((P, 9), dtype=dtype)
    normal = np.zeros((P, 3), dtype=dtype)
    facing = np.ones(P, bool)      # the normal's orientation decision (the DUAL_VISIABLE flip)
    if s.transmat_precomp is not None:
        transmat[:] = s.transmat_precomp.astype(dtype)
        if variant == PLAIN:
            normal[:, 2] = 1.0       # P0/cr/forward.cu:206
        # P1 leaves the normal uninitialised with a precomputed transMat
        # (P1/cr/forward.cu:212-218); it is defined as zero here.
    else:
        R = quat_to_rotmat(s.rotations.astype(dtype))
        sc = s.scales.astype(dtype)
        if variant == PLAIN:
            mod = f(s.scale_modifier)
            L0 = R[:, :, 0] * (mod * sc[:, 0:1])
            L1 = R[:, :, 1] * (mod * sc[:, 1:2])
            L2 = R[:, :, 2]
            n0 = np.array([W / 2.0, 0.0, 0.0, (W - 1) / 2.0], dtype=dtype)
            n1 = np.array([0.0, H / 2.0, 0.0, (H - 1) / 2.0], dtype=dtype)
            n2 = np.array([0.0, 0.0, 0.0, 1.0], dtype=dtype)
            Nmat = np.stack([n0, n1, n2], axis=1)                       # [4,3]
            A0 = L0 @ F[:3, :]
            A1 = L1 @ F[:3, :]
            A2 = p @ F[:3, :] + F[3, :]
            Tu = np.stack([A0 @ Nmat[:, 0], A1 @ Nmat[:, 0], A2 @ Nmat[:, 0]], 1)
            Tv = np.stack([A0 @ Nmat[:, 1], A1 @ Nmat[:, 1], A2 @ Nmat[:, 1]], 1)
            Tw = np.stack([A0 @ Nmat[:, 2], A1 @ Nmat[:, 2], A2 @ Nmat[:, 2]], 1)
            transmat = np.concatenate([Tu, Tv, Tw], 1)
            normal = L2 @ Vm[:3, :3]
        else:
            W3 = Vm[:3, :3].T
            cx, cy = f(W / 2.0), f(H / 2.0)
            m0 = (R[:, :, 0] * sc[:, 0:1]) @ W3.T
            m1 = (R[:, :, 1] * sc[:, 1:2]) @ W3.T
            pv = p @ W3.T + Vm[3, :3]
            tn = R[:, :, 2] @ W3.T
            cosv = np.sum(-tn * pv, 1)
            alive &= cosv != 0
            facing = cosv > 0
            tn = tn * np.where(cosv > 0, 1.0, -1.0).astype(dtype)[:, None]
            Tu = np.stack([fx * m0[:, 0] + cx * m0[:, 2], fx * m1[:, 0] + cx * m1[:, 2], fx * pv[:, 0] + cx * pv[:, 2]], 1)
            Tv = np.stack([fy * m0[:, 1] + cy * m0[:, 2], fy * m1[:, 1] + cy * m1[:, 2], fy * pv[:, 1] + cy * pv[:, 2]], 1)
            Tw = np.stack([m0[:, 2], m1[:, 2], pv[:, 2]], 1)
            transmat = np.concatenate([Tu, Tv, Tw], 1)
            normal = tn

    if variant == PLAIN:
        # DUAL_VISIABLE flip (P0/cr/forward.cu:209-214)
        cosv = -np.sum(p_view * normal, 1)
        alive &= cosv != 0
        facing = cosv > 0
        normal = normal * np.where(cosv > 0, 1.0, -1.0).astype(dtype)[:, None]

    Tu, Tv, Tw = transmat[:, 0:3], transmat[:, 3:6], transmat[:, 6:9]
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        if variant == PLAIN:
            t = np.array([9.0, 9.0, -1.0], dtype=dtype)
            d = np.sum(t * Tw * Tw, 1)
            alive &= d != 0
            fv = (1.0 / d)[:, None] * t
            px = np.sum(fv * Tu * Tw, 1)
            py = np.sum(fv * Tv * Tw, 1)
            h0x = px * px - np.sum(fv * Tu * Tu, 1)
            h0y = py * py - np.sum(fv * Tv * Tv, 1)
            lo = f(np.float32(1e-4))
            hx = np.sqrt(np.maximum(lo, h0x))
            hy = np.sqrt(np.maximum(lo, h0y))
            ext = np.maximum(hx, hy)
            rad_in = np.maximum(ext, f(np.float32(3.0) * np.float32(FILTER_SIZE_P0)))
            radius = np.ceil(rad_in)
            amb |= (ext > 2.2) & _near_int(ext, amb_tol)
            # the extent is a difference of products of pixel-scale terms: its
            # FP32 evaluation can miss by far more than a relative 2e-6
            ex = _extent_err(h0x, px * px + np.abs(np.sum(fv * Tu * Tu, 1)))
            ey = _extent_err(h0y, py * py + np.abs(np.sum(fv * Tv * Tv, 1)))
            e_ext = np.where(hx >= hy, ex, ey)
            amb |= (ext > 2.2) & _near_int_abs(ext, e_ext)
            rad_err = np.where(ext > 2.2, np.maximum(amb_tol * np.abs(ext), e_ext), 0.0)
        else:
            t = np.array([1.0, 1.0, -1.0], dtype=dtype)
            d = np.sum(t * Tw * Tw, 1)
            alive &= d != 0
            fv = t * (1.0 / d)[:, None]
            px = np.sum(fv * Tu * Tw, 1)
            py = np.sum(fv * Tv * Tw, 1)
            h0x = px * px - np.sum(fv * Tu * Tu, 1)
            h0y = py * py - np.sum(fv * Tv * Tv, 1)
            hx = np.sqrt(np.maximum(0.0, h0x))
            hy = np.sqrt(np.maximum(0.0, h0y))
            ext = np.maximum(hx, hy).astype(np.float64)
            rad_in = 3.0 * np.maximum(ext, FILTER_SIZE_P1)
            radius = np.ceil(rad_in).astype(dtype)
            amb |= (ext > FILTER_SIZE_P1) & _near_int(rad_in, amb_tol)
            ex = _extent_err(h0x, px * px + np.abs(np.sum(fv * Tu * Tu, 1)))
            ey = _extent_err(h0y, py * py + np.abs(np.sum(fv * Tv * Tv, 1)))
            e_ext = np.where(hx >= hy, ex, ey)
            amb |= (ext > FILTER_SIZE_P1) & _near_int_abs(rad_in, 3.0 * e_ext)
            rad_err = np.where(ext > FILTER_SIZE_P1, np.maximum(amb_tol * np.abs(rad_in), 3.0 * e_ext), 0.0)
        # FP32 error bound of the screen centre (a short sum of products)
        ctr_err = np.stack([FP32_ROUNDINGS * EPS32 * np.sum(np.abs(fv * Tu * Tw), 1),
                            FP32_ROUNDINGS * EPS32 * np.sum(np.abs(fv * Tv * Tw), 1)], 1)
        radius = np.where(alive, radius, 0).astype(dtype)
        px = np.where(alive, px, 0).astype(dtype)
        py = np.where(alive, py, 0).astype(dtype)
        xmin, ymin, xmax, ymax = _rect(px, py, radius, gx, gy, f)
        for v, ce in (((px - radius) / f(BLOCK_X), ctr_err[:, 0]), ((py - radius) / f(BLOCK_Y), ctr_err[:, 1]),
                      ((px + radius + f(BLOCK_X - 1)) / f(BLOCK_X), ctr_err[:, 0]),
                      ((py + radius + f(BLOCK_Y - 1)) / f(BLOCK_Y), ctr_err[:, 1])):
            near = _near_int(v, amb_tol) | _near_int_abs(v, ce / BLOCK_X)
            amb |= near & (v > -1) & (v < max(gx, gy) + 1)
    # a decision close to its threshold matters only for surfels that reach
    # the rectangle stage, or sit on the near plane
    amb = (amb & alive) | amb_near
    touched = (ymax - ymin) * (xmax - xmin)
    alive &= touched > 0

    rgb = np.zeros((P, 3), dtype=dtype)
    clamped = np.zeros((P, 3), dtype=bool)
    if s.colors_precomp is not None:
        rgb = s.colors_precomp.astype(dtype).copy()
    else:
        rgb, clamped, _ = sh_to_rgb(s.sh_degree, s.shs.astype(dtype), p, cam.campos.astype(dtype))

    radii = np.where(alive, radius, 0).astype(np.int32)
    return dict(
        radii=radii,
        tiles_touched=np.where(alive, touched, 0).astype(np.int64),
        rect=(xmin, ymin, xmax, ymax),
        means2D=np.stack([px, py], 1),
        depths=p_view[:, 2].copy(),
        transmat=transmat,
        normal_opacity=np.concatenate([normal, opac[:, None]], 1),
        rgb=rgb,
        clamped=clamped,
        alive=alive,
        amb=amb,
        facing=facing,
        rad_in=np.where(alive, rad_in, 0.0).astype(np.float64),
        rad_err=np.where(alive, rad_err, 0.0).astype(np.float64),
        ctr_err=ctr_err.astype(np.float64),
        grid=(gx, gy),
        focal=(fx, fy),
    )


# --------------------------------------------------------------------------
# tile binning (P0/cr/rasterizer_impl.cu:70-138, 278-318)
# --------------------------------------------------------------------------
def bin_tiles(pre: dict, exact_depth: bool = False):
    """Per-tile depth-ordered lists: (point_list, ranges [tiles, 2], keys).
    The reference orders by the FP32 bits of the depth (ties by index);
    with ``exact_depth`` the order uses the depth itself (finite-difference
    checks: FP32 ties among neighbouring surfels would otherwise trade
    places under tiny perturbations)."""
    gx, gy = pre["grid"]
    xmin, ymin, xmax, ymax = pre["rect"]
    alive = pre["alive"]
    depth_bits = pre["depths"].astype(np.float32).view(np.uint32).astype(np.uint64)
    ntiles = gx * gy
    vis = np.nonzero(alive)[0]
    w = (xmax - xmin)[vis]
    n = ((ymax - ymin)[vis] * w).astype(np.int64)
    if n.sum() == 0:
        return (np.zeros(0, np.int64), np.zeros((ntiles, 2), np.int64), np.zeros(0, np.uint64))
    # one key per (surfel, tile), surfels in index order, tiles row-major
    # inside each surfel's rectangle (P0/cr/rasterizer_impl.cu:98-109)
    ids = np.repeat(vis, n)
    starts = np.cumsum(n) - n
    local = np.arange(int(n.sum()), dtype=np.int64) - np.repeat(starts, n)
    wr = np.repeat(w, n)
    tiles = (ymin[ids] + local // wr) * gx + (xmin[ids] + local % wr)
    tiles = tiles.astype(np.int64)
    keys = (tiles.astype(np.uint64) << np.uint64(32)) | depth_bits[ids]
    # stable sort by the 64-bit key: equal keys keep emission (index) order
    if exact_depth:
        order = np.lexsort((np.arange(len(ids)), pre["depths"][ids], tiles))
    else:
        order = np.argsort(keys, kind="stable")
    keys = keys[order]
    point_list = ids[order]
    tsorted = tiles[order]
    starts = np.searchsorted(tsorted, np.arange(ntiles), side="left")
    ends = np.searchsorted(tsorted, np.arange(ntiles), side="right")
    ranges = np.stack([starts, ends], 1).astype(np.int64)
    ranges[starts == ends] = 0
    return point_list, ranges, keys


def _tile_pixels(gx, gy, W, H, variant, f, tiles=None):
    """Per tile, per thread: pixel coordinates and the inside mask (all
    tiles, or the subset ``tiles``)."""
    ids = np.arange(gx * gy) if tiles is None else np.asarray(tiles)
    ty, tx = np.divmod(ids, gx)
    ly, lx = np.divmod(np.arange(BLOCK_SIZE), BLOCK_X)
    X = tx[:, None] * BLOCK_X + lx[None, :]
    Y = ty[:, None] * BLOCK_Y + ly[None, :]
    inside = (X < W) & (Y < H)
    off = 0.5 if variant == PART else 0.0
    return X, Y, X.astype(f) + f(off), Y.astype(f) + f(off), inside


def _padded_lists(point_list, ranges, tiles=None):
    if tiles is not None:
        ranges = ranges[np.asarray(tiles)]
    lens = ranges[:, 1] - ranges[:, 0]
    L = int(lens.max()) if lens.size else 0
    lists = np.full((ranges.shape[0], max(L, 1)), -1, dtype=np.int64)
    for t in np.nonzero(lens)[0]:
        lists[t, :lens[t]] = point_list[ranges[t, 0]:ranges[t, 1]]
    return lists, lens, L


# --------------------------------------------------------------------------
# blend forward
# --------------------------------------------------------------------------
def _intersect(variant, f, px_f, py_f, Tu, Tv, Tw, xy):
    """Ray-splat intersection shared by the forward and the backward
    (P0/cr/forward.cu:349-366, P1/cr/forward.cu:361-387)."""
    if variant == PLAIN:
        k = [px_f * Tw[..., i] - Tu[..., i] for i in range(3)]
        l = [py_f * Tw[..., i] - Tv[..., i] for i in range(3)]
    else:
        k = [-Tu[..., i] + px_f * Tw[..., i] for i in range(3)]
        l = [-Tv[..., i] + py_f * Tw[..., i] for i in range(3)]
    pvec = [k[1] * l[2] - k[2] * l[1], k[2] * l[0] - k[0] * l[2], k[0] * l[1] - k[1] * l[0]]
    with np.errstate(divide="ignore", invalid="ignore"):
        sx = pvec[0] / pvec[2]
        sy = pvec[1] / pvec[2]
    rho3d = sx * sx + sy * sy
    dx = xy[..., 0] - px_f
    dy = xy[..., 1] - py_f
    if variant == PLAIN:
        rho2d = f(FILTER_INV_SQUARE_P0) * (dx * dx + dy * dy)
    else:
        rho2d = (FILTER_INV_SQUARE_P1 * (dx * dx + dy * dy).astype(np.float64)).astype(f)
    use3d = rho3d <= rho2d
    rho = np.minimum(rho3d, rho2d)
    depth = np.where(use3d, (sx * Tw[..., 0] + sy * Tw[..., 1]) + Tw[..., 2], Tw[..., 2])
    return k, l, pvec, sx, sy, rho3d, rho2d, rho, depth, use3d, dx, dy


def _mapped_depth(variant, f, depth):
    if variant == PLAIN:
        return f(FAR_N) / (f(FAR_N) - f(NEAR_N)) * (1.0 - f(NEAR_N) / depth)
    d64 = depth.astype(np.float64)
    return ((100.0 * d64 - 100.0 * 0.2) / ((100.0 - 0.2) * d64)).astype(f)


def render_forward(pre, point_list, ranges, cam: Camera, s: Surfels, bg, variant=PLAIN, dtype=np.float64,
                   amb_tol=2e-6, tiles=None, alpha_tol=None):
    f = _f(dtype)
    gx, gy = pre["grid"]
    W, H = cam.width, cam.height
    X, Y, pxf, pyf, inside = _tile_pixels(gx, gy, W, H, variant, f, tiles)
    lists, lens, L = _padded_lists(point_list, ranges, tiles)
    nt = lists.shape[0]
    Sn = 0 if s.semantics is None else s.semantics.shape[1]
    sem_all = None if s.semantics is None else s.semantics.astype(dtype)
    tm, xy2, no, rgb = pre["transmat"], pre["means2D"], pre["normal_opacity"], pre["rgb"]
    bg = np.asarray(bg, dtype=dtype)

    shape = (nt, BLOCK_SIZE)
    T = np.ones(shape, dtype)
    done = ~inside
    contributor = np.zeros(shape, np.int64)
    last_contributor = np.zeros(shape, np.int64)
    C = np.zeros(shape + (3,), dtype)
    Nn = np.zeros(shape + (3,), dtype)
    D = np.zeros(shape, dtype)
    M1 = np.zeros(shape, dtype)
    M2 = np.zeros(shape, dtype)
    dist = np.zeros(shape, dtype)
    med_depth = np.zeros(shape, dtype)
    med_weight = np.zeros(shape, dtype)
    med_contrib = np.full(shape, -1, np.int64)
    Sem = np.zeros(shape + (Sn,), dtype)
    amb = np.zeros(shape, bool)
    # rolling hash of the discrete path per pixel (which surfels were blended
    # at which list positions -- so two surfels trading depth order count
    # too -- through which branch, with which normal orientation, whether
    # alpha sat at its 0.99 cap, which colour channels the SH clamp zeroed,
    # and where the walk stopped): equal signatures mean the same decisions
    # (finite-difference checks use it)
    sig = np.zeros(shape, np.int64)
    frags = 0
    for j in range(L):
        if done.all():
            break
        ids = lists[:, j]
        has = (ids >= 0)[:, None]
        act = has & ~done
        if not act.any():
            continue
        idc = np.where(ids >= 0, ids, 0)
        contributor += act
        frags += int(act.sum())
        Tu = tm[idc, 0:3][:, None, :]
        Tv = tm[idc, 3:6][:, None, :]
        Tw = tm[idc, 6:9][:, None, :]
        xy = xy2[idc][:, None, :]
        k, l, pv, sx, sy, rho3d, rho2d, rho, depth, use3d, dx, dy = _intersect(variant, f, pxf, pyf, Tu, Tv, Tw, xy)
        ok = act & (pv[2] != 0)
        ok &= ~(depth < NEAR_N) if variant == PART else ~(depth < f(np.float32(NEAR_N)))
        power = f(-0.5) * rho
        ok &= ~(power > 0)
        opa = no[idc, 3][:, None]
        with np.errstate(over="ignore", invalid="ignore"):
            alpha = np.minimum(f(0.99), opa * np.exp(power))
        ok &= ~(alpha < f(1.0) / f(255.0))
        test_T = T * (1 - alpha)
        # ambiguity bookkeeping (only where a decision is close)
        # the alpha cutoff and the stop test take alpha_tol (default amb_tol):
        # near the cutoff alpha carries the FP32 error of the splat
        # intersection's cross product, which cancels for distant pixels
        a_tol = amb_tol if alpha_tol is None else alpha_tol
        near_alpha = act & (np.abs(alpha - 1 / 255.0) <= a_tol / 255.0)
        near_branch = act & (np.abs(rho3d - rho2d) <= amb_tol * np.maximum(rho3d, rho2d)) & (rho < 12.0)
        stop = ok & (test_T < f(1e-4))
        near_stop = ok & (np.abs(test_T - 1e-4) <= a_tol * 1e-4)
        acc = ok & ~stop
        near_med = acc & (np.abs(T - 0.5) <= amb_tol)
        amb |= near_alpha | near_branch | near_stop | near_med
        done = done | stop
        if not acc.any():
            continue
        w = alpha * T
        m = _mapped_depth(variant, f, depth)
        A = 1 - T
        if variant == PLAIN:
            dist_new = dist + (m * m * A + M2 - 2 * m * M1) * w
            D_new = D + depth * w
            M1_new = M1 + m * w
            M2_new = M2 + m * m * w
        else:
            err = m * m * A + M2 - 2 * m * M1
            dist_new = dist + err * alpha * T
            D_new = D + depth * alpha * T
            M1_new = M1 + m * alpha * T
            M2_new = M2 + m * m * alpha * T
        dist = np.where(acc, dist_new, dist)
        D = np.where(acc, D_new, D)
        M1 = np.where(acc, M1_new, M1)
        M2 = np.where(acc, M2_new, M2)
        med = acc & (T > 0.5)
        med_depth = np.where(med, depth, med_depth)
        med_weight = np.where(med, alpha * T, med_weight)
        med_contrib = np.where(med, contributor, med_contrib)
        nrm = no[idc, 0:3][:, None, :]
        col = rgb[idc][:, None, :]
        if variant == PLAIN:
            Nn = np.where(acc[..., None], Nn + nrm * w[..., None], Nn)
            C = np.where(acc[..., None], C + col * w[..., None], C)
        else:
            Nn = np.where(acc[..., None], Nn + nrm * alpha[..., None] * T[..., None], Nn)
            C = np.where(acc[..., None], C + col * alpha[..., None] * T[..., None], C)
            if Sn:
                sid = s_surfel_ids(idc)
                sv = sem_all[sid][:, None, :]
                Sem = np.where(acc[..., None], Sem + sv * alpha[..., None] * T[..., None], Sem)
        T = np.where(acc, test_T, T)
        last_contributor = np.where(acc, contributor, last_contributor)
        sat = alpha >= f(0.99)
        clamp = pre["clamped"][idc].astype(np.int64) @ np.array([1, 2, 4], np.int64)
        code = ((((contributor + idc.astype(np.int64)[:, None] * 4099) * 8 + clamp[:, None]) * 16
                 + sat.astype(np.int64) * 8 + use3d.astype(np.int64) * 4 + med.astype(np.int64) * 2
                 + pre["facing"][idc].astype(np.int64)[:, None]))
        sig = np.where(acc, sig * np.int64(1000003) + code, sig)

    HW = (H, W)
    out = lambda a, fill=0: _scatter_pixels(a, X, Y, inside, HW, fill)  # noqa: E731
    final_T = np.stack([out(T), out(M1), out(M2)])
    n_contrib = np.stack([out(last_contributor), out(np.maximum(med_contrib, 0))]).astype(np.int64)
    color = np.stack([out(C[..., c] + T * bg[c]) for c in range(3)])
    others = [out(D), out(1 - T)] + [out(Nn[..., c]) for c in range(3)] + [out(med_depth), out(dist)]
    if variant == PART:
        others.append(out(med_weight))
    semantic = None
    if variant == PART:
        semantic = (np.stack([out(Sem[..., c]) for c in range(Sn)]) if Sn
                    else np.zeros((0, H, W), dtype=dtype))
    return dict(final_T=final_T, n_contrib=n_contrib, color=color, others=np.stack(others),
                semantic=semantic, amb_pixel=out(amb).astype(bool), fragments=frags,
                signature=out(sig * np.int64(31) + done.astype(np.int64)))


def s_surfel_ids(idc):
    return idc


def _scatter_pixels(a, X, Y, inside, HW, fill=0):
    out = np.full(HW, fill, dtype=a.dtype)
    out[Y[inside], X[inside]] = a[inside]
    return out


def _gather_pixels(img, X, Y, inside):
    out = np.zeros(X.shape, dtype=img.dtype)
    out[inside] = img[Y[inside], X[inside]]
    return out


# --------------------------------------------------------------------------
# full forward of one view
# --------------------------------------------------------------------------
def forward_view(s: Surfels, cam: Camera, bg, variant=PLAIN, dtype=np.float64, amb_tol=2e-6,
                 tiles=None, alpha_tol=None, exact_depth=False) -> ViewState:
    """Forward of one view; with ``tiles`` only those tiles are blended (the
    other pixels stay zero)."""
    pre = preprocess(s, cam, variant, dtype, amb_tol)
    point_list, ranges, keys = bin_tiles(pre, exact_depth)
    rf = render_forward(pre, point_list, ranges, cam, s, bg, variant, dtype, amb_tol, tiles, alpha_tol)
    st = ViewState(
        radii=pre["radii"], tiles_touched=pre["tiles_touched"], means2D=pre["means2D"],
        depths=pre["depths"], transmat=pre["transmat"], normal_opacity=pre["normal_opacity"],
        rgb=pre["rgb"], clamped=pre["clamped"], point_list=point_list, ranges=ranges, keys=keys,
        final_T=rf["final_T"], n_contrib=rf["n_contrib"], color=rf["color"], others=rf["others"],
        semantic=rf["semantic"], amb_surfel=pre["amb"], amb_pixel=rf["amb_pixel"], fragments=rf["fragments"])
    st.extra["pre"] = pre
    st.extra["signature"] = rf["signature"]
    # An ambiguous surfel's rectangle may come out one tile larger or
    # smaller in FP32: the tiles inside some but not all of the rectangles
    # its radius and centre can round to may or may not list it.  Those
    # tiles' lists are ambiguous; so are, in them, the pixels the surfel can
    # reach (alpha at the cut-off) and the pixels whose last contributor
    # lies after the surfel's place in the list (their contributor count
    # shifts by one).
    gx, gy = pre["grid"]
    amb_tiles = np.zeros((gy, gx), bool)
    f = _f(dtype)
    last = st.n_contrib[0]
    shift = np.zeros_like(st.amb_pixel)
    for i in np.nonzero(pre["amb"])[0]:
        cx, cy = pre["means2D"][i]
        r_lo = np.ceil(max(pre["rad_in"][i] - pre["rad_err"][i], 0.0))
        r_hi = np.ceil(pre["rad_in"][i] + pre["rad_err"][i])
        ex, ey = pre["ctr_err"][i] + 1e-9
        rects = [_rect(np.array([x]), np.array([y]), np.array([r]), gx, gy, np.float64)
                 for x in (cx - ex, cx + ex) for y in (cy - ey, cy + ey) for r in (r_lo, r_hi)]
        R = np.array([[int(c[0]) for c in rc] for rc in rects])       # [8, 4] xmin ymin xmax ymax
        ux0, uy0, ux1, uy1 = R[:, 0].min(), R[:, 1].min(), R[:, 2].max(), R[:, 3].max()
        ix0, iy0, ix1, iy1 = R[:, 0].max(), R[:, 1].max(), R[:, 2].min(), R[:, 3].min()
        band = np.zeros((gy, gx), bool)
        band[uy0:uy1, ux0:ux1] = True
        if ix1 > ix0 and iy1 > iy0:
            band[iy0:iy1, ix0:ix1] = False
        if not band.any():
            continue
        amb_tiles |= band
        key_i = int(np.float32(pre["depths"][i]).view(np.uint32))
        off = 0.5 if variant == PART else 0.0
        tmi = pre["transmat"][i]
        for ty, tx in zip(*np.nonzero(band)):
            px0, px1 = tx * BLOCK_X, min(cam.width, (tx + 1) * BLOCK_X)
            py0, py1 = ty * BLOCK_Y, min(cam.height, (ty + 1) * BLOCK_Y)
            yy, xx = np.mgrid[py0:py1, px0:px1]
            res = _intersect(variant, f, xx.astype(f) + f(off), yy.astype(f) + f(off),
                             tmi[0:3], tmi[3:6], tmi[6:9], pre["means2D"][i])
            with np.errstate(over="ignore", invalid="ignore"):
                a = pre["normal_opacity"][i, 3] * np.exp(-0.5 * res[7])
            t = ty * gx + tx
            lst = st.point_list[st.ranges[t, 0]:st.ranges[t, 1]]
            dk = pre["depths"][lst].astype(np.float32).view(np.uint32).astype(np.int64)
            place = int(np.sum((dk < key_i) | ((dk == key_i) & (lst < i))))   # the surfel's list position
            st.amb_pixel[py0:py1, px0:px1] |= a >= (1.0 - 1e-3) / 255.0
            shift[py0:py1, px0:px1] |= last[py0:py1, px0:px1] > place
    st.extra["amb_count_pixel"] = st.amb_pixel | shift
    st.extra["amb_tiles"] = amb_tiles.reshape(-1)
    return st


def fp32_sensitivity(st: ViewState, cam: Camera, s: Surfels, bg, variant=PLAIN, trials=2, seed=0):
    """Per pixel, how far the FP64 blend moves when every surfel's
    splat-to-pixel matrix and screen centre are rounded by one FP32 unit
    (relative 2^-23, random signs, ``trials`` draws): [3+others, H, W] of
    |change| relative to max(1, |value|).  Every FP32 implementation stores
    those quantities rounded, so where this exceeds a tolerance the
    algorithm itself is too ill-conditioned in FP32 (nearly edge-on splats,
    long transmittance products) for two FP32 evaluations to agree to it."""
    pre = st.extra["pre"]
    rng = np.random.default_rng(seed)
    base = np.concatenate([st.color, st.others])
    worst = np.zeros_like(base)
    for _ in range(trials):
        p2 = dict(pre)
        p2["transmat"] = pre["transmat"] * (1.0 + rng.choice([-1.0, 1.0], pre["transmat"].shape) * 2.0 ** -23)
        p2["means2D"] = pre["means2D"] * (1.0 + rng.choice([-1.0, 1.0], pre["means2D"].shape) * 2.0 ** -23)
        rf = render_forward(p2, st.point_list, st.ranges, cam, s, bg, variant, np.float64)
        out = np.concatenate([rf["color"], rf["others"]])
        worst = np.maximum(worst, np.abs(out - base) / np.maximum(1.0, np.abs(base)))
    return worst


# --------------------------------------------------------------------------
# backward
# --------------------------------------------------------------------------
def render_backward(st: ViewState, cam: Camera, s: Surfels, bg, dL_dcolor, dL_dothers, dL_dsem=None,
                    variant=PLAIN, dtype=np.float64, tiles=None):
    """Blend backward, P0/cr/backward.cu:143-440 / P1/cr/backward.cu:143-470.
    Returns per-surfel accumulators (dL_dtransmat, dL_dmean2D, dL_dnormal,
    dL_dopacity, dL_dcolor, dL_dsemantics)."""
    f = _f(dtype)
    pre = st.extra["pre"]
    gx, gy = pre["grid"]
    W, H = cam.width, cam.height
    P = s.P
    X, Y, pxf, pyf, inside = _tile_pixels(gx, gy, W, H, variant, f, tiles)
    lists, lens, L = _padded_lists(st.point_list, st.ranges, tiles)
    nt = lists.shape[0]
    tm, xy2, no, rgb = st.transmat, st.means2D, st.normal_opacity, st.rgb
    bg = np.asarray(bg, dtype=dtype)
    Sn = 0 if s.semantics is None else s.semantics.shape[1]
    sem_all = None if s.semantics is None else s.semantics.astype(dtype)

    g = lambda img: _gather_pixels(img.astype(dtype), X, Y, inside)  # noqa: E731
    T_final = g(st.final_T[0])
    final_D = g(st.final_T[1])
    final_D2 = g(st.final_T[2])
    final_A = 1 - T_final
    last_contrib = _gather_pixels(st.n_contrib[0], X, Y, inside)
    med_contrib = _gather_pixels(st.n_contrib[1], X, Y, inside)
    dpix = np.stack([g(dL_dcolor[c]) for c in range(3)], -1)
    dL_ddepth = g(dL_dothers[0])
    dL_daccum = g(dL_dothers[1])
    dL_dnormal2D = np.stack([g(dL_dothers[2 + c]) for c in range(3)], -1)
    dL_dmedian = g(dL_dothers[5])
    dL_dreg = g(dL_dothers[6])
    dL_dmaxw = g(dL_dothers[7]) if variant == PART else None
    dpix_sem = np.stack([g(dL_dsem[c]) for c in range(Sn)], -1) if Sn else None
    bg_dot = np.sum(bg[None, None, :] * dpix, -1)

    shape = (nt, BLOCK_SIZE)
    T = T_final.copy()
    accum_rec = np.zeros(shape + (3,), dtype)
    last_color = np.zeros(shape + (3,), dtype)
    accum_sem = np.zeros(shape + (Sn,), dtype)
    last_sem = np.zeros(shape + (Sn,), dtype)
    last_alpha = np.zeros(shape, dtype)
    last_depth = np.zeros(shape, dtype)
    last_normal = np.zeros(shape + (3,), dtype)
    accum_depth = np.zeros(shape, dtype)
    accum_alpha = np.zeros(shape, dtype)
    accum_normal = np.zeros(shape + (3,), dtype)
    last_dL_dT = np.zeros(shape, dtype)

    gT = np.zeros((P, 9), dtype)
    gm2 = np.zeros((P, 2), dtype)
    gn = np.zeros((P, 3), dtype)
    go = np.zeros(P, dtype)
    gc = np.zeros((P, 3), dtype)
    gs = np.zeros((P, Sn), dtype)

    def acc(target, ids, vals, mask):
        m = mask.reshape(-1)
        np.add.at(target, ids.reshape(-1)[m], vals.reshape((-1,) + vals.shape[2:])[m])

    for j in range(L - 1, -1, -1):
        ids = lists[:, j]
        act = (ids >= 0)[:, None] & inside & (j < last_contrib)
        if not act.any():
            continue
        idc = np.where(ids >= 0, ids, 0)
        idb = np.broadcast_to(idc[:, None], shape)
        Tu = tm[idc, 0:3][:, None, :]
        Tv = tm[idc, 3:6][:, None, :]
        Tw = tm[idc, 6:9][:, None, :]
        xy = xy2[idc][:, None, :]
        k, l, pv, sx, sy, rho3d, rho2d, rho, c_d, use3d, dx, dy = _intersect(variant, f, pxf, pyf, Tu, Tv, Tw, xy)
        ok = act & (pv[2] != 0)
        ok &= ~(c_d < NEAR_N) if variant == PART else ~(c_d < f(np.float32(NEAR_N)))
        power = f(-0.5) * rho
        ok &= ~(power > 0)
        opa = no[idc, 3][:, None]
        with np.errstate(over="ignore", invalid="ignore", divide="ignore"):
            G = np.exp(power)
            alpha = np.minimum(f(0.99), opa * G)
        ok &= ~(alpha < f(1.0) / f(255.0))
        if not ok.any():
            continue
        with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
            Tn = T / (1.0 - alpha)
        T = np.where(ok, Tn, T)
        wgt = alpha * T
        dL_dalpha = np.zeros(shape, dtype)
        col = rgb[idc][:, None, :]
        new_acc = last_alpha[..., None] * last_color + (1.0 - last_alpha[..., None]) * accum_rec
        accum_rec = np.where(ok[..., None], new_acc, accum_rec)
        last_color = np.where(ok[..., None], col, last_color)
        dL_dalpha = dL_dalpha + np.sum((col - accum_rec) * dpix, -1)
        acc(gc, idb, wgt[..., None] * dpix, ok)
        if Sn:
            sv = sem_all[idc][:, None, :]
            new_s = last_alpha[..., None] * last_sem + (1.0 - last_alpha[..., None]) * accum_sem
            accum_sem = np.where(ok[..., None], new_s, accum_sem)
            last_sem = np.where(ok[..., None], sv, last_sem)
            acc(gs, idb, wgt[..., None] * dpix_sem, ok)
        dL_dz = np.zeros(shape, dtype)
        dL_dweight = np.zeros(shape, dtype)
        with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
            if variant == PLAIN:
                m_d = f(FAR_N) / (f(FAR_N) - f(NEAR_N)) * (1 - f(NEAR_N) / c_d)
                dmd_dd = (f(FAR_N) * f(NEAR_N)) / ((f(FAR_N) - f(NEAR_N)) * c_d * c_d)
            else:
                cd64 = c_d.astype(np.float64)
                m_d = ((100.0 * cd64 - 100.0 * 0.2) / ((100.0 - 0.2) * cd64)).astype(dtype)
                dmd_dd = ((100.0 * 0.2) / ((100.0 - 0.2) * cd64 * cd64)).astype(dtype)
        is_med = (j == med_contrib - 1)
        dL_dz = dL_dz + np.where(is_med, dL_dmedian, 0)
        if variant == PART:
            dL_dweight = dL_dweight + np.where(is_med, dL_dmaxw, 0)
        dL_dweight = dL_dweight + (final_D2 + m_d * m_d * final_A - 2 * m_d * final_D) * dL_dreg
        dL_dalpha = dL_dalpha + dL_dweight - last_dL_dT
        last_dL_dT = np.where(ok, dL_dweight * alpha + (1 - alpha) * last_dL_dT, last_dL_dT)
        dL_dmd = 2.0 * (T * alpha) * (m_d * final_A - final_D) * dL_dreg
        dL_dz = dL_dz + dL_dmd * dmd_dd
        new_ad = last_alpha * last_depth + (1 - last_alpha) * accum_depth
        accum_depth = np.where(ok, new_ad, accum_depth)
        last_depth = np.where(ok, c_d, last_depth)
        dL_dalpha = dL_dalpha + (c_d - accum_depth) * dL_ddepth
        new_aa = last_alpha * 1.0 + (1 - last_alpha) * accum_alpha
        accum_alpha = np.where(ok, new_aa, accum_alpha)
        dL_dalpha = dL_dalpha + (1 - accum_alpha) * dL_daccum
        nrm = no[idc, 0:3][:, None, :]
        new_an = last_alpha[..., None] * last_normal + (1 - last_alpha[..., None]) * accum_normal
        accum_normal = np.where(ok[..., None], new_an, accum_normal)
        last_normal = np.where(ok[..., None], nrm, last_normal)
        dL_dalpha = dL_dalpha + np.sum((nrm - accum_normal) * dL_dnormal2D, -1)
        acc(gn, idb, (alpha * T)[..., None] * dL_dnormal2D, ok)
        dL_dalpha = dL_dalpha * T
        last_alpha = np.where(ok, alpha, last_alpha)
        with np.errstate(divide="ignore", invalid="ignore"):
            dL_dalpha = dL_dalpha + (-T_final / (1.0 - alpha)) * bg_dot
        dL_dG = opa * dL_dalpha
        dL_dz = dL_dz + alpha * T * dL_ddepth
        m3 = ok & use3d
        m2 = ok & ~use3d
        if m3.any():
            with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
                dsx = dL_dG * -G * sx + dL_dz * Tw[..., 0]
                dsy = dL_dG * -G * sy + dL_dz * Tw[..., 1]
                dsx_pz = dsx / pv[2]
                dsy_pz = dsy / pv[2]
            dp = [dsx_pz, dsy_pz, -(dsx_pz * sx + dsy_pz * sy)]
            dk = [l[1] * dp[2] - l[2] * dp[1], l[2] * dp[0] - l[0] * dp[2], l[0] * dp[1] - l[1] * dp[0]]
            dl = [dp[1] * k[2] - dp[2] * k[1], dp[2] * k[0] - dp[0] * k[2], dp[0] * k[1] - dp[1] * k[0]]
            dz_dTw = [sx, sy, np.ones_like(sx)]
            vals = np.stack([-dk[0], -dk[1], -dk[2], -dl[0], -dl[1], -dl[2]]
                            + [pxf * dk[i] + pyf * dl[i] + dL_dz * dz_dTw[i] for i in range(3)], -1)
            acc(gT, idb, vals, m3)
        if m2.any():
            if variant == PLAIN:
                dG_ddelx = -G * f(FILTER_INV_SQUARE_P0) * dx
                dG_ddely = -G * f(FILTER_INV_SQUARE_P0) * dy
            else:
                dG_ddelx = ((-G).astype(np.float64) * FILTER_INV_SQUARE_P1 * dx).astype(dtype)
                dG_ddely = ((-G).astype(np.float64) * FILTER_INV_SQUARE_P1 * dy).astype(dtype)
            acc(gm2, idb, np.stack([dL_dG * dG_ddelx, dL_dG * dG_ddely], -1), m2)
            v8 = np.zeros(shape + (9,), dtype)
            v8[..., 8] = dL_dz
            acc(gT, idb, v8, m2)
        acc(go, idb, G * dL_dalpha, ok)
    return dict(dL_dtransmat=gT, dL_dmean2D=gm2, dL_dnormal=gn, dL_dopacity=go, dL_dcolor=gc,
                dL_dsemantics=gs)


def preprocess_backward(st: ViewState, rb: dict, cam: Camera, s: Surfels, variant=PLAIN, dtype=np.float64):
    """P0/cr/backward.cu:443-630 and P1/cr/backward.cu:473-671.
    Returns the per-surfel gradients the reference's binding returns."""
    f = _f(dtype)
    P = s.P
    W, H = cam.width, cam.height
    vm = cam.viewmatrix.astype(dtype)
    Vm = vm.reshape(4, 4)
    F = cam.projmatrix.astype(dtype).reshape(4, 4)
    fx = focal(W, cam.tanfovx, dtype)
    fy = focal(H, cam.tanfovy, dtype)
    vis = st.radii > 0
    p = s.means3D.astype(dtype)
    gT = rb["dL_dtransmat"].copy()
    gm2 = rb["dL_dmean2D"]
    gn = rb["dL_dnormal"]
    dmean3D = np.zeros((P, 3), dtype)
    dscale = np.zeros((P, 2), dtype)
    drot = np.zeros((P, 4), dtype)
    dsh = None if s.shs is None else np.zeros_like(s.shs, dtype=dtype)
    dmean2D_out = np.zeros((P, 3), dtype)
    precomp = s.transmat_precomp is not None
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        if variant == PLAIN:
            # W and H recovered from focal * tan * 2 with truncation
            # (P0/cr/backward.cu:607-608)
            if np.dtype(dtype) == np.float32:
                Wb = int(np.float32(np.float32(fx) * np.float32(cam.tanfovx)) * np.float32(2))
                Hb = int(np.float32(np.float32(fy) * np.float32(cam.tanfovy)) * np.float32(2))
            else:
                Wb = int(fx * cam.tanfovx * 2)
                Hb = int(fy * cam.tanfovy * 2)
            if precomp:
                T9 = s.transmat_precomp.astype(dtype)
                nrm = np.zeros((P, 3), dtype)
            else:
                R = quat_to_rotmat(s.rotations.astype(dtype))
                sc = s.scales.astype(dtype)
                L0 = R[:, :, 0] * sc[:, 0:1]
                L1 = R[:, :, 1] * sc[:, 1:2]
                L2 = R[:, :, 2]
                Nmat = np.array([[Wb / 2.0, 0.0, 0.0], [0.0, Hb / 2.0, 0.0], [0.0, 0.0, 0.0],
                                 [(Wb - 1) / 2.0, (Hb - 1) / 2.0, 1.0]], dtype=dtype)
                Pm = F @ Nmat                                          # [4,3]
                T3 = np.stack([L0 @ Pm[:3], L1 @ Pm[:3], p @ Pm[:3] + Pm[3]], 1)  # rows (L0,L1,p) x cols
                # glm columns: Tu = T3[:, :, 0] etc.
                T9 = np.concatenate([T3[:, :, 0], T3[:, :, 1], T3[:, :, 2]], 1)
                nrm = L2 @ Vm[:3, :3]
            dT = gT.copy()
            has_m2 = (gm2[:, 0] != 0) | (gm2[:, 1] != 0)
            T0, T1, T2 = T9[:, 0:3], T9[:, 3:6], T9[:, 6:9]
            tv = np.array([9.0, 9.0, -1.0], dtype=dtype)
            d = np.sum(tv * T2 * T2, 1)
            fvec = tv * (1.0 / d)[:, None]
            mx, my = gm2[:, 0:1], gm2[:, 1:2]
            dT0 = mx * fvec * T2
            dT1 = my * fvec * T2
            dT3 = mx * fvec * T0 + my * fvec * T1
            dL_df = mx * T0 * T2 + my * T1 * T2
            dL_dd = (np.sum(dL_df * fvec, 1).astype(np.float64) * (-1.0 / d.astype(np.float64))).astype(dtype)
            dT3 = dT3 + dL_dd[:, None] * (tv * T2 * 2.0)
            upd = np.concatenate([dT0, dT1, dT3], 1)
            dT = np.where(has_m2[:, None], dT + upd, dT)
            if precomp:
                gT = np.where((has_m2 & vis)[:, None], dT, gT)
            else:
                # dL_dM = P * transpose(dL_dT): column i = sum_j P[:, j] * G[i][j]
                G = np.stack([dT[:, 0:3], dT[:, 3:6], dT[:, 6:9]], 2)    # G[:, i, j] = d/dT_math[i][j]
                dM = np.einsum("rj,pij->pri", Pm, G)                      # [P,4,3]
                dtn = gn @ Vm[:3, :3].T
                pview = p @ Vm[:3, :3] + Vm[3, :3]
                cosv = -np.sum(pview * nrm, 1)
                dtn = dtn * np.where(cosv > 0, 1.0, -1.0).astype(dtype)[:, None]
                dR = np.stack([dM[:, :3, 0] * sc[:, 0:1], dM[:, :3, 1] * sc[:, 1:2], dtn], 2)
                drot = quat_to_rotmat_vjp(s.rotations.astype(dtype), dR)
                dscale = np.stack([np.sum(dM[:, :3, 0] * R[:, :, 0], 1), np.sum(dM[:, :3, 1] * R[:, :, 1], 1)], 1)
                dmean3D = dM[:, :3, 2].copy()
        else:
            T9 = st.transmat
            T0, T1, T3 = T9[:, 0:3], T9[:, 3:6], T9[:, 6:9]
            tv = np.array([1.0, 1.0, -1.0], dtype=dtype)
            d = np.sum(tv * T3 * T3, 1)
            fvec = tv * (1.0 / d)[:, None]
            mx, my = gm2[:, 0:1], gm2[:, 1:2]
            dT0 = mx * fvec * T3
            dT1 = my * fvec * T3
            dT3 = mx * fvec * T0 + my * fvec * T1
            dL_df = (mx * T0 * T3) + (my * T1 * T3)
            dL_dd = (np.sum(dL_df * fvec, 1).astype(np.float64) * (-1.0 / d.astype(np.float64))).astype(dtype)
            dT3 = dT3 + dL_dd[:, None] * (tv * T3 * 2.0)
            gT = np.where(vis[:, None], gT + np.concatenate([dT0, dT1, dT3], 1), gT)
            if not precomp:
                R = quat_to_rotmat(s.rotations.astype(dtype))
                sc = s.scales.astype(dtype)
                cxb, cyb = fx * f(cam.tanfovx), fy * f(cam.tanfovy)
                W3 = Vm[:3, :3].T
                # dL_dM_aug = P^T G4 with G4 rows (dTu, dTv, dTw, 0); keep the top 3 rows
                dTu, dTv, dTw = gT[:, 0:3], gT[:, 3:6], gT[:, 6:9]
                dM = np.stack([fx * dTu, fy * dTv, cxb * dTu + cyb * dTv + dTw], 1)   # [P, row, col]
                dRS = np.einsum("rk,pkc->prc", W3.T, dM)                              # W^T dM
                dRS0, dRS1, dpw = dRS[:, :, 0], dRS[:, :, 1], dRS[:, :, 2]
                dtn = gn @ W3                                                          # W^T n as row vec
                tn = R[:, :, 2] @ W3.T
                pv = p @ W3.T + Vm[3, :3]
                cosv = np.sum(-tn * pv, 1)
                dtn = dtn * np.where(cosv > 0, 1.0, -1.0).astype(dtype)[:, None]
                dR = np.stack([dRS0 * sc[:, 0:1], dRS1 * sc[:, 1:2], dtn], 2)
                drot = quat_to_rotmat_vjp(s.rotations.astype(dtype), dR)
                dscale = np.stack([np.sum(dRS0 * R[:, :, 0], 1), np.sum(dRS1 * R[:, :, 1], 1)], 1)
                dmean3D = dpw.copy()
        if s.shs is not None:
            rgb_, clamped, dir_orig = sh_to_rgb(s.sh_degree, s.shs.astype(dtype), p, cam.campos.astype(dtype))
            dsh_v, dmean_sh = sh_backward(s.sh_degree, s.shs.astype(dtype), dir_orig, st.clamped, rb["dL_dcolor"])
            dsh = np.where(vis[:, None, None], dsh_v, 0)
            dmean3D = dmean3D + dmean_sh
        if variant == PLAIN:
            depth = st.transmat[:, 8]
            dmean2D_out[:, 0] = (gT[:, 2] * depth).astype(np.float64) * 0.5 * float(Wb)
            dmean2D_out[:, 1] = (gT[:, 5] * depth).astype(np.float64) * 0.5 * float(Hb)
        else:
            z = st.transmat[:, 8]
            Wf = f(fx) * f(cam.tanfovx)
            Hf = f(fy) * f(cam.tanfovy)
            dmean2D_out[:, 0] = gT[:, 2] * z * Wf
            dmean2D_out[:, 1] = gT[:, 5] * z * Hf
    z3 = lambda a: np.where(vis.reshape((-1,) + (1,) * (a.ndim - 1)), a, 0)  # noqa: E731
    out = dict(
        dL_dmeans2D=z3(dmean2D_out),
        dL_dcolors=rb["dL_dcolor"],
        dL_dopacity=rb["dL_dopacity"][:, None],
        dL_dmeans3D=z3(dmean3D),
        dL_dtransmat=gT,
        dL_dsh=dsh,
        dL_dscales=z3(dscale),
        dL_drotations=z3(drot),
    )
    if variant == PART:
        out["dL_dsemantics"] = rb["dL_dsemantics"]
    return out


def backward_view(st, cam, s, bg, dL_dcolor, dL_dothers, dL_dsem=None, variant=PLAIN, dtype=np.float64,
                  tiles=None):
    rb = render_backward(st, cam, s, bg, dL_dcolor, dL_dothers, dL_dsem, variant, dtype, tiles)
    return preprocess_backward(st, rb, cam, s, variant, dtype)


def mark_visible(means3D, viewmatrix):
    """checkFrustum, P0/cr/rasterizer_impl.cu:54-66."""
    Vm = np.asarray(viewmatrix, dtype=np.float64).reshape(4, 4)
    pv = np.asarray(means3D, dtype=np.float64) @ Vm[:3, :3] + Vm[3, :3]
    return pv[:, 2] > 0.2
