"""Pinhole cameras in the reference's matrix conventions.

The rasteriser consumes the matrices PartGS's ``Camera`` builds
(``scene/cameras.py:54-63``): a world-to-view transform and a full projection,
both stored *transposed* (row-vector convention, i.e. glm column-major when
read as flat arrays), plus the camera centre.  ``world_to_view`` restates
``utils/graphics_utils.py:29-40`` (getWorld2View2) and ``projection`` restates
``utils/graphics_utils.py:42-62`` (getProjectionMatrix).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

ZNEAR = 0.01   # scene/cameras.py:54-55
ZFAR = 100.0


def world_to_view(R: np.ndarray, t: np.ndarray) -> np.ndarray:
    """4x4 world-to-view matrix (column-vector form); R is the camera-to-world
    rotation, t the world-to-view translation (utils/graphics_utils.py:29-40
    with translate 0 and scale 1)."""
    Rt = np.zeros((4, 4))
    Rt[:3, :3] = R.T
    Rt[:3, 3] = t
    Rt[3, 3] = 1.0
    C2W = np.linalg.inv(Rt)
    Rt = np.linalg.inv(C2W)
    return np.float32(Rt)


def projection(znear: float, zfar: float, fovx: float, fovy: float) -> np.ndarray:
    """4x4 perspective projection, utils/graphics_utils.py:42-62."""
    tan_y = math.tan(fovy / 2)
    tan_x = math.tan(fovx / 2)
    top = tan_y * znear
    bottom = -top
    right = tan_x * znear
    left = -right
    P = np.zeros((4, 4), dtype=np.float32)
    P[0, 0] = 2.0 * znear / (right - left)
    P[1, 1] = 2.0 * znear / (top - bottom)
    P[0, 2] = (right + left) / (right - left)
    P[1, 2] = (top + bottom) / (top - bottom)
    P[3, 2] = 1.0
    P[2, 2] = zfar / (zfar - znear)
    P[2, 3] = -(zfar * znear) / (zfar - znear)
    return P


@dataclass
class PinholeCamera:
    """The fields ``GaussianRasterizationSettings`` takes from a camera."""
    height: int
    width: int
    fovx: float
    fovy: float
    world_view_transform: np.ndarray   # [4,4] float32, transposed (row-vector)
    full_proj_transform: np.ndarray    # [4,4] float32, transposed
    camera_center: np.ndarray          # [3] float32

    @property
    def tanfovx(self) -> float:
        return math.tan(self.fovx * 0.5)

    @property
    def tanfovy(self) -> float:
        return math.tan(self.fovy * 0.5)


def make_camera(R: np.ndarray, t: np.ndarray, fovx: float, fovy: float, height: int, width: int) -> PinholeCamera:
    """Same construction as scene/cameras.py:58-63: transposed world-to-view,
    transposed projection, their product, and the centre taken from the inverse."""
    wv = world_to_view(R, t).T.astype(np.float32)
    pj = projection(ZNEAR, ZFAR, fovx, fovy).T.astype(np.float32)
    full = (wv.astype(np.float32) @ pj.astype(np.float32)).astype(np.float32)
    center = np.linalg.inv(wv.astype(np.float64))[3, :3].astype(np.float32)
    return PinholeCamera(height, width, fovx, fovy, wv, full, center)


def look_at(center: np.ndarray, target=(0.0, 0.0, 0.0), up=(0.0, 0.0, 1.0)):
    """Camera-to-world rotation and world-to-view translation of a camera at
    ``center`` looking at ``target`` (x right, y down, z forward)."""
    c = np.asarray(center, dtype=np.float64)
    fwd = np.asarray(target, dtype=np.float64) - c
    fwd /= np.linalg.norm(fwd)
    upv = np.asarray(up, dtype=np.float64)
    if abs(np.dot(fwd, upv)) > 0.999:
        upv = np.array([0.0, 1.0, 0.0])
    right = np.cross(fwd, upv)
    right /= np.linalg.norm(right)
    down = np.cross(fwd, right)
    C2W = np.stack([right, down, fwd], axis=1)
    t = -C2W.T @ c
    return C2W, t


def fovy_from_fovx(fovx: float, width: int, height: int) -> float:
    return 2.0 * math.atan(math.tan(fovx / 2.0) * height / width)


def orbit_cameras(n: int, radius: float, height: int, width: int, fovx_deg: float, seed: int = 0):
    """``n`` cameras on a sphere of ``radius`` looking at the origin; the
    directions are seeded and spread with a Fibonacci lattice."""
    rng = np.random.default_rng(seed)
    fovx = math.radians(fovx_deg)
    fovy = fovy_from_fovx(fovx, width, height)
    phase = rng.uniform(0, 2 * math.pi)
    cams = []
    for i in range(n):
        z = 1.0 - 2.0 * (i + 0.5) / n
        r = math.sqrt(max(0.0, 1.0 - z * z))
        phi = phase + i * math.pi * (3.0 - math.sqrt(5.0))
        d = np.array([r * math.cos(phi), r * math.sin(phi), 0.8 * z])
        d /= np.linalg.norm(d)
        R, t = look_at(radius * d)
        cams.append(make_camera(R, t, fovx, fovy, height, width))
    return cams
