"""The blend kernels' row test (sgr_blend.cu, row_reaches) is conservative:
it never rejects a (record, strip) pair in which the kernels' own per-pixel
reach test -- p.z != 0 and (rho2d <= c or |p.xy|^2 <= c p.z^2), in fp32 as
the blends compute it -- accepts some pixel.  The row test is restated here
operation for operation in numpy fp32 and checked on every (record, strip)
pair of scenes preprocessed by the oracle, including strongly tilted
surfels (grazing views) and very large ones."""
import numpy as np
import pytest

from oracle import surfel_oracle as O

f32 = np.float32


def _cross(a, b):
    return np.stack([a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1], a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2],
                     a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]], -1)


def row_reaches(Tu, Tv, Tw, cx, cy, c, y, xa, xb):
    """numpy restatement of row_reaches (fp32, vectorised over records)."""
    cc = (c * f32(1.01)).astype(f32)
    dy = (cy - y).astype(f32)
    h2 = (f32(0.5) * cc - dy * dy).astype(f32)
    with np.errstate(invalid="ignore"):
        h = np.sqrt(np.maximum(h2, 0)).astype(f32)
    disk = (h2 >= 0) & (cx + h >= xa - f32(0.5)) & (cx - h <= xb + f32(0.5))
    l = (y[..., None] * Tw - Tv).astype(f32)
    A = _cross(Tw, l).astype(f32)
    B = _cross((xa * Tw - Tu).astype(f32), l).astype(f32)
    a = (A[..., 0] * A[..., 0] + A[..., 1] * A[..., 1] - cc * (A[..., 2] * A[..., 2])).astype(f32)
    bh = (A[..., 0] * B[..., 0] + A[..., 1] * B[..., 1] - cc * (A[..., 2] * B[..., 2])).astype(f32)
    e = (B[..., 0] * B[..., 0] + B[..., 1] * B[..., 1] - cc * (B[..., 2] * B[..., 2])).astype(f32)
    bad = ~(np.isfinite(a) & np.isfinite(bh) & np.isfinite(e))
    ua, ub = f32(-0.5), f32(xb - xa + 0.5)
    ends = ((a * ua + 2 * bh) * ua + e <= 0) | ((a * ub + 2 * bh) * ub + e <= 0)
    with np.errstate(all="ignore"):
        us = -bh / a
        inner = (a > 0) & (us > ua) & (us < ub) & (e - bh * (bh / a) <= 0)
    return disk | bad | ends | inner


def _scene(seed, tilt, scale):
    from partgs_gb300.cameras import orbit_cameras
    from partgs_gb300.scenes import random_surfels
    sc = random_surfels(2500, seed=seed)
    scales = sc.scales.numpy() * scale
    if tilt:   # flatten one axis hard: edge-on views of thin surfels
        scales[:, 1] *= 0.02
    cam = orbit_cameras(1, 3.0, 96, 128, 60.0, seed=seed)[0]
    ocam = O.Camera(cam.world_view_transform.reshape(-1), cam.full_proj_transform.reshape(-1), cam.camera_center,
                    cam.tanfovx, cam.tanfovy, cam.height, cam.width)
    osf = O.Surfels(sc.means3D.numpy(), sc.opacities.numpy(), scales, sc.rotations.numpy(), shs=sc.shs.numpy(),
                    sh_degree=3)
    return O.preprocess(osf, ocam, O.PLAIN, np.float32), ocam


@pytest.mark.parametrize("seed,tilt,scale", [(1, False, 1.0), (2, True, 1.0), (3, False, 8.0), (4, True, 4.0)])
def test_row_test_never_rejects_a_reaching_strip(seed, tilt, scale):
    pre, cam = _scene(seed, tilt, scale)
    keep = np.nonzero(pre["radii"] > 0)[0]
    Tm = pre["transmat"][keep].astype(f32)
    Tu, Tv, Tw = Tm[:, 0:3], Tm[:, 3:6], Tm[:, 6:9]
    xy = pre["means2D"][keep].astype(f32)
    op = pre["normal_opacity"][keep, 3].astype(f32)
    c = (2 * np.log(255 * op) * 1.001 + 0.01).astype(f32)   # a reach threshold of the kernels' form
    gx, gy = (cam.width + 15) // 16, (cam.height + 15) // 16
    checked = rejected = 0
    for ty in range(gy):
        for tx in range(gx):
            x0 = f32(16 * tx)
            px = x0 + np.arange(16, dtype=f32)
            for strip in range(8):                       # the forward's 16 x 2 strips
                ys = f32(16 * ty + 2 * strip) + np.arange(2, dtype=f32)
                # the kernels' per-pixel test on the strip's 32 pixels
                k = px[None, :, None] * Tw[:, None, :] - Tu[:, None, :]            # [n, 16, 3]
                hit = np.zeros(len(keep), bool)
                ok = np.zeros(len(keep), bool)
                for y in ys:
                    l = (y * Tw - Tv)[:, None, :]
                    p = _cross(k, np.broadcast_to(l, k.shape)).astype(f32)
                    dx, dy = xy[:, 0:1] - px[None], xy[:, 1:2] - y
                    rho2d = f32(2.0) * (dx * dx + dy * dy)
                    within = (p[..., 2] != 0) & ~((rho2d > c[:, None]) &
                                                  (p[..., 0] ** 2 + p[..., 1] ** 2 > c[:, None] * p[..., 2] ** 2))
                    hit |= within.any(1)
                    ok |= row_reaches(Tu, Tv, Tw, xy[:, 0], xy[:, 1], c, np.full(len(keep), y, f32), x0,
                                      f32(x0 + 15))
                assert not (hit & ~ok).any(), (tx, ty, strip, np.nonzero(hit & ~ok)[0][:5])
                checked += len(keep)
                rejected += int((~ok).sum())
    assert checked > 0 and rejected > 0.5 * checked          # it does reject most pairs of a tile
