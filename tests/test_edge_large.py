"""Shapes the small parity cases do not reach: a surfel that covers the whole
image over many small ones (every tile's list holds it; unbounded reach
boxes), a wide 640x384 image (a 40 x 24 tile grid, 5 x 3 cells), and 40
views in one batch (more depth-key view bits), against the oracle or the
one-view path."""
import numpy as np
import pytest
import torch

from oracle import surfel_oracle as O
from tests._util import grad_error, image_error, oracle_camera, oracle_surfels, settings

pytestmark = pytest.mark.gpu

IMG_TOL = 1e-5
AUX_TOL = 3e-5
# Relative margin of the alpha cutoff (1/255) and the stop test within which
# a pixel's outcome may go either way in FP32: near the cutoff, alpha carries
# up to ~2e-5 relative error from the cancelling cross product of the splat
# intersection (seen: a fragment 1.8e-5 above 1/255 in FP64), and these
# larger images hold such fragments.
ALPHA_TOL = 1e-4


def _render(scene, cam):
    from partgs_gb300 import _lib as L
    from partgs_gb300 import raster
    sc = scene.to("cuda")
    rs = settings(__import__("partgs_gb300.diff_surfel_rasterization", fromlist=["x"]), cam, [0.0, 0.0, 0.0])
    vs = raster.ViewSet(rs.viewmatrix.reshape(1, 16), rs.projmatrix.reshape(1, 16), rs.campos.reshape(1, 3),
                        [(cam.tanfovx, cam.tanfovy)], cam.height, cam.width)
    color, others, _, radii, state = raster.forward(L.SGR_VARIANT_PLAIN, sc.means3D, sc.opacities, sc.shs, None,
                                                    sc.scales, sc.rotations, None, None, vs, rs.bg, 3)
    return color[0], others[0], radii, state


def _check_against_oracle(scene, cam, grads=True):
    from partgs_gb300 import raster
    color, others, radii, state = _render(scene, cam)
    ocam, osf = oracle_camera(cam), oracle_surfels(scene)
    st64 = O.forward_view(osf, ocam, np.zeros(3), O.PLAIN, np.float64, alpha_tol=ALPHA_TOL)
    st32 = O.forward_view(osf, ocam, np.zeros(3), O.PLAIN, np.float32, alpha_tol=ALPHA_TOL)
    amb = st64.amb_pixel | st32.amb_pixel
    assert amb.mean() < 0.03
    # the bars, or twice the FP32 oracle's own error where it is larger: with
    # up to ~140 fragments per pixel FP32 blending drifts past 1e-5
    col_tol = max(IMG_TOL, 2 * max(image_error(st32.color, st64.color, amb)))
    oth_tol = max(AUX_TOL, 2 * max(image_error(st32.others, st64.others, amb)))
    assert max(image_error(color.cpu().numpy(), st64.color, amb)) <= col_tol
    assert max(image_error(others.cpu().numpy(), st64.others, amb)) <= oth_tol
    nc = raster.debug_state(state)["n_contrib"][0].cpu().numpy()
    np.testing.assert_array_equal(nc[0][~amb], st64.n_contrib[0][~amb])
    if grads:
        g = np.random.default_rng(3)
        dcol = g.standard_normal((3, cam.height, cam.width)).astype(np.float32)
        doth = g.standard_normal((7, cam.height, cam.width)).astype(np.float32)
        dcol[:, amb] = 0
        doth[:, amb] = 0
        mine = raster.backward(state, torch.from_numpy(dcol)[None].cuda(), torch.from_numpy(doth)[None].cuda())
        ref = O.backward_view(st64, ocam, osf, np.zeros(3), dcol, doth, variant=O.PLAIN, dtype=np.float64)
        ref32 = O.backward_view(st32, ocam, osf, np.zeros(3), dcol, doth, variant=O.PLAIN, dtype=np.float32)
        for k in ("dL_dcolors", "dL_dopacity", "dL_dmeans3D", "dL_dscales", "dL_drotations"):
            # 1e-4, or four times the FP32 oracle's own error where the
            # gradient sums many cancelling pixel terms: a large surfel's
            # transMat Tw row weights its adjoints by pixel coordinates (seen:
            # 1.4e-4 in FP32 numpy for one surfel's mean; the warp reductions
            # and atomics add in yet another order)
            floor = grad_error(ref32[k], ref[k])
            assert grad_error(mine[k].cpu().numpy(), ref[k]) <= max(1e-4, 4 * floor), (k, floor)


def test_screen_covering_surfel_over_small_ones(sgr_lib):
    from partgs_gb300.cameras import orbit_cameras
    from partgs_gb300.scenes import random_surfels
    scene = random_surfels(600, seed=41)
    cam = orbit_cameras(1, 3.0, 96, 128, 60.0, seed=2)[0]
    d = torch.as_tensor(cam.camera_center, dtype=torch.float32)
    d = d / d.norm()
    # one large, half-transparent surfel behind the others, its normal (the
    # rotation's z axis) turned towards the camera: q rotates z onto d
    q = torch.tensor([1.0 + float(d[2]), -float(d[1]), float(d[0]), 0.0])
    scene.rotations[0] = q / q.norm()
    scene.means3D[0] = -0.6 * d
    scene.scales[0] = torch.tensor([4.0, 4.0])
    scene.opacities[0] = 0.5
    _check_against_oracle(scene, cam)


def test_wide_image(sgr_lib):
    from partgs_gb300.cameras import orbit_cameras
    from partgs_gb300.scenes import random_surfels
    scene = random_surfels(2000, seed=43)
    cam = orbit_cameras(1, 3.0, 384, 640, 60.0, seed=5)[0]
    _check_against_oracle(scene, cam, grads=False)


def test_forty_views_equal_one_view_renders(sgr_lib):
    import partgs_gb300.diff_surfel_rasterization as dsr
    from partgs_gb300.batched import MultiViewRasterizer
    from partgs_gb300.cameras import orbit_cameras
    from partgs_gb300.scenes import random_surfels
    scene = random_surfels(1500, seed=47).to("cuda")
    cams = orbit_cameras(40, 3.0, 48, 64, 55.0, seed=6)
    img, amap, _, _ = MultiViewRasterizer(cams, [0, 0, 0], 3, num_surfels=1500)(
        scene.means3D, scene.opacities, scene.shs, scene.scales, scene.rotations)
    for v in (0, 17, 39):
        rs = settings(dsr, cams[v], [0, 0, 0])
        i1, _, a1 = dsr.GaussianRasterizer(rs)(means3D=scene.means3D, means2D=torch.zeros_like(scene.means3D),
                                               opacities=scene.opacities, shs=scene.shs, scales=scene.scales,
                                               rotations=scene.rotations)
        assert torch.equal(img[v], i1) and torch.equal(amap[v], a1), v
