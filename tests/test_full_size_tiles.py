"""Parity at the bench workload's full size: view 0 of the 500k-surfel scene
at 800x600, rendered on the GPU, against the FP64 oracle on a seeded sample
of its tiles.  Images, contributor counts and median indices on the sampled
tiles, the radii of every surfel, and the gradients of every surfel when the
upstream gradient lives on the sampled tiles only (so the oracle's tile
subset sees all of it)."""
import numpy as np
import pytest
import torch

from oracle import surfel_oracle as O
from tests._util import grad_check, image_error

pytestmark = pytest.mark.gpu

IMG_TOL, AUX_TOL = 1e-5, 3e-5
N_TILES = 10


@pytest.fixture(scope="module")
def case(sgr_lib):
    from partgs_gb300 import _lib as L
    from partgs_gb300 import raster
    from partgs_gb300.scenes import workload
    scene, cams = workload("sq500k_16x800x600", 0)
    cam = cams[0]
    H, W = cam.height, cam.width
    dev = torch.device("cuda")
    sc = scene.to(dev)
    vm = torch.as_tensor(cam.world_view_transform, device=dev).reshape(1, 16)
    pm = torch.as_tensor(cam.full_proj_transform, device=dev).reshape(1, 16)
    cp = torch.as_tensor(cam.camera_center, device=dev).reshape(1, 3)
    vs = raster.ViewSet(vm, pm, cp, [(cam.tanfovx, cam.tanfovy)], H, W)
    bg = torch.zeros(3, device=dev)
    color, others, _, radii, state = raster.forward(L.SGR_VARIANT_PLAIN, sc.means3D, sc.opacities, sc.shs, None,
                                                    sc.scales, sc.rotations, None, None, vs, bg, 3, cell_tiles=2)
    s = state.sizes
    nc = state.geom[s.off_n_contrib:s.off_n_contrib + 2 * H * W * 4].view(torch.int32).reshape(2, H, W)

    ocam = O.Camera(cam.world_view_transform.reshape(-1), cam.full_proj_transform.reshape(-1), cam.camera_center,
                    cam.tanfovx, cam.tanfovy, H, W)
    osf = O.Surfels(scene.means3D.numpy(), scene.opacities.numpy(), scene.scales.numpy(), scene.rotations.numpy(),
                    shs=scene.shs.numpy(), sh_degree=3)
    # Surfels whose radius (a ceil of an fp32 expression) lands within fp32
    # rounding of an integer may get another radius in fp32 than in fp64; at
    # 500k surfels there are a few dozen.  The reference's fp32 CUDA flips on
    # them as this kernel does.  Their tiles' lists can then differ, so the
    # tiles along both of their rectangles are left out of the comparison.
    pre64 = O.preprocess(osf, ocam, O.PLAIN, np.float64)
    pre32 = O.preprocess(osf, ocam, O.PLAIN, np.float32)
    gpu_r = radii.cpu().numpy()
    divergent = pre64["amb"] | pre32["amb"] | (gpu_r != pre64["radii"]) | (pre32["radii"] != pre64["radii"])
    gx, gy = pre64["grid"]
    touched = np.zeros((gy, gx), bool)
    for i in np.nonzero(divergent)[0]:
        for r in {int(gpu_r[i]), int(pre64["radii"][i]), int(pre32["radii"][i])}:
            x0, y0, x1, y1 = O._rect(pre64["means2D"][i, 0], pre64["means2D"][i, 1], np.float64(r), gx, gy,
                                     np.float64)
            touched[max(0, y0 - 1):min(gy, max(y1, y0 + 1) + 1), max(0, x0 - 1):min(gx, max(x1, x0 + 1) + 1)] = True
    _, ranges64, _ = O.bin_tiles(pre64)
    usable = np.nonzero((ranges64[:, 1] > ranges64[:, 0]) & ~touched.reshape(-1))[0]
    tiles = np.sort(np.random.default_rng(7).choice(usable, N_TILES, replace=False))
    st = O.forward_view(osf, ocam, np.zeros(3), O.PLAIN, np.float64, tiles=tiles)
    on = np.zeros((H, W), bool)                      # pixels of the sampled tiles
    for t in tiles:
        ty, tx = divmod(int(t), gx)
        on[16 * ty:16 * ty + 16, 16 * tx:16 * tx + 16] = True
    amb = st.amb_pixel | ~on

    g = np.random.default_rng(3)
    dcol = (g.standard_normal((3, H, W)) * on).astype(np.float32)
    doth = (g.standard_normal((7, H, W)) * 0.1 * on).astype(np.float32)
    dcol[:, st.amb_pixel] = 0
    doth[:, st.amb_pixel] = 0
    grads = raster.backward(state, torch.from_numpy(dcol)[None].cuda(), torch.from_numpy(doth)[None].cuda())
    ref_g = O.backward_view(st, ocam, osf, np.zeros(3), dcol, doth, variant=O.PLAIN, dtype=np.float64, tiles=tiles)
    torch.cuda.synchronize()
    return dict(color=color[0].cpu().numpy(), others=others[0].cpu().numpy(), nc=nc.cpu().numpy(),
                radii=gpu_r, st=st, amb=amb, on=on, pre32=pre32, divergent=divergent,
                grads={k: v.cpu().numpy() for k, v in grads.items()}, ref_g=ref_g)


def test_radii(case):
    """Every radius equals the fp64 oracle's except on surfels where fp32 and
    fp64 may round it differently (flagged by either oracle as near a
    boundary, or rounded differently by them, or by this kernel), and those
    are rare."""
    st, d = case["st"], case["divergent"]
    P = len(case["radii"])
    np.testing.assert_array_equal(case["radii"][~d], st.radii[~d])
    # fp32 against fp64 flips: about 1e-4 of the surfels; the oracles also
    # flag those within FP32 rounding of a boundary, counting the
    # cancellation in the extent: about 0.25%
    flips = int((case["radii"] != st.radii).sum())
    assert flips <= 2e-4 * P, flips
    assert d.sum() <= 4e-3 * P, int(d.sum())
    assert (case["radii"] > 0).sum() > 100_000


def test_images_and_contributors_on_sampled_tiles(case):
    st, amb = case["st"], case["amb"]
    assert (~amb).sum() >= 0.9 * case["on"].sum()
    assert max(image_error(case["color"], st.color, amb)) <= IMG_TOL
    assert max(image_error(case["others"], st.others, amb)) <= AUX_TOL
    np.testing.assert_array_equal(case["nc"][0][~amb], st.n_contrib[0][~amb])
    np.testing.assert_array_equal(case["nc"][1][~amb], st.n_contrib[1][~amb])
    assert st.n_contrib[0][~amb].max() > 50     # deep lists: the scene's dense regions are sampled


def test_gradients_from_sampled_tiles(case):
    g, r = case["grads"], case["ref_g"]
    names = ["dL_dcolors", "dL_dopacity", "dL_dmeans3D", "dL_dtransmat", "dL_dsh", "dL_dscales",
             "dL_drotations", "dL_dmeans2D"]
    errs, bad = grad_check(g, r, names)
    assert not bad, errs
    assert float(np.abs(r["dL_dmeans3D"]).max()) > 0
