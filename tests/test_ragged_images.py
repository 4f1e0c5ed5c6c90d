"""Images whose sides are not multiples of the 16-pixel tile (77 x 45 and
a 1-pixel-high, 33-pixel-wide strip): the last tile column and row are
partial, and the pixels beyond the image exist in neither the outputs nor
the gradients.  Both variants, against the oracle, through the drop-in API.

Tolerances are the stated bars, or twice the distance between the oracle
run in FP32 and in FP64 on the same case where that rounding floor of the
reference's algorithm is higher."""
import numpy as np
import pytest
import torch

from oracle import surfel_oracle as O
from tests._util import grad_check, grad_error, image_error, oracle_camera, oracle_surfels, settings

pytestmark = pytest.mark.gpu

IMG_TOL = 1e-5
AUX_TOL = 3e-5
BG = [0.3, 0.2, 0.6]


def _floor(spec, fp32_err):
    return max(spec, 2.0 * fp32_err)


@pytest.mark.parametrize("variant", [O.PLAIN, O.PART], ids=["plain", "part"])
@pytest.mark.parametrize("hw", [(45, 77), (1, 33)], ids=["45x77", "1x33"])
def test_partial_tiles(sgr_lib, hw, variant):
    import partgs_gb300.diff_surfel_rasterization as dsr
    import partgs_gb300.diff_surfel_rasterization_part as dsrp
    from partgs_gb300.cameras import orbit_cameras
    from partgs_gb300.scenes import random_surfels
    H, W = hw
    scene = random_surfels(1500, seed=41)
    cam = orbit_cameras(1, 3.0, H, W, 50.0, seed=17)[0]
    mod = dsr if variant == O.PLAIN else dsrp
    S = 5
    sem = torch.rand(scene.P, S, generator=torch.Generator().manual_seed(3)) if variant == O.PART else None
    sc = scene.to("cuda")
    leaves = {k: getattr(sc, k).clone().requires_grad_(True)
              for k in ("means3D", "shs", "opacities", "scales", "rotations")}
    means2D = torch.zeros_like(leaves["means3D"], requires_grad=True)
    rs = settings(mod, cam, BG)
    kw = dict(means3D=leaves["means3D"], means2D=means2D, opacities=leaves["opacities"], shs=leaves["shs"],
              scales=leaves["scales"], rotations=leaves["rotations"])
    sem_img = None
    if variant == O.PART:
        sem_d = sem.cuda().requires_grad_(True)
        kw["semantics"] = sem_d
        img, sem_img, radii, allmap = mod.GaussianRasterizer(rs)(**kw)
        assert sem_img.shape == (S, H, W)
    else:
        img, radii, allmap = mod.GaussianRasterizer(rs)(**kw)
    assert img.shape == (3, H, W) and allmap.shape == (7 if variant == O.PLAIN else 8, H, W)

    ocam = oracle_camera(cam)
    osf = oracle_surfels(scene, semantics=sem)
    st = O.forward_view(osf, ocam, np.array(BG), variant, np.float64)
    st32 = O.forward_view(osf, ocam, np.array(BG), variant, np.float32)
    amb = st.amb_pixel | st32.amb_pixel
    assert amb.mean() < 0.05
    pairs = [(img, st.color, st32.color, IMG_TOL), (allmap, st.others, st32.others, AUX_TOL)]
    if variant == O.PART:
        pairs.append((sem_img, st.semantic, st32.semantic, AUX_TOL))
    for mine, r64, r32, spec in pairs:
        err = max(image_error(mine.detach().cpu().numpy(), r64, amb))
        assert err <= _floor(spec, max(image_error(r32, r64, amb))), err
    ok = ~st.amb_surfel
    np.testing.assert_array_equal(radii.cpu().numpy()[ok], st.radii[ok])
    assert (st.radii > 0).sum() > 0

    g = np.random.default_rng(11)
    dcol = g.standard_normal(st.color.shape).astype(np.float32)
    doth = (g.standard_normal(st.others.shape) * 0.1).astype(np.float32)
    dcol[:, amb] = 0
    doth[:, amb] = 0
    loss = (img * torch.from_numpy(dcol).cuda()).sum() + (allmap * torch.from_numpy(doth).cuda()).sum()
    dsem = None
    if variant == O.PART:
        dsem = g.standard_normal(st.semantic.shape).astype(np.float32)
        dsem[:, amb] = 0
        loss = loss + (sem_img * torch.from_numpy(dsem).cuda()).sum()
    loss.backward()
    ref = O.backward_view(st, ocam, osf, np.array(BG), dcol, doth, dsem, variant=variant, dtype=np.float64)
    got = {name: leaves[leaf].grad for name, leaf in
           (("dL_dsh", "shs"), ("dL_dmeans3D", "means3D"), ("dL_dopacity", "opacities"),
            ("dL_dscales", "scales"), ("dL_drotations", "rotations"))}
    got["dL_dmeans2D"] = means2D.grad
    if variant == O.PART:
        got["dL_dsemantics"] = sem_d.grad
    errs, bad = grad_check({k: t.cpu().numpy() for k, t in got.items()}, ref)
    assert not bad, errs
