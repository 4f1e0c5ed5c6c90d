"""The rasteriser at SH degrees 0, 1 and 2 with all 16 coefficients per
surfel stored, as in training.  The reference raises the active degree by
one every 1000 iterations (train.py:214, scene/gaussian_model.py:223-225)
and keeps passing the full [P, 16, 3] SH tensor with sh_degree =
active_sh_degree.  Images and gradients are compared with the oracle.  The
gradients of the coefficients above the active degree must be exactly
zero.

Tolerances are the stated bars, or twice the distance between the oracle
run in FP32 and in FP64 on the same case where that rounding floor of the
reference's algorithm is higher (the rotation and mean gradients cancel:
up to 1.7e-4 here)."""
import numpy as np
import pytest
import torch

from oracle import surfel_oracle as O
from tests._util import grad_check, grad_error, image_error, oracle_camera, oracle_surfels, settings

pytestmark = pytest.mark.gpu

IMG_TOL = 1e-5
AUX_TOL = 3e-5
BG = [0.2, 0.4, 0.1]


def _floor(spec, fp32_err):
    return max(spec, 2.0 * fp32_err)


@pytest.fixture(scope="module")
def base(sgr_lib):
    from partgs_gb300.cameras import orbit_cameras
    from partgs_gb300.scenes import random_surfels
    return random_surfels(2000, seed=31), orbit_cameras(1, 3.0, 80, 96, 55.0, seed=13)[0]


@pytest.mark.parametrize("variant", [O.PLAIN, O.PART], ids=["plain", "part"])
@pytest.mark.parametrize("deg", [0, 1, 2])
def test_lower_sh_degree_with_sixteen_coefficients(base, deg, variant):
    import partgs_gb300.diff_surfel_rasterization as dsr
    import partgs_gb300.diff_surfel_rasterization_part as dsrp
    scene, cam = base
    mod = dsr if variant == O.PLAIN else dsrp
    assert scene.shs.shape[1] == 16
    sem = torch.rand(scene.P, 3, generator=torch.Generator().manual_seed(deg)) if variant == O.PART else None
    sc = scene.to("cuda")
    leaves = {k: getattr(sc, k).clone().requires_grad_(True)
              for k in ("means3D", "shs", "opacities", "scales", "rotations")}
    means2D = torch.zeros_like(leaves["means3D"], requires_grad=True)
    rs = settings(mod, cam, BG, sh_degree=deg)
    kw = dict(means3D=leaves["means3D"], means2D=means2D, opacities=leaves["opacities"], shs=leaves["shs"],
              scales=leaves["scales"], rotations=leaves["rotations"])
    if variant == O.PART:
        kw["semantics"] = sem.cuda()
        img, _, radii, allmap = mod.GaussianRasterizer(rs)(**kw)
    else:
        img, radii, allmap = mod.GaussianRasterizer(rs)(**kw)

    ocam = oracle_camera(cam)
    osf = oracle_surfels(scene, semantics=sem, sh_degree=deg)
    st = O.forward_view(osf, ocam, np.array(BG), variant, np.float64)
    st32 = O.forward_view(osf, ocam, np.array(BG), variant, np.float32)
    amb = st.amb_pixel | st32.amb_pixel
    assert amb.mean() < 0.01
    for mine, r64, r32, spec in ((img, st.color, st32.color, IMG_TOL), (allmap, st.others, st32.others, AUX_TOL)):
        err = max(image_error(mine.detach().cpu().numpy(), r64, amb))
        assert err <= _floor(spec, max(image_error(r32, r64, amb))), err
    ok = ~st.amb_surfel
    np.testing.assert_array_equal(radii.cpu().numpy()[ok], st.radii[ok])

    g = np.random.default_rng(7 + deg)
    dcol = g.standard_normal(st.color.shape).astype(np.float32)
    doth = (g.standard_normal(st.others.shape) * 0.1).astype(np.float32)
    dcol[:, st.amb_pixel] = 0
    doth[:, st.amb_pixel] = 0
    loss = (img * torch.from_numpy(dcol).cuda()).sum() + (allmap * torch.from_numpy(doth).cuda()).sum()
    loss.backward()
    dsem = np.zeros((3,) + st.color.shape[1:], np.float32) if variant == O.PART else None
    ref = O.backward_view(st, ocam, osf, np.array(BG), dcol, doth, dsem, variant=variant, dtype=np.float64)

    dsh = leaves["shs"].grad.cpu().numpy()
    used = (deg + 1) ** 2
    assert np.count_nonzero(dsh[:, used:]) == 0, "gradient reached coefficients above the active degree"
    assert np.abs(dsh[:, :used]).max() > 0
    got, want = {}, {}
    for name, leaf in (("dL_dsh", "shs"), ("dL_dmeans3D", "means3D"), ("dL_dopacity", "opacities"),
                       ("dL_dscales", "scales"), ("dL_drotations", "rotations")):
        mine = leaves[leaf].grad.cpu().numpy()
        r64 = np.asarray(ref[name]).reshape(mine.shape)
        if name == "dL_dsh":
            mine, r64 = mine[:, :used], r64[:, :used]
        got[name], want[name] = mine, r64
    errs, bad = grad_check(got, want)
    assert not bad, errs
