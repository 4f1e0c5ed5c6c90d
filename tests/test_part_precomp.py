"""The part variant with precomputed colours (override_color,
renderer/gaussian_renderer_2d/__init__.py:78-79), with scales and rotations
or with a precomputed splat-to-pixel matrix (cov3D_precomp, :58-59).  The matrix's gradient
runs through the part variant's own transMat adjoint
(P1/cr/backward.cu:556-671).  Images, semantics and gradients against the
oracle, through the drop-in API.

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
BG = [0.1, 0.5, 0.3]


def _floor(spec, fp32_err):
    return max(spec, 2.0 * fp32_err)


@pytest.fixture(scope="module")
def base(sgr_lib):
    from partgs_gb300.cameras import orbit_cameras
    from partgs_gb300.scenes import random_surfels
    scene = random_surfels(1500, seed=51)
    cam = orbit_cameras(1, 3.0, 64, 80, 55.0, seed=23)[0]
    sem = torch.rand(scene.P, 4, generator=torch.Generator().manual_seed(6))
    cols = torch.rand(scene.P, 3, generator=torch.Generator().manual_seed(7))
    return scene, cam, sem, cols


def test_part_precomputed_colours_with_scales_and_rotations(base):
    """Precomputed colours with scales and rotations (the transMat from the
    part variant's own preprocess and its adjoint, P1/cr/backward.cu:473-671,
    and the AABB-centre adjoint, :621-671).  The upstream-gradient mask comes
    from the FP64 oracle alone, so the case is the same on every host."""
    import partgs_gb300.diff_surfel_rasterization_part as dsrp
    scene, cam, sem, cols = base
    ocam = oracle_camera(cam)
    sc = scene.to("cuda")
    leaves = {"dL_dmeans3D": sc.means3D, "dL_dcolors": cols.cuda(), "dL_dopacity": sc.opacities,
              "dL_dsemantics": sem.cuda(), "dL_dscales": sc.scales, "dL_drotations": sc.rotations}
    leaves = {k: v.clone().requires_grad_(True) for k, v in leaves.items()}
    means2D = torch.zeros_like(leaves["dL_dmeans3D"], requires_grad=True)
    rs = settings(dsrp, cam, BG)
    img, sem_img, radii, allmap = dsrp.GaussianRasterizer(rs)(
        means3D=leaves["dL_dmeans3D"], means2D=means2D, opacities=leaves["dL_dopacity"],
        colors_precomp=leaves["dL_dcolors"], semantics=leaves["dL_dsemantics"], scales=leaves["dL_dscales"],
        rotations=leaves["dL_drotations"])
    osf = oracle_surfels(scene, colors_precomp=cols, semantics=sem)
    st = O.forward_view(osf, ocam, np.array(BG), O.PART, np.float64)
    amb = st.amb_pixel
    assert amb.mean() < 0.01
    assert max(image_error(img.detach().cpu().numpy(), st.color, amb)) <= IMG_TOL
    assert max(image_error(allmap.detach().cpu().numpy(), st.others, amb)) <= AUX_TOL
    assert max(image_error(sem_img.detach().cpu().numpy(), st.semantic, amb)) <= AUX_TOL
    ok = ~st.amb_surfel
    np.testing.assert_array_equal(radii.cpu().numpy()[ok], st.radii[ok])
    g = np.random.default_rng(5)
    dcol = g.standard_normal(st.color.shape).astype(np.float32)
    doth = (g.standard_normal(st.others.shape) * 0.1).astype(np.float32)
    dsem = g.standard_normal(st.semantic.shape).astype(np.float32)
    for a in (dcol, doth, dsem):
        a[:, amb] = 0
    loss = (img * torch.from_numpy(dcol).cuda()).sum() + (allmap * torch.from_numpy(doth).cuda()).sum() + \
        (sem_img * torch.from_numpy(dsem).cuda()).sum()
    loss.backward()
    ref = O.backward_view(st, ocam, osf, np.array(BG), dcol, doth, dsem, variant=O.PART, dtype=np.float64)
    got = {k: v.grad for k, v in leaves.items()}
    got["dL_dmeans2D"] = means2D.grad
    assert all(t is not None for t in got.values())
    errs, bad = grad_check({k: t.cpu().numpy() for k, t in got.items()}, ref)
    assert not bad, errs


def test_part_precomputed_transmat_and_colours(base):
    import partgs_gb300.diff_surfel_rasterization_part as dsrp
    scene, cam, sem, cols = base
    ocam = oracle_camera(cam)
    sc = scene.to("cuda")
    leaves = {"dL_dmeans3D": sc.means3D, "dL_dcolors": cols.cuda(), "dL_dopacity": sc.opacities,
              "dL_dsemantics": sem.cuda()}
    pre = O.preprocess(oracle_surfels(scene, semantics=sem), ocam, O.PART, np.float64)
    T = torch.tensor(pre["transmat"], dtype=torch.float32)
    leaves["dL_dtransmat"] = T.cuda()
    osf = oracle_surfels(scene, colors_precomp=cols, transmat=T, semantics=sem)
    leaves = {k: v.clone().requires_grad_(True) for k, v in leaves.items()}
    means2D = torch.zeros_like(leaves["dL_dmeans3D"], requires_grad=True)
    rs = settings(dsrp, cam, BG)
    img, sem_img, radii, allmap = dsrp.GaussianRasterizer(rs)(
        means3D=leaves["dL_dmeans3D"], means2D=means2D, opacities=leaves["dL_dopacity"],
        colors_precomp=leaves["dL_dcolors"], semantics=leaves["dL_dsemantics"],
        cov3D_precomp=leaves["dL_dtransmat"])

    st = O.forward_view(osf, ocam, np.array(BG), O.PART, np.float64)
    st32 = O.forward_view(osf, ocam, np.array(BG), O.PART, np.float32)
    amb = st.amb_pixel | st32.amb_pixel
    assert amb.mean() < 0.01
    for mine, r64, r32, spec in ((img, st.color, st32.color, IMG_TOL), (allmap, st.others, st32.others, AUX_TOL),
                                 (sem_img, st.semantic, st32.semantic, AUX_TOL)):
        err = max(image_error(mine.detach().cpu().numpy(), r64, amb))
        assert err <= _floor(spec, max(image_error(r32, r64, amb))), err
    ok = ~st.amb_surfel
    np.testing.assert_array_equal(radii.cpu().numpy()[ok], st.radii[ok])

    g = np.random.default_rng(5)
    dcol = g.standard_normal(st.color.shape).astype(np.float32)
    doth = (g.standard_normal(st.others.shape) * 0.1).astype(np.float32)
    dsem = g.standard_normal(st.semantic.shape).astype(np.float32)
    for a in (dcol, doth, dsem):
        a[:, amb] = 0
    loss = (img * torch.from_numpy(dcol).cuda()).sum() + (allmap * torch.from_numpy(doth).cuda()).sum() + \
        (sem_img * torch.from_numpy(dsem).cuda()).sum()
    loss.backward()
    ref = O.backward_view(st, ocam, osf, np.array(BG), dcol, doth, dsem, variant=O.PART, dtype=np.float64)
    got = {k: v.grad for k, v in leaves.items()}
    got["dL_dmeans2D"] = means2D.grad
    assert all(t is not None for t in got.values())
    errs, bad = grad_check({k: t.cpu().numpy() for k, t in got.items()}, ref)
    assert not bad, errs
