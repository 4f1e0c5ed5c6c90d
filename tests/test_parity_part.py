"""Parity of the part-map variant (semantic channels, 8-channel aux maps,
half-pixel centres, double-precision constants) against the oracle."""
import numpy as np
import pytest
import torch

from oracle import surfel_oracle as O
from tests._util import grad_check, grad_error, image_error, oracle_camera, oracle_surfels, settings

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=[5, 13, 16], ids=lambda n: f"S{n}")
def case(sgr_lib, request):
    """S semantic channels: 5 (the 8-value reduction), 13 (the 16-value one,
    with a partly filled float4 group) and 16 (the maximum)."""
    S = request.param
    import partgs_gb300.diff_surfel_rasterization_part as dsrp
    from partgs_gb300.scenes import random_surfels
    from partgs_gb300.cameras import orbit_cameras
    scene = random_surfels(3000, seed=11)
    cam = orbit_cameras(1, 3.0, 96, 112, 55.0, seed=5)[0]
    sem = torch.rand(scene.P, S, generator=torch.Generator().manual_seed(2))
    sc = scene.to("cuda")
    rs = settings(dsrp, cam, [0.3, 0.1, 0.2])
    means3D = sc.means3D.clone().requires_grad_(True)
    means2D = torch.zeros_like(means3D, requires_grad=True)
    sem_d = sem.cuda().requires_grad_(True)
    shs = sc.shs.clone().requires_grad_(True)
    opac = sc.opacities.clone().requires_grad_(True)
    scales = sc.scales.clone().requires_grad_(True)
    rots = sc.rotations.clone().requires_grad_(True)
    img, sem_img, radii, allmap = dsrp.GaussianRasterizer(rs)(means3D=means3D, means2D=means2D, opacities=opac,
                                                              semantics=sem_d, shs=shs, scales=scales,
                                                              rotations=rots)
    ocam = oracle_camera(cam)
    osf = oracle_surfels(scene, semantics=sem)
    st = O.forward_view(osf, ocam, np.array([0.3, 0.1, 0.2]), O.PART, np.float64)
    g = np.random.default_rng(4)
    dcol = g.standard_normal(st.color.shape).astype(np.float32)
    doth = (g.standard_normal(st.others.shape) * 0.1).astype(np.float32)
    dsem = g.standard_normal(st.semantic.shape).astype(np.float32)
    amb = st.amb_pixel
    for a in (dcol, doth, dsem):
        a[:, amb] = 0
    loss = (img * torch.from_numpy(dcol).cuda()).sum() + (allmap * torch.from_numpy(doth).cuda()).sum() + \
        (sem_img * torch.from_numpy(dsem).cuda()).sum()
    loss.backward()
    ref = O.backward_view(st, ocam, osf, np.array([0.3, 0.1, 0.2]), dcol, doth, dsem, variant=O.PART,
                          dtype=np.float64)
    # the same algorithm in FP32 (numpy): its distance to FP64 is the
    # rounding floor any FP32 implementation of the reference sits at
    st32 = O.forward_view(osf, ocam, np.array([0.3, 0.1, 0.2]), O.PART, np.float32)
    return dict(S=S, img=img.detach().cpu().numpy(), sem=sem_img.detach().cpu().numpy(),
                allmap=allmap.detach().cpu().numpy(), radii=radii.cpu().numpy(), st=st, amb=amb, ref=ref,
                st32=st32,
                grads=dict(dL_dmeans3D=means3D.grad, dL_dsh=shs.grad, dL_dopacity=opac.grad,
                           dL_dscales=scales.grad, dL_drotations=rots.grad, dL_dsemantics=sem_d.grad,
                           dL_dmeans2D=means2D.grad))


def test_part_shapes(case):
    assert case["img"].shape == (3, 96, 112)
    assert case["sem"].shape == (case["S"], 96, 112)
    assert case["allmap"].shape == (8, 96, 112)


def test_part_radii_bit_exact(case):
    st = case["st"]
    ok = ~st.amb_surfel
    np.testing.assert_array_equal(case["radii"][ok], st.radii[ok])


def _floor(spec, fp32_err):
    """Tolerance: the stated bound, or twice the FP32 rounding floor of the
    reference's algorithm on this very case when that floor is higher."""
    return max(spec, 2.0 * fp32_err)


def test_part_images(case):
    st, st32, amb = case["st"], case["st32"], case["amb"] | case["st32"].amb_pixel
    for mine, ref, ref32, spec in ((case["img"], st.color, st32.color, 1e-5),
                                   (case["sem"], st.semantic, st32.semantic, 3e-5),
                                   (case["allmap"], st.others, st32.others, 3e-5)):
        err = max(image_error(mine, ref, amb))
        assert err <= _floor(spec, max(image_error(ref32, ref, amb))), err


def test_part_gradients(case):
    got = {k: v.cpu().numpy() for k, v in case["grads"].items()}
    errs, bad = grad_check(got, case["ref"])
    assert not bad, errs
