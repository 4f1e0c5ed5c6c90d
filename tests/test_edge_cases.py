"""Edge cases the reference's API admits: empty inputs, nothing visible (both
variants), precomputed colours and transMats, the scale modifier, the
prefiltered contract, key-list overflow, near-plane visibility."""
import numpy as np
import pytest
import torch

from oracle import surfel_oracle as O
from tests._util import grad_error, image_error, oracle_camera, oracle_surfels, settings

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def base(sgr_lib):
    from partgs_gb300.cameras import orbit_cameras
    from partgs_gb300.scenes import random_surfels
    return random_surfels(1500, seed=21), orbit_cameras(1, 3.0, 64, 64, 60.0, seed=9)[0]


def _render(mod, cam, bg=(0.0, 0.0, 0.0), **kw):
    rs = settings(mod, cam, list(bg), scale_modifier=kw.pop("scale_modifier", 1.0),
                  prefiltered=kw.pop("prefiltered", False))
    return mod.GaussianRasterizer(rs)(**kw)


def test_empty_scene_returns_zero_images(base):
    import partgs_gb300.diff_surfel_rasterization as dsr
    _, cam = base
    x = torch.zeros(0, 3, device="cuda")
    img, radii, allmap = _render(dsr, cam, (0.5, 0.5, 0.5), means3D=x, means2D=x, opacities=torch.zeros(0, 1, device="cuda"),
                                 colors_precomp=x, scales=torch.zeros(0, 2, device="cuda"),
                                 rotations=torch.zeros(0, 4, device="cuda"))
    assert img.shape == (3, 64, 64) and float(img.abs().max()) == 0.0
    assert allmap.shape == (7, 64, 64) and radii.numel() == 0


def test_everything_behind_the_camera_gives_background(base):
    import partgs_gb300.diff_surfel_rasterization as dsr
    scene, cam = base
    sc = scene.to("cuda")
    campos = torch.as_tensor(cam.camera_center, device="cuda")
    behind = campos * 2.0 + (sc.means3D * 0.01)        # on the far side of the camera
    img, radii, allmap = _render(dsr, cam, (0.25, 0.5, 0.75), means3D=behind, means2D=behind, opacities=sc.opacities,
                                 shs=sc.shs, scales=sc.scales, rotations=sc.rotations)
    assert int((radii > 0).sum()) == 0
    np.testing.assert_allclose(img.cpu().numpy().reshape(3, -1).mean(1), [0.25, 0.5, 0.75], atol=1e-7)
    assert float(allmap.abs().max()) == 0.0


def test_prefiltered_violation_raises(base):
    import partgs_gb300.diff_surfel_rasterization as dsr
    scene, cam = base
    sc = scene.to("cuda")
    campos = torch.as_tensor(cam.camera_center, device="cuda")
    m = sc.means3D.clone()
    m[0] = campos * 2.0
    with pytest.raises(RuntimeError, match="prefiltered"):
        _render(dsr, cam, prefiltered=True, means3D=m, means2D=m, opacities=sc.opacities, shs=sc.shs,
                scales=sc.scales, rotations=sc.rotations)


def test_colors_precomp_and_scale_modifier(base):
    import partgs_gb300.diff_surfel_rasterization as dsr
    scene, cam = base
    sc = scene.to("cuda")
    cols = torch.rand(scene.P, 3, generator=torch.Generator().manual_seed(1))
    img, radii, allmap = _render(dsr, cam, scale_modifier=0.8, means3D=sc.means3D, means2D=sc.means3D,
                                 opacities=sc.opacities, colors_precomp=cols.cuda(), scales=sc.scales,
                                 rotations=sc.rotations)
    st = O.forward_view(oracle_surfels(scene, colors_precomp=cols, scale_modifier=0.8), oracle_camera(cam),
                        np.zeros(3), O.PLAIN, np.float64)
    assert max(image_error(img.cpu().numpy(), st.color, st.amb_pixel)) <= 1e-5
    assert max(image_error(allmap.cpu().numpy(), st.others, st.amb_pixel)) <= 3e-5


def test_transmat_precomp_forward_and_gradient(base):
    """cov3D_precomp carries the splat-to-pixel matrix; its gradient is the
    accumulated dL/dT plus the centre adjoint (P0/cr/backward.cu:514-542)."""
    import partgs_gb300.diff_surfel_rasterization as dsr
    scene, cam = base
    pre = O.preprocess(oracle_surfels(scene), oracle_camera(cam), O.PLAIN, np.float64)
    T = torch.tensor(pre["transmat"], dtype=torch.float32)
    cols = torch.rand(scene.P, 3, generator=torch.Generator().manual_seed(3))
    sc = scene.to("cuda")
    Td = T.cuda().requires_grad_(True)
    img, radii, allmap = _render(dsr, cam, means3D=sc.means3D, means2D=sc.means3D, opacities=sc.opacities,
                                 colors_precomp=cols.cuda(), cov3D_precomp=Td)
    osf = oracle_surfels(scene, colors_precomp=cols, transmat=T)
    st = O.forward_view(osf, oracle_camera(cam), np.zeros(3), O.PLAIN, np.float64)
    assert max(image_error(img.detach().cpu().numpy(), st.color, st.amb_pixel)) <= 1e-5
    g = np.random.default_rng(0)
    dcol = g.standard_normal(st.color.shape).astype(np.float32)
    dcol[:, st.amb_pixel] = 0
    (img * torch.from_numpy(dcol).cuda()).sum().backward()
    ref = O.backward_view(st, oracle_camera(cam), osf, np.zeros(3), dcol, np.zeros_like(st.others), variant=O.PLAIN)
    assert grad_error(Td.grad.cpu().numpy(), ref["dL_dtransmat"]) <= 3e-4


def test_cell_list_overflow_is_flagged_not_faulted(base):
    from partgs_gb300 import _lib as L
    from partgs_gb300 import raster
    scene, cam = base
    sc = scene.to("cuda")
    rs = settings(__import__("partgs_gb300.diff_surfel_rasterization", fromlist=["x"]), cam, [0, 0, 0])
    vs = raster.ViewSet(rs.viewmatrix.reshape(1, 16), rs.projmatrix.reshape(1, 16), rs.campos.reshape(1, 3),
                        [(cam.tanfovx, cam.tanfovy)], cam.height, cam.width)
    status = torch.zeros(L.STATUS_BYTES, dtype=torch.uint8).pin_memory()
    args = (0, sc.means3D, sc.opacities, sc.shs, None, sc.scales, sc.rotations, None, None, vs, rs.bg, 3)
    color, others, _, radii, st = raster.forward(*args, bin_capacity=100, status_host=status)
    torch.cuda.synchronize()
    K, flags, nbins = raster.read_status(status)
    assert nbins > 100 and flags & L.SGR_FLAG_BIN_OVERFLOW
    assert torch.isfinite(color).all() and torch.isfinite(others).all()
    # with room for every entry the same call is exact and raises no flag
    color2, _, _, _, _ = raster.forward(*args, bin_capacity=nbins, status_host=status)
    torch.cuda.synchronize()
    assert raster.read_status(status)[1] == 0
    color3, _, _, _, _ = raster.forward(*args)
    assert torch.equal(color2, color3)


def test_mark_visible(base):
    import partgs_gb300.diff_surfel_rasterization as dsr
    scene, cam = base
    m = scene.means3D.clone()
    m[::7] = torch.as_tensor(cam.camera_center) * 1.5
    rs = settings(dsr, cam, [0, 0, 0])
    vis = dsr.GaussianRasterizer(rs).markVisible(m.cuda()).cpu().numpy()
    np.testing.assert_array_equal(vis, O.mark_visible(m.numpy(), cam.world_view_transform.reshape(-1)))
    assert vis.dtype == bool and (~vis).sum() > 0


def test_part_empty_scene_returns_zero_maps(base):
    """The part drop-in with no surfels: zero colour, semantic and auxiliary
    maps, no radii (the packed part kernels launch with every list empty)."""
    import partgs_gb300.diff_surfel_rasterization_part as dsrp
    _, cam = base
    x = torch.zeros(0, 3, device="cuda")
    img, sem, radii, allmap = _render(dsrp, cam, (0.5, 0.5, 0.5), means3D=x, means2D=x,
                                      opacities=torch.zeros(0, 1, device="cuda"),
                                      semantics=torch.zeros(0, 6, device="cuda"), colors_precomp=x,
                                      scales=torch.zeros(0, 2, device="cuda"),
                                      rotations=torch.zeros(0, 4, device="cuda"))
    assert img.shape == (3, 64, 64) and float(img.abs().max()) == 0.0
    assert sem.shape == (6, 64, 64) and float(sem.abs().max()) == 0.0
    assert allmap.shape == (8, 64, 64) and radii.numel() == 0


def test_part_everything_behind_the_camera_gives_background(base):
    """The part drop-in with every surfel behind the camera: the background,
    zero semantics and auxiliary maps, and zero gradients."""
    import partgs_gb300.diff_surfel_rasterization_part as dsrp
    scene, cam = base
    sc = scene.to("cuda")
    campos = torch.as_tensor(cam.camera_center, device="cuda")
    behind = (campos * 2.0 + (sc.means3D * 0.01)).requires_grad_(True)
    sem = torch.rand(sc.means3D.shape[0], 6, device="cuda").requires_grad_(True)
    img, smap, radii, allmap = _render(dsrp, cam, (0.25, 0.5, 0.75), means3D=behind, means2D=torch.zeros_like(behind),
                                       opacities=sc.opacities, semantics=sem, shs=sc.shs, scales=sc.scales,
                                       rotations=sc.rotations)
    assert int((radii > 0).sum()) == 0
    np.testing.assert_allclose(img.detach().cpu().numpy().reshape(3, -1).mean(1), [0.25, 0.5, 0.75], atol=1e-7)
    assert float(smap.detach().abs().max()) == 0.0 and float(allmap.detach().abs().max()) == 0.0
    (img.sum() + smap.sum() + allmap.sum()).backward()
    assert float(behind.grad.abs().max()) == 0.0 and float(sem.grad.abs().max()) == 0.0
