"""The batched paths: many views in one call equal per-view calls; uneven
scenes in one call equal separate calls; the graph-captured training step
equals the eager step."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup(sgr_lib):
    from partgs_gb300.cameras import orbit_cameras
    from partgs_gb300.scenes import random_surfels
    return random_surfels(2500, seed=31), orbit_cameras(4, 3.0, 72, 88, 55.0, seed=13)


def _per_view(scene, cams, dcol, doth):
    import partgs_gb300.diff_surfel_rasterization as dsr
    from tests._util import settings
    sc = scene.to("cuda")
    m = sc.means3D.clone().requires_grad_(True)
    imgs, maps, radii = [], [], []
    for v, cam in enumerate(cams):
        rs = settings(dsr, cam, [0.1, 0.1, 0.1])
        img, r, am = dsr.GaussianRasterizer(rs)(means3D=m, means2D=torch.zeros_like(m), opacities=sc.opacities,
                                                shs=sc.shs, scales=sc.scales, rotations=sc.rotations)
        imgs.append(img)
        maps.append(am)
        radii.append(r)
    loss = sum((i * dcol[v]).sum() + (a * doth[v]).sum() for v, (i, a) in enumerate(zip(imgs, maps)))
    loss.backward()
    return torch.stack(imgs), torch.stack(maps), torch.cat(radii), m.grad


def test_multiview_equals_per_view(setup):
    from partgs_gb300.batched import MultiViewRasterizer
    scene, cams = setup
    V = len(cams)
    g = torch.Generator().manual_seed(5)
    dcol = torch.randn(V, 3, 72, 88, generator=g).cuda()
    doth = (torch.randn(V, 7, 72, 88, generator=g) * 0.1).cuda()
    ref_img, ref_map, ref_radii, ref_g = _per_view(scene, cams, dcol, doth)
    sc = scene.to("cuda")
    m = sc.means3D.clone().requires_grad_(True)
    mv = MultiViewRasterizer(cams, [0.1, 0.1, 0.1], 3, num_surfels=scene.P)
    img, amap, _, radii = mv(m, sc.opacities, sc.shs, sc.scales, sc.rotations)
    ((img * dcol).sum() + (amap * doth).sum()).backward()
    assert torch.equal(img, ref_img) and torch.equal(amap, ref_map) and torch.equal(radii, ref_radii)
    err = float((m.grad - ref_g).abs().max() / ref_g.abs().max())
    assert err < 1e-5, err


def test_uneven_scenes_in_one_call(setup):
    from partgs_gb300.batched import MultiViewRasterizer
    from partgs_gb300.scenes import random_surfels
    _, cams = setup
    a, b = random_surfels(700, seed=41), random_surfels(1300, seed=42)
    sizes, views = [700, 1300], [1, 3]
    both = MultiViewRasterizer(cams, [0, 0, 0], 3, scene_sizes=sizes, scene_views=views)
    cat = lambda f: torch.cat([f(a), f(b)]).cuda()  # noqa: E731
    img, amap, _, radii = both(cat(lambda s: s.means3D), cat(lambda s: s.opacities), cat(lambda s: s.shs),
                               cat(lambda s: s.scales), cat(lambda s: s.rotations))
    ia, ma, _, ra = MultiViewRasterizer(cams[:1], [0, 0, 0], 3, num_surfels=700)(
        *(t.cuda() for t in (a.means3D, a.opacities, a.shs, a.scales, a.rotations)))
    ib, mb, _, rb = MultiViewRasterizer(cams[1:], [0, 0, 0], 3, num_surfels=1300)(
        *(t.cuda() for t in (b.means3D, b.opacities, b.shs, b.scales, b.rotations)))
    assert torch.equal(img, torch.cat([ia, ib])) and torch.equal(amap, torch.cat([ma, mb]))
    assert torch.equal(radii, torch.cat([ra, rb]))


def test_graph_captured_step_matches_eager(setup):
    from partgs_gb300.surfel_step import SurfelTrainer
    scene, cams = setup
    targets = torch.rand(len(cams), 3, 72, 88, generator=torch.Generator().manual_seed(9)).cuda()
    eager = SurfelTrainer(scene, cams)
    losses_e = [float(eager.step(targets).detach()) for _ in range(5)]
    graphed = SurfelTrainer(scene, cams)
    graphed.capture(targets, warmup=3)      # three eager warm-up steps inside
    losses_g = [float(graphed.replay().detach()) for _ in range(2)]
    K, flags, nbins = graphed.raster.counts()
    assert flags == 0 and K > 0 and 0 < nbins <= graphed.raster.bin_capacity
    np.testing.assert_allclose(losses_g, losses_e[3:5], rtol=2e-4)
