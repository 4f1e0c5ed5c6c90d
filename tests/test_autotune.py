"""The launch-shape autotuners: every candidate cell edge, warp footprint,
tile schedule and staged batch renders the same images (they only change
how tiles find their lists, how pixels and tiles are handed to warps and
CTAs, and how many list entries are staged at a time), the tuners restore
the parameters they trained through, and pick a candidate."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_cell_size_does_not_change_the_render(sgr_lib):
    from partgs_gb300.batched import MultiViewRasterizer
    from partgs_gb300.cameras import orbit_cameras
    from partgs_gb300.scenes import random_surfels
    sc = random_surfels(3000, seed=51).to("cuda")
    cams = orbit_cameras(3, 3.0, 96, 160, 55.0, seed=8)
    outs = []
    for edge in (1, 2, 4, 8, 16):
        img, amap, _, radii = MultiViewRasterizer(cams, [0, 0, 0], 3, num_surfels=3000, cell_tiles=edge)(
            sc.means3D, sc.opacities, sc.shs, sc.scales, sc.rotations)
        outs.append((img, amap, radii))
    for img, amap, radii in outs[1:]:
        assert torch.equal(img, outs[0][0]) and torch.equal(amap, outs[0][1]) and torch.equal(radii, outs[0][2])


def test_tuner_picks_a_candidate_and_restores_the_parameters(sgr_lib):
    from partgs_gb300 import autotune
    from partgs_gb300.cameras import orbit_cameras
    from partgs_gb300.scenes import random_surfels
    from partgs_gb300.surfel_step import SurfelTrainer
    scene, cams = random_surfels(2500, seed=31), orbit_cameras(4, 3.0, 72, 88, 55.0, seed=13)
    targets = torch.rand(len(cams), 3, 72, 88, generator=torch.Generator().manual_seed(9)).cuda()
    tr = SurfelTrainer(scene, cams)
    before = [p.detach().clone() for p in tr.params()]
    best = autotune.tune_cells(tr, targets, candidates=(2, 8), steps=2)
    assert best in (2, 8) and tr.raster.cell_tiles == best
    assert set(autotune.tune_cells.last_timings) == {2, 8}
    for p, q in zip(tr.params(), before):
        assert torch.equal(p.detach(), q)


def test_warp_footprint_and_schedule_do_not_change_the_results(sgr_lib):
    """Both warp footprints, both tile schedules and both staged batches:
    identical images and radii (every pixel walks the same list with the same
    arithmetic), and gradients equal up to the order of the float atomics."""
    from partgs_gb300 import _lib as L
    from partgs_gb300.batched import MultiViewRasterizer
    from partgs_gb300.cameras import orbit_cameras
    from partgs_gb300.scenes import random_surfels
    sc = random_surfels(3000, seed=52).to("cuda")
    cams = orbit_cameras(3, 3.0, 96, 160, 55.0, seed=9)
    g = torch.Generator(device="cuda").manual_seed(4)
    up_c = torch.randn(3, 3, 96, 160, device="cuda", generator=g)
    up_o = torch.randn(3, 7, 96, 160, device="cuda", generator=g) * 0.1
    outs = []
    for shape in (L.SGR_BLEND_STRIP16, L.SGR_BLEND_PATCH8):
        for sched in (L.SGR_SCHEDULE_GRID, L.SGR_SCHEDULE_QUEUE):
            for stage in (L.SGR_STAGE_DEFAULT, L.SGR_STAGE_SMALL, L.SGR_STAGE_TINY):
                leaves = [t.clone().requires_grad_(True) for t in (sc.means3D, sc.opacities, sc.shs, sc.scales,
                                                                    sc.rotations)]
                mv = MultiViewRasterizer(cams, [0.1, 0.2, 0.3], 3, num_surfels=3000, blend_shape=shape,
                                         tile_schedule=sched, stage_entries=stage)
                img, amap, _, radii = mv(*leaves)
                ((img * up_c).sum() + (amap * up_o).sum()).backward()
                outs.append((img.detach(), amap.detach(), radii, [t.grad for t in leaves]))
    for img, amap, radii, grads in outs[1:]:
        assert torch.equal(img, outs[0][0]) and torch.equal(amap, outs[0][1]) and torch.equal(radii, outs[0][2])
        for a, b in zip(grads, outs[0][3]):
            assert float((a - b).norm() / b.norm()) < 1e-5


@pytest.mark.parametrize("channels", [5, 16])
def test_part_variant_launch_options_do_not_change_the_results(sgr_lib, channels):
    """The part variant (semantic sums and staged semantics in shared memory
    sized by the channel count and the staged batch): identical images,
    semantics and radii for every footprint, schedule and staged batch;
    gradients equal up to the order of the float atomics."""
    from partgs_gb300 import _lib as L
    from partgs_gb300.batched import MultiViewRasterizer
    from partgs_gb300.cameras import orbit_cameras
    from partgs_gb300.scenes import random_surfels
    sc = random_surfels(3000, seed=53).to("cuda")
    cams = orbit_cameras(2, 3.0, 80, 112, 55.0, seed=10)
    g = torch.Generator(device="cuda").manual_seed(5)
    sem0 = torch.softmax(torch.randn(3000, channels, device="cuda", generator=g) * 2, -1)
    up_c = torch.randn(2, 3, 80, 112, device="cuda", generator=g)
    up_o = torch.randn(2, 8, 80, 112, device="cuda", generator=g) * 0.1
    up_s = torch.randn(2, channels, 80, 112, device="cuda", generator=g)
    outs = []
    for shape in (L.SGR_BLEND_STRIP16, L.SGR_BLEND_PATCH8):
        for sched in (L.SGR_SCHEDULE_GRID, L.SGR_SCHEDULE_QUEUE):
            for stage in (L.SGR_STAGE_DEFAULT, L.SGR_STAGE_SMALL, L.SGR_STAGE_TINY):
                leaves = [t.clone().requires_grad_(True) for t in (sc.means3D, sc.opacities, sc.shs, sc.scales,
                                                                    sc.rotations)]
                sem = sem0.clone().requires_grad_(True)
                mv = MultiViewRasterizer(cams, [0.1, 0.2, 0.3], 3, variant=L.SGR_VARIANT_PART, num_surfels=3000,
                                         blend_shape=shape, tile_schedule=sched, stage_entries=stage)
                img, amap, smap, radii = mv(*leaves, semantics=sem)
                ((img * up_c).sum() + (amap * up_o).sum() + (smap * up_s).sum()).backward()
                outs.append((img.detach(), amap.detach(), smap.detach(), radii, [t.grad for t in leaves + [sem]]))
    for img, amap, smap, radii, grads in outs[1:]:
        assert torch.equal(img, outs[0][0]) and torch.equal(amap, outs[0][1])
        assert torch.equal(smap, outs[0][2]) and torch.equal(radii, outs[0][3])
        for a, b in zip(grads, outs[0][4]):
            assert float((a - b).norm() / b.norm()) < 1e-5


def test_blend_tuner_picks_a_pair(sgr_lib):
    from partgs_gb300 import autotune
    from partgs_gb300.cameras import orbit_cameras
    from partgs_gb300.scenes import random_surfels
    from partgs_gb300.surfel_step import SurfelTrainer
    scene, cams = random_surfels(2500, seed=32), orbit_cameras(4, 3.0, 72, 88, 55.0, seed=14)
    targets = torch.rand(len(cams), 3, 72, 88, generator=torch.Generator().manual_seed(10)).cuda()
    tr = SurfelTrainer(scene, cams)
    before = [p.detach().clone() for p in tr.params()]
    best = autotune.tune_blend(tr, targets, steps=2)
    assert best == (tr.raster.blend_shape, tr.raster.tile_schedule, tr.raster.stage_entries)
    assert len(autotune.tune_blend.last_timings) == 12
    for p, q in zip(tr.params(), before):
        assert torch.equal(p.detach(), q)


def test_part_variant_without_semantics_matches_with(sgr_lib):
    """The part variant with no semantic channels (no dynamic shared memory,
    every semantic loop skipped) renders the same colour and auxiliary maps
    as with 5 channels, whose weights do not enter them, for every staged
    batch; gradients of the shared inputs agree up to the order of the float
    atomics."""
    from partgs_gb300 import _lib as L
    from partgs_gb300.batched import MultiViewRasterizer
    from partgs_gb300.cameras import orbit_cameras
    from partgs_gb300.scenes import random_surfels
    sc = random_surfels(3000, seed=54).to("cuda")
    cams = orbit_cameras(2, 3.0, 80, 112, 55.0, seed=11)
    g = torch.Generator(device="cuda").manual_seed(6)
    sem0 = torch.softmax(torch.randn(3000, 5, device="cuda", generator=g) * 2, -1)
    up_c = torch.randn(2, 3, 80, 112, device="cuda", generator=g)
    up_o = torch.randn(2, 8, 80, 112, device="cuda", generator=g) * 0.1
    for stage in (L.SGR_STAGE_DEFAULT, L.SGR_STAGE_SMALL, L.SGR_STAGE_TINY):
        outs = []
        for sem in (None, sem0):
            leaves = [t.clone().requires_grad_(True) for t in (sc.means3D, sc.opacities, sc.shs, sc.scales,
                                                                sc.rotations)]
            mv = MultiViewRasterizer(cams, [0.1, 0.2, 0.3], 3, variant=L.SGR_VARIANT_PART, num_surfels=3000,
                                     tile_schedule=L.SGR_SCHEDULE_QUEUE, stage_entries=stage)
            img, amap, smap, radii = mv(*leaves, semantics=sem)
            assert (smap is None) == (sem is None)
            ((img * up_c).sum() + (amap * up_o).sum()).backward()
            outs.append((img.detach(), amap.detach(), radii, [t.grad for t in leaves]))
        (i0, a0, r0, g0), (i1, a1, r1, g1) = outs
        assert torch.equal(i0, i1) and torch.equal(a0, a1) and torch.equal(r0, r1)
        for a, b in zip(g0, g1):
            assert float((a - b).norm() / b.norm()) < 1e-5
