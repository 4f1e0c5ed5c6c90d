"""The cell-size autotuner: every candidate edge renders the same images
(the cell lists only change how tiles find their lists), the tuner restores
the parameters it trained through, and picks a candidate."""
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
