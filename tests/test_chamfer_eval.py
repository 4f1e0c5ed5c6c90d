"""GPU Chamfer evaluation against the CPU restatement of the reference's
evaluate_mesh: the same mesh samples, the same downsample (exact greedy
order), the same nearest-neighbour distances and scores.  The mesh is a
bound superquadric surface; the ground truth is a jittered sample of it."""
import math

import numpy as np
import pytest
import torch

from oracle import chamfer_oracle as O

pytestmark = pytest.mark.gpu


def _case(seed=0):
    from partgs_gb300 import sq_data as D
    g = torch.Generator().manual_seed(seed)
    eta, omega, faces = D.grid_topology(40, 40)
    e1, e2 = 0.6, 1.3
    sp = lambda t, e: np.sign(t) * np.abs(t) ** e  # noqa: E731
    v = np.stack([sp(np.cos(eta), e1) * sp(np.sin(omega), e2), sp(np.sin(eta), e1),
                  sp(np.cos(eta), e1) * sp(np.cos(omega), e2)], -1) * np.array([0.3, 0.2, 0.25])
    semi = torch.tensor([[0.3, 0.2, 0.25]])
    gt = D.surface_samples(semi, torch.tensor([[e1, e2]]), torch.tensor([[1.0, 0, 0, 0]]), torch.zeros(1, 3), 20000,
                           g).reshape(-1, 3)
    gt = gt + 0.002 * torch.randn(gt.shape, generator=g)
    return v, faces, gt.numpy()


def test_samples_downsample_and_scores_match_the_oracle(sgr_lib):
    from partgs_gb300 import chamfer_eval as E
    verts, faces, gt = _case()
    density = O.DOWNSAMPLE_DENSITY
    pcd = E.sample_mesh(verts, faces, density)
    ref_pcd = O.sample_mesh(verts, faces, density)
    assert pcd.shape[0] == ref_pcd.shape[0]
    np.testing.assert_allclose(pcd.cpu().numpy(), ref_pcd, rtol=0, atol=1e-12)
    perm = torch.randperm(pcd.shape[0], generator=torch.Generator().manual_seed(3))
    acc, comp, avg, ref_shuffled, ref_mask = O.evaluate(verts, faces, gt, perm.numpy(), density=density)
    keep, rounds = E.radius_downsample(pcd[perm.cuda()], density)
    np.testing.assert_array_equal(keep.cpu().numpy(), ref_mask)
    assert rounds < 200
    d = E.nn_distance(pcd[perm.cuda()], torch.from_numpy(gt).cuda())
    from scipy.spatial import cKDTree
    ref_d, _ = cKDTree(gt).query(ref_shuffled, k=1)
    np.testing.assert_allclose(d.cpu().numpy(), ref_d, rtol=1e-5, atol=1e-6)
    a2, c2, v2 = E.evaluate(verts, faces, gt, density=density, seed=3)
    assert math.isclose(a2, acc, rel_tol=1e-5) and math.isclose(c2, comp, rel_tol=1e-5)
    assert math.isclose(v2, avg, rel_tol=1e-5)


def test_nn_indices_and_empty_inputs(sgr_lib):
    from partgs_gb300 import chamfer_eval as E
    g = torch.Generator().manual_seed(1)
    q, r = torch.rand(3001, 3, generator=g), torch.rand(5003, 3, generator=g)
    d, i = E.nn_distance(q.cuda(), r.cuda(), with_index=True)
    ref = torch.cdist(q.double(), r.double())
    np.testing.assert_allclose(d.cpu().numpy(), ref.min(dim=1).values.numpy(), rtol=1e-5, atol=1e-7)
    picked = ref.gather(1, i.long().cpu()[:, None])[:, 0]
    np.testing.assert_allclose(picked.numpy(), ref.min(dim=1).values.numpy(), rtol=1e-5, atol=1e-7)
    assert E.nn_distance(torch.zeros(0, 3).cuda(), r.cuda()).shape == (0,)


def test_downsample_duplicates_and_single_points(sgr_lib):
    """Exact duplicates (distance 0): only the first of each is kept; one
    point is kept; points exactly one radius apart remove each other, as the
    reference's inclusive radius test does."""
    from partgs_gb300 import chamfer_eval as E
    g = torch.Generator().manual_seed(4)
    base = torch.rand(500, 3, generator=g, dtype=torch.float64)
    pts = torch.cat([base, base[:100]], 0)[torch.randperm(600, generator=g)]
    keep, _ = E.radius_downsample(pts.cuda(), 1e-5)
    ref = O.downsample_mask(pts.numpy(), 1e-5)
    np.testing.assert_array_equal(keep.cpu().numpy(), ref)
    assert int(keep.sum()) == 500
    one, rounds = E.radius_downsample(torch.zeros(1, 3, dtype=torch.float64).cuda(), 0.005)
    assert bool(one[0]) and rounds == 1
    line = torch.tensor([[0.0, 0, 0], [0.25, 0, 0], [0.5, 0, 0]], dtype=torch.float64)
    keep, _ = E.radius_downsample(line.cuda(), 0.25)
    np.testing.assert_array_equal(keep.cpu().numpy(), O.downsample_mask(line.numpy(), 0.25))
    assert keep.tolist() == [True, False, True]
