"""The grid nearest-neighbour search (sgr_nn_search_grid) against the
brute-force scan (sgr_nn_search): the same distances and indices, bit for
bit, on volume and surface point sets, with duplicate points (ties go to the
first index), degenerate boxes (a plane, a single point), queries far
outside the reference box (the brute-force fallback inside the call) and
coordinates far from the origin."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _both(q, r):
    from partgs_gb300 import chamfer_eval as E
    q, r = q.float().cuda(), r.float().cuda()
    db, ib = E.nn_distance(q, r, with_index=True, method="brute")
    dg, ig = E.nn_distance(q, r, with_index=True, method="grid")
    torch.cuda.synchronize()
    return db.cpu().numpy(), ib.cpu().numpy(), dg.cpu().numpy(), ig.cpu().numpy()


def _check(q, r):
    db, ib, dg, ig = _both(q, r)
    np.testing.assert_array_equal(dg, db)
    np.testing.assert_array_equal(ig, ib)
    return db


def _sphere(n, g, radius=1.0, noise=0.0):
    v = torch.randn(n, 3, generator=g, dtype=torch.float64)
    v = v / v.norm(dim=1, keepdim=True) * radius
    return v + noise * torch.randn(n, 3, generator=g, dtype=torch.float64)


def test_volume_points(sgr_lib):
    g = torch.Generator().manual_seed(0)
    _check(torch.rand(20000, 3, generator=g), torch.rand(50000, 3, generator=g))


def test_surface_points_and_far_queries(sgr_lib):
    g = torch.Generator().manual_seed(1)
    r = _sphere(80000, g, 1.0, 0.002)
    q = torch.cat([_sphere(30000, g, 1.0, 0.01),                     # near the surface
                   torch.rand(2000, 3, generator=g, dtype=torch.float64) * 1.6 - 0.8,   # inside the hollow
                   torch.randn(500, 3, generator=g, dtype=torch.float64) * 20.0])      # far outside the box
    d = _check(q, r)
    ref = torch.cdist(q[-500:], r).min(dim=1).values.numpy()
    np.testing.assert_allclose(d[-500:], ref, rtol=1e-5)


def test_duplicates_and_exact_hits(sgr_lib):
    g = torch.Generator().manual_seed(2)
    base = torch.rand(3000, 3, generator=g)
    r = torch.cat([base, base, base[:500]])[torch.randperm(6500, generator=g)]
    q = torch.cat([base[:1000], torch.rand(4000, 3, generator=g)])
    db, ib, dg, ig = _both(q, r)
    np.testing.assert_array_equal(dg, db)
    np.testing.assert_array_equal(ig, ib)
    assert (db[:1000] == 0).all()
    rn = r.numpy()
    for i in range(0, 1000, 97):                   # the first of the equal points
        hits = np.nonzero((rn == q[i].numpy()).all(1))[0]
        assert ib[i] == hits.min()


def test_degenerate_boxes(sgr_lib):
    g = torch.Generator().manual_seed(3)
    plane = torch.rand(20000, 3, generator=g)
    plane[:, 2] = 0.25
    _check(torch.rand(5000, 3, generator=g), plane)
    line = torch.zeros(4000, 3)
    line[:, 1] = torch.rand(4000, generator=g)
    _check(torch.rand(3000, 3, generator=g), line)
    _check(torch.rand(3000, 3, generator=g), torch.full((7, 3), 0.5))          # one location, seven points
    _check(torch.rand(3000, 3, generator=g), torch.tensor([[0.1, 0.2, 0.3]]))  # one point


def test_far_from_origin(sgr_lib):
    g = torch.Generator().manual_seed(4)
    off = torch.tensor([1500.0, -800.0, 320.0], dtype=torch.float64)
    r = _sphere(40000, g, 5.0, 0.01) + off
    q = _sphere(20000, g, 5.0, 0.05) + off
    _check(q, r)


def test_empty_queries(sgr_lib):
    from partgs_gb300 import chamfer_eval as E
    r = torch.rand(100, 3).cuda()
    assert E.nn_distance(torch.zeros(0, 3).cuda(), r, method="grid").shape == (0,)
    with pytest.raises(ValueError):
        E.nn_distance(r, r, method="kd")
