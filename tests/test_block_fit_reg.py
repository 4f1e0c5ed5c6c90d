"""The block fit with the block model's regularisers (ray coverage and
uncoverage, occupancy, overlap from the fused superquadric-loss kernels):
the block frames follow the reference's parameterisation, and a short fit
runs, keeps every term finite and lowers the Chamfer distance."""
import numpy as np
import pytest
import torch

from oracle import binding_oracle as BO


def test_block_frames_follow_the_binding():
    from partgs_gb300 import sq_losses as Q
    g = torch.Generator().manual_seed(0)
    q = torch.randn(7, 4, generator=g, dtype=torch.float64)
    qn = torch.nn.functional.normalize(q, dim=-1)
    R = Q.quaternion_to_rotation_matrix(qn)
    np.testing.assert_allclose(R.numpy(), BO.quat_to_rotmat(qn).numpy(), rtol=0, atol=1e-14)
    sq_s, sq_t, sq_eps = torch.randn(7, 3, generator=g), torch.randn(7, 3, generator=g), torch.randn(7, 2, generator=g)
    S, R2, T, e1, e2 = Q.block_frames(sq_s, q.float(), sq_t, sq_eps, 0.2)
    torch.testing.assert_close(S, torch.exp(sq_s) + 0.2)
    torch.testing.assert_close(e1, torch.sigmoid(sq_eps[:, 0]) * 1.8 + 0.1)
    torch.testing.assert_close(e2, torch.sigmoid(sq_eps[:, 1]) * 1.8 + 0.1)
    assert T is sq_t


def _reg(fit, params, seed=0):
    """Weighted regulariser sum over every view on fixed rays."""
    from partgs_gb300 import sq_losses as Q
    from partgs_gb300.sq_data import RATIO, SMIN
    sq_s, sq_eps, sq_r, sq_t = params
    S, R, T, e1, e2 = Q.block_frames(sq_s, sq_r, sq_t, sq_eps, SMIN)
    occ = torch.full((sq_s.shape[0],), 4.6, device="cuda")
    g = torch.Generator(device="cuda").manual_seed(seed)
    w = torch.tensor([10.0, 100.0, 0.02, 2.0], device="cuda")
    total, per_view = 0.0, []
    for v, c in enumerate(fit.cams):
        rays = Q.cast_rays(Q.intrinsics(c.height, c.width, c.fovx, c.fovy), torch.as_tensor(c.world_view_transform).cuda(),
                           c.height, c.width, fit.mask_t[v], *Q.NEAR_FAR["blender"], generator=g)
        terms = Q.sq_losses(S, R, T, e1, e2, occ, RATIO, rays, Q.overlap_samples(S.shape[0], generator=g))
        per_view.append(terms)
        total += float((w * terms.nan_to_num(0.0)).sum())
    return total, torch.stack(per_view)


@pytest.mark.gpu
def test_regularised_block_fit(sgr_lib):
    """At the target the rays agree with the rendered silhouettes (rays outside
    the masks miss every block, rays inside rarely do), and the regularised
    fit lowers the weighted regulariser on fixed rays, with finite terms."""
    from partgs_gb300 import sq_data as D
    from partgs_gb300.block_fit import BlockFit
    from partgs_gb300.proposal import plain_init
    b = D.sample_sq_batch(1, torch.Generator().manual_seed(3))
    k = max(2, int(b.counts[0]))
    target = (b.semi[0, :k], b.eps[0, :k], b.quat[0, :k], b.trans[0, :k])
    fit = BlockFit(target, views=4, res=64, seed=1)
    _, at_target = _reg(fit, [t.float().cuda() for t in D.to_binding_params(*target)])
    assert float(at_target[:, 1].max()) < 0.01 and float(at_target[:, 0].max()) < 0.1
    pts = D.surface_samples(*target, 512, torch.Generator().manual_seed(2)).reshape(-1, 3)
    init = plain_init(pts.float().cuda(), k, g=torch.Generator().manual_seed(4))
    before, _ = _reg(fit, [t.float().cuda() for t in D.to_binding_params(*init)])
    hist = fit.fit(init, iters=40, eval_every=20, reg=True)
    assert fit.last_reg is not None and torch.isfinite(fit.last_reg.nan_to_num(0.0)).all()
    assert all(np.isfinite(c) for _, c in hist)
    after, _ = _reg(fit, fit.last_params)
    assert after < before
