"""The batched block-level fit (block_fit.BatchFit: all scenes bound and
rasterised in one multi-scene call) against the single-scene BlockFit it
batches: for each scene of an uneven batch, the same target maps, the same
loss and the same gradients of the block parameters at the start of the
fit (up to the FP32 order of the gradient atomics), and a fit that lowers
every scene's loss."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def _targets(S, seed):
    from partgs_gb300 import sq_data as D
    b = D.sample_sq_batch(S, torch.Generator().manual_seed(seed))
    return [(b.semi[s, :k], b.eps[s, :k], b.quat[s, :k], b.trans[s, :k]) for s, k in enumerate(b.counts.tolist())]


def _plain_inits(targets):
    """Per scene: the generating blocks moved off (a start the fit must work from)."""
    g = torch.Generator().manual_seed(3)
    out = []
    for semi, eps, quat, trans in targets:
        out.append(((semi * (1 + 0.2 * torch.rand(semi.shape, generator=g))).clamp(0.1, 0.5),
                    (eps + 0.2 * torch.randn(eps.shape, generator=g)).clamp(0.2, 1.8), quat,
                    trans + 0.05 * torch.randn(trans.shape, generator=g)))
    return out


def test_batch_matches_single_scene_fits(sgr_lib):
    from partgs_gb300.block_fit import BatchFit, BlockFit
    from partgs_gb300.sq_data import to_binding_params
    targets = _targets(4, 11)
    seeds = [100, 101, 102, 103]
    init = _plain_inits(targets)
    bf = BatchFit(targets, seeds, views=4, res=64)
    raw = [t.detach().clone().requires_grad_(True) for t in bf.raw(init)]
    per_scene = bf.loss(bf.render(*raw))
    per_scene.sum().backward()
    o = 0
    for s, (tgt, sd) in enumerate(zip(targets, seeds)):
        k = tgt[0].shape[0]
        one = BlockFit(tgt, views=4, res=64, seed=sd)
        V = 4
        assert torch.equal(one.mask_t, bf.mask_t[s * V:(s + 1) * V])
        assert float((one.depth_t - bf.depth_t[s * V:(s + 1) * V]).abs().max()) <= 1e-5
        r1 = [t.float().cuda().clone().requires_grad_(True) for t in to_binding_params(*init[s])]
        others = one.render(*r1)
        loss = (others[:, 1] - one.alpha_t).abs().mean() + (one.mask_t * (others[:, 5] - one.depth_t).abs()).mean()
        loss.backward()
        assert abs(float(loss) - float(per_scene[s])) <= 1e-5 * max(1.0, abs(float(loss)))
        for a, b in zip(r1, raw):
            ga, gb = a.grad, b.grad[o:o + k]
            assert float((ga - gb).norm()) <= 1e-3 * float(ga.norm()) + 1e-7, (s, ga, gb)
        o += k


def test_batch_fit_lowers_every_scene_loss(sgr_lib):
    from partgs_gb300.block_fit import BatchFit
    targets = _targets(6, 12)
    init = _plain_inits(targets)
    bf = BatchFit(targets, list(range(6)), views=4, res=64)
    with torch.no_grad():
        start = bf.loss(bf.render(*bf.raw(init)))
    fitted, last = bf.fit(init, 40)
    assert bool((last < start).all()), (start, last)
    for (semi, eps, quat, trans), tgt in zip(fitted, targets):
        assert semi.shape == tgt[0].shape and bool((quat[:, 0] >= 0).all())
        assert torch.allclose(quat.norm(dim=-1), torch.ones(quat.shape[0], device=quat.device), atol=1e-5)


def test_captured_fit_equals_eager_fit(sgr_lib):
    """The graph-captured fit (an eager first iteration sizing the cell
    lists, then replays) ends where the eager fit ends, up to the order of
    the gradient atomics."""
    from partgs_gb300.block_fit import BatchFit
    targets = _targets(5, 13)
    init = _plain_inits(targets)
    bf = BatchFit(targets, list(range(5)), views=4, res=64)
    eager, l_e = bf.fit(init, 30)
    graphed, l_g = bf.fit(init, 30, capture=True)
    assert torch.allclose(l_e, l_g, rtol=1e-2, atol=1e-5), (l_e, l_g)
    # Adam moves an element by about lr whatever its gradient's size, so an
    # element whose gradient is at the atomics' noise level may drift; the
    # bulk must agree
    d = torch.cat([(x - y).abs().reshape(-1) for a, b in zip(eager, graphed) for x, y in zip(a, b)])
    assert float(d.median()) <= 1e-4 and float(d.max()) <= 0.1, (float(d.median()), float(d.max()))
