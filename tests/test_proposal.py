"""The point-set proposal network on the tensor cores: forward outputs and
every weight / bias gradient against the CPU oracle (same bf16 rounding
points), the synthetic scene renderer, and a short training run whose loss
falls."""
import numpy as np
import pytest
import torch

from oracle import proposal_oracle as O

pytestmark = pytest.mark.gpu

# bf16 activations: a rounding flip of an intermediate moves later values by
# up to ~2^-8 of their size; relative to each tensor's largest magnitude
TOL = 3e-2


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def test_forward_and_gradients_match_oracle(sgr_lib):
    from partgs_gb300.proposal import ProposalNet
    net = ProposalNet(seed=3)
    g = torch.Generator().manual_seed(4)
    pts = (torch.rand(3, 2048, 3, generator=g) * 2 - 1).cuda()
    out, cache = net.forward(pts)
    dout = torch.randn(out.shape, generator=g).cuda()
    net.backward(cache, dout)
    torch.cuda.synchronize()
    W = [w.detach().cpu().numpy() for w in net.W]
    b = [x.detach().cpu().numpy() for x in net.b]
    ref, c = O.forward(W, b, pts.cpu().numpy())
    assert _rel(out.cpu().numpy(), ref) < TOL
    gW, gB = O.backward(c, dout.cpu().numpy().astype(np.float64))
    for i in range(5):
        assert _rel(net.W[i].grad.cpu().numpy(), gW[i]) < TOL, ("W", i)
        assert _rel(net.b[i].grad.cpu().numpy(), gB[i]) < TOL, ("b", i)
    from partgs_gb300 import proposal_gemm as G
    assert int(G.status_word("cuda").item()) == 0


def test_scene_points_lie_on_the_superquadrics(sgr_lib):
    from partgs_gb300 import sq_data as D
    g = torch.Generator().manual_seed(0)
    batch = D.sample_sq_batch(6, g)
    pts, covered = D.SceneRenderer(res=96).points(batch, n_points=2048, seed=1)
    assert pts.shape == (6, 2048, 3) and bool((covered > 50).all())
    for s in range(6):
        k = int(batch.counts[s])
        # dense samples: their own spacing bounds the nearest-neighbour distance
        surf = D.surface_samples(batch.semi[s, :k], batch.eps[s, :k], batch.quat[s, :k], batch.trans[s, :k], 40000,
                                 g).reshape(-1, 3)
        d = torch.cdist(pts[s].cpu(), surf).min(dim=1).values
        assert float(d.median()) < 0.02, (s, float(d.median()))


def test_training_lowers_the_loss(sgr_lib):
    from partgs_gb300 import sq_data as D
    from partgs_gb300.proposal import ProposalNet, Trainer
    g = torch.Generator().manual_seed(0)
    batch = D.sample_sq_batch(256, g)
    pts, _ = D.SceneRenderer(res=96).points(batch, seed=2)
    tr = Trainer(ProposalNet(seed=0), lr=1e-3)
    losses = []
    for it in range(150):
        sel = torch.randint(0, 256, (32,), generator=g)
        sub = D.SQBatch(*(t[sel] for t in (batch.semi, batch.eps, batch.quat, batch.trans, batch.exist)))
        losses.append(float(tr.step(pts[sel.cuda()].contiguous(), sub)))
    assert np.mean(losses[-10:]) < 0.75 * np.mean(losses[:5]), losses
