"""The fused parameter getters against the PyTorch statement (exp, F.normalize,
sigmoid, cat) and its autograd, including a rotation below normalize's clamp."""
import pytest
import torch
import torch.nn.functional as F

pytestmark = pytest.mark.gpu


def test_activations_match_torch(sgr_lib):
    from partgs_gb300.activations import activate
    g = torch.Generator().manual_seed(0)
    P = 1000
    mk = lambda *s: torch.randn(*s, generator=g).cuda().requires_grad_(True)  # noqa: E731
    ls, rot, op, dc, rest = mk(P, 2), mk(P, 4), mk(P, 1), mk(P, 1, 3), mk(P, 15, 3)
    with torch.no_grad():
        rot[7] = 1e-14                                   # below F.normalize's 1e-12 clamp
    outs = activate(ls, rot, op, dc, rest)
    ref = (torch.exp(ls), F.normalize(rot), torch.sigmoid(op), torch.cat((dc, rest), dim=1))
    for a, b in zip(outs, ref):
        assert a.shape == b.shape and torch.allclose(a, b, rtol=1e-6, atol=1e-7)
    ups = [torch.randn(t.shape, generator=g).cuda() for t in ref]
    mine = torch.autograd.grad(sum((o * u).sum() for o, u in zip(outs, ups)), (ls, rot, op, dc, rest))
    theirs = torch.autograd.grad(sum((o * u).sum() for o, u in zip(ref, ups)), (ls, rot, op, dc, rest))
    for a, b in zip(mine, theirs):
        assert torch.allclose(a, b, rtol=1e-5, atol=1e-6), float((a - b).abs().max())
