"""The one-launch surfel Adam (sgr_adam_step) against torch.optim.Adam with
the reference's settings (eps 1e-15, a learning rate per tensor), over
several steps, for tensor sizes with and without a float4 tail."""
import pytest
import torch

pytestmark = pytest.mark.gpu

# Relative to each tensor's largest total update (the step size is formed in
# FP32 on the device, in double on the host by torch), plus two float ulps of
# the parameter for the rounding of p + update itself.
TOL = 1e-5
ULP = 2 * torch.finfo(torch.float32).eps


def test_surfel_adam_matches_torch(sgr_lib):
    from partgs_gb300.optim import SurfelAdam
    g = torch.Generator().manual_seed(0)
    shapes = [(1000, 3), (1001,), (257, 15, 3), (999, 4)]
    lrs = [1.6e-4, 0.05, 1.25e-4, 0.001]
    init = [torch.randn(s, generator=g) for s in shapes]
    grads = [[torch.randn(s, generator=g) * 10 ** (-k) for k, s in enumerate(shapes)] for _ in range(4)]
    mine = [t.clone().cuda().requires_grad_(True) for t in init]
    ref = [t.clone().cuda().requires_grad_(True) for t in init]
    opt = SurfelAdam([{"params": [p], "lr": lr} for p, lr in zip(mine, lrs)], eps=1e-15)
    topt = torch.optim.Adam([{"params": [p], "lr": lr} for p, lr in zip(ref, lrs)], lr=0.0, eps=1e-15,
                            foreach=False)
    for step in grads:
        with torch.no_grad():
            for p, q, gr in zip(mine, ref, step):
                p.grad.copy_(gr.cuda())
                q.grad = gr.cuda().clone()
        opt.step()
        topt.step()
        torch.cuda.synchronize()
        for p in mine:
            assert float(p.grad.abs().max()) == 0.0          # cleared by the update
    assert float(opt.step_count.item()) == len(grads)
    for p, q, t0 in zip(mine, ref, init):
        moved = float((q.detach().cpu() - t0).abs().max())
        err = float((p.detach() - q.detach()).abs().max().cpu())
        assert err <= TOL * moved + ULP * float(t0.abs().max()), (err, moved)
