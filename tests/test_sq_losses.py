"""Fused block-stage superquadric losses against the torch restatement of the
reference (oracle/sq_loss_oracle.py): the SDF, the four losses, and their
gradients to the block parameters against torch autograd (fp32), on a view's
2048 rays x 128 samples and 2048 overlap points per block."""
import math
import time

import numpy as np
import pytest
import torch

from oracle import sq_loss_oracle as O

pytestmark = pytest.mark.gpu

RATIO = 0.25
# Forward values: fp32 rounding of a ~30-op chain (the torch path's batched
# matmul sums in another order).  Gradients: relative to each tensor's largest
# entry; a ray whose two best samples are within rounding of each other may
# pick the other one, moving its single-point contribution slightly.
RTOL_F = 2e-5
RTOL_G = 2e-4


def _quat_to_R(q):
    q = q / q.norm(dim=-1, keepdim=True)
    w, x, y, z = q.unbind(-1)
    return torch.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
                        2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
                        2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1).reshape(-1, 3, 3)


def _blocks(n, seed=0, eps_range=(0.2, 1.8)):
    g = torch.Generator().manual_seed(seed)
    S = torch.rand(n, 3, generator=g) * 1.2 + 0.4
    R = _quat_to_R(torch.randn(n, 4, generator=g))
    T = torch.randn(n, 3, generator=g)
    T = T / T.norm(dim=-1, keepdim=True) * torch.rand(n, 1, generator=g) * 0.3
    lo, hi = eps_range
    e1 = torch.rand(n, generator=g) * (hi - lo) + lo
    e2 = torch.rand(n, generator=g) * (hi - lo) + lo
    occ = torch.randn(n, generator=g) * 0.5 + 2.5   # opaque enough for the overlap term to be active
    return [t.cuda() for t in (S, R, T, e1, e2, occ)]


def _rays(seed=0, n_rays=2048, samples=128, label_p=0.5):
    from partgs_gb300 import sq_losses as Q
    from partgs_gb300.cameras import make_camera
    g = torch.Generator(device="cuda").manual_seed(seed)
    th = 0.3 + seed
    Rc = np.array([[math.cos(th), 0, -math.sin(th)], [0, 1, 0], [math.sin(th), 0, math.cos(th)]])
    cam = make_camera(Rc, np.array([0.0, 0.0, 3.0]), math.radians(50), math.radians(40), 300, 400)
    K = Q.intrinsics(300, 400, cam.fovx, cam.fovy)
    mask = (torch.rand(300, 400, device="cuda", generator=g) < label_p).float()
    return Q.cast_rays(K, torch.from_numpy(cam.world_view_transform).cuda(), 300, 400, mask, 2.0, 5.0,
                       num_samples=samples, num_rays=n_rays, generator=g)


def _ovl(n, seed=0, P=2048):
    from partgs_gb300 import sq_losses as Q
    return Q.overlap_samples(n, P, generator=torch.Generator(device="cuda").manual_seed(seed + 100))


def _oracle(params, rays, ovl):
    out = []
    if rays is not None:
        out += list(O.ray_losses(*params, RATIO, rays.origin, rays.dirs, rays.jitter, rays.label, rays.near, rays.far))
    else:
        out += [torch.zeros((), device="cuda")] * 3
    if ovl is not None:
        out.append(O.overlap_loss(*params, RATIO, ovl.unit, ovl.noise, ovl.temperature, ovl.max_blocks))
    else:
        out.append(torch.zeros((), device="cuda"))
    return torch.stack(out)


def _close(a, b, rtol):
    scale = max(float(b.abs().max()), 1e-12)
    err = float((a - b).abs().max())
    assert err <= rtol * scale, f"max err {err:.3e} vs scale {scale:.3e}"


def test_sdf_matches_torch(sgr_lib):
    from partgs_gb300 import sq_losses as Q
    S, R, T, e1, e2, _ = _blocks(8)
    pts = (torch.rand(50000, 3, generator=torch.Generator().manual_seed(1)) * 4 - 2).cuda()
    got = Q.implicit_sq(pts, S, R, T, e1, e2, RATIO)
    ref = O.implicit_sq(O.to_block_frames(pts, S, R, T, RATIO), e1[:, None], e2[:, None])
    # sdf = (...)^(eps1/2) - 1: the fp32 rounding is relative to sdf + 1, the
    # value the power chain produces before the subtraction
    rel = ((got - ref).abs() / (ref + 1).abs()).max()
    assert float(rel) < 2e-6


@pytest.mark.parametrize("n,seed,eps_range", [(8, 0, (0.2, 1.8)), (16, 1, (0.2, 1.8)), (1, 2, (0.2, 1.8)),
                                              (5, 3, (0.1, 0.15)), (5, 4, (1.85, 1.9))])
def test_losses_and_gradients_match_autograd(sgr_lib, n, seed, eps_range):
    from partgs_gb300 import sq_losses as Q
    params = _blocks(n, seed, eps_range)
    rays, ovl = _rays(seed), _ovl(n, seed)
    w = torch.tensor([10.0, 100.0, 0.02, 2.0], device="cuda")
    p1 = [t.clone().requires_grad_(True) for t in params]
    got = Q.sq_losses(*p1, RATIO, rays, ovl)
    (w * got).sum().backward()
    p2 = [t.clone().requires_grad_(True) for t in params]
    ref = _oracle(p2, rays, ovl)
    (w * ref).sum().backward()
    _close(got.detach(), ref.detach(), RTOL_F)
    assert n == 1 or float(got[3].detach()) > 0, "overlap term active"
    for name, a, b in zip(("S", "R", "T", "eps1", "eps2", "occ"), p1, p2):
        assert a.grad is not None and torch.isfinite(a.grad).all(), name
        _close(a.grad, b.grad, RTOL_G)


def test_terms_separately_and_empty_mask(sgr_lib):
    from partgs_gb300 import sq_losses as Q
    params = _blocks(6, 5)
    rays = _rays(5, n_rays=512, samples=64, label_p=0.0)   # no ray inside the mask: ray_in_mask is NaN, as in torch
    got = Q.sq_losses(*params, RATIO, rays, None)
    ref = _oracle(params, rays, None)
    assert torch.isnan(got[0]) and torch.isnan(ref[0])
    _close(got[1:], ref[1:], RTOL_F)
    ovl = _ovl(6, 5, P=1000)
    got = Q.sq_losses(*params, RATIO, None, ovl)
    ref = _oracle(params, None, ovl)
    _close(got, ref, RTOL_F)
    assert float(got[:3].abs().sum()) == 0.0


def test_deterministic(sgr_lib):
    from partgs_gb300 import sq_losses as Q
    params = _blocks(8, 6)
    rays, ovl = _rays(6), _ovl(8, 6)
    outs = []
    for _ in range(2):
        p = [t.clone().requires_grad_(True) for t in params]
        loss = Q.sq_losses(*p, RATIO, rays, ovl)
        loss.sum().backward()
        outs.append([loss.detach()] + [t.grad for t in p])
    for a, b in zip(*outs):
        assert torch.equal(a, b)


def test_fused_is_faster_than_the_torch_path(sgr_lib):
    """One view's losses and gradients, 16 blocks: the fused kernels against
    the reference's torch formulation (printed; the fused path must win)."""
    from partgs_gb300 import sq_losses as Q
    params = _blocks(16, 7)
    rays, ovl = _rays(7), _ovl(16, 7)

    def run(fn):
        p = [t.clone().requires_grad_(True) for t in params]
        fn(p).sum().backward()

    fused = lambda p: Q.sq_losses(*p, RATIO, rays, ovl)  # noqa: E731
    torch_path = lambda p: _oracle(p, rays, ovl)  # noqa: E731
    times = {}
    for name, fn in (("fused", fused), ("torch", torch_path)):
        for _ in range(3):
            run(fn)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(20):
            run(fn)
        torch.cuda.synchronize()
        times[name] = (time.perf_counter() - t0) / 20 * 1e3
    print(f"block-stage losses fwd+bwd, 16 blocks, 2048x128 ray samples, 32768 overlap points: "
          f"fused {times['fused']:.3f} ms, torch {times['torch']:.3f} ms")
    assert times["fused"] < times["torch"]


def test_kernels_on_the_reference_fixture(sgr_lib):
    """The fused kernels on the inputs of tests/golden/sq_losses.npz (the
    reference's summarize_losses, float64) in fp32."""
    import os
    from partgs_gb300 import sq_losses as Q
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "sq_losses.npz"))
    t = {k: torch.from_numpy(np.asarray(d[k])) for k in d.files}
    f = lambda k: t[k].float().cuda()  # noqa: E731
    origin, dirs = Q.ray_geometry(f("K"), f("world_view"), int(d["height"]), int(d["width"]), t["ray_idx"].cuda())
    label = f("mask").reshape(-1)[t["ray_idx"].cuda()]
    rays = Q.RaySamples(origin, dirs, f("jitter"), label, float(d["near"]), float(d["far"]))
    ovl = Q.OverlapSamples(f("unit01") * 2 - 1, f("noise"))
    p = [f(k).requires_grad_(True) for k in ("in_S", "in_R", "in_T")]
    e = [f(k)[:, 0].clone().requires_grad_(True) for k in ("in_eps1", "in_eps2", "in_sq_occ")]
    losses = Q.sq_losses(*p, *e, float(d["ratio"]), rays, ovl)
    (f("weights") * losses).sum().backward()
    _close(losses.detach().double().cpu(), torch.from_numpy(d["losses"]), RTOL_F)
    for name, got in zip(("S", "R", "T"), p):
        _close(got.grad.double().cpu(), torch.from_numpy(d[f"grad_{name}"]), RTOL_G)
    for name, got in zip(("eps1", "eps2", "sq_occ"), e):
        _close(got.grad.double().cpu(), torch.from_numpy(d[f"grad_{name}"][:, 0]), RTOL_G)


def test_the_largest_block_count(sgr_lib):
    """SGR_SQ_MAX_BLOCKS (64) blocks: losses and gradients still match."""
    from partgs_gb300 import sq_losses as Q
    n = Q.MAX_BLOCKS
    params = _blocks(n, 8)
    rays, ovl = _rays(8, n_rays=256, samples=32), _ovl(n, 8, P=64)
    w = torch.tensor([10.0, 100.0, 0.02, 2.0], device="cuda")
    p1 = [t.clone().requires_grad_(True) for t in params]
    (w * Q.sq_losses(*p1, RATIO, rays, ovl)).sum().backward()
    p2 = [t.clone().requires_grad_(True) for t in params]
    (w * _oracle(p2, rays, ovl)).sum().backward()
    for a, b in zip(p1, p2):
        _close(a.grad, b.grad, RTOL_G)
    with pytest.raises(ValueError):
        Q.sq_losses(*_blocks(n + 1, 9), RATIO, rays, None)
