"""Every superquadric parameter's gradient through the CUDA binding and
rasteriser (``sgr_bind_backward`` after ``sgr_backward``, FP32) against
float64 central finite differences of the oracle chain, on the block-level
workload's layout: 8 superquadrics x 2,500 surfels (50 x 50 grid), cameras
400x300 at fovx 50 deg on a radius-3 sphere (two of the eight views, to
bound the oracle's time), the loss a fixed weighted sum of colour and all
seven auxiliary maps.

All 104 parameters: sq_s (3), sq_r (4), sq_t (3), sq_eps (2: the exponents
through signed_pow, games/block_mesh_splatting/utils/pytorch.py:28-29, and
parametric_sq, utils/superquadric.py:10-14) and sq_occ (1), per block.

Pixels whose discrete decisions flip between +h and -h (the oracle's
per-pixel decision signature differs) are left out of both sides for that
parameter; the analytic side is then the gradient of the loss with those
pixels' upstream weights zeroed.  The flip counts are reported.

Bar: |analytic - fd| <= 1e-4 * max(|fd|, 1e-2 * max |fd| over the same
parameter kind): per-parameter relative, floored for parameters whose
derivative is tiny next to its kind's (a quaternion's radial direction has
none at all: the binding normalises it)."""
import numpy as np
import pytest
import torch

from oracle import fd_check as F

pytestmark = pytest.mark.gpu

TOL = 1e-4
FLOOR = 1e-2
H = 1e-6


def _analytic(case, masks=None):
    """Gradients of the five block-parameter tensors (float64 numpy) from the
    CUDA chain; ``masks`` [V,H,W] bool zeroes those pixels' weights."""
    from partgs_gb300.batched import MultiViewRasterizer
    from partgs_gb300.binding import SuperquadricBinding
    inp = case["inp"]
    bind = SuperquadricBinding(inp["eta"].cuda(), inp["omega"].cuda(), inp["faces"].cuda(), inp["alpha_raw"].cuda(),
                               inp["scale"].cuda(), inp["ratio_block_scene"], inp["scale_block_min"])
    P = inp["faces"].shape[0] * inp["faces"].shape[1]
    mv = MultiViewRasterizer(case["cams"], [0, 0, 0], 3, num_surfels=P)
    pc = [inp[k].float().cuda().requires_grad_(True) for k in F.NAMES]
    xyz, ls, rot, op = bind(*pc)
    color, others, _, _ = mv(xyz, op, case["shs"].float().cuda(), torch.exp(ls),
                             torch.nn.functional.normalize(rot))
    wc = torch.tensor(np.stack(case["w_col"]), dtype=torch.float32, device="cuda")
    wo = torch.tensor(np.stack(case["w_oth"]), dtype=torch.float32, device="cuda")
    if masks is not None:
        keep = torch.tensor(~masks, device="cuda")[:, None]
        wc, wo = wc * keep, wo * keep
    ((color * wc).sum() + (others * wo).sum()).backward()
    torch.cuda.synchronize()
    return {k: p.grad.double().cpu().numpy() for k, p in zip(F.NAMES, pc)}


@pytest.fixture(scope="module")
def fd_run(sgr_lib):
    case = F.make_case()
    params = F.parameter_list(case)
    res = F.finite_differences({}, params, h=H)
    return case, res


def test_every_block_parameter_against_fd(fd_run):
    case, res = fd_run
    V, Hh, Ww = len(case["cams"]), case["cams"][0].height, case["cams"][0].width
    base = _analytic(case)
    kind_max = {}
    rows = []
    for r in res:
        if r["flips"]:
            masks = np.zeros((V, Hh * Ww), bool)
            fd = 0.0
            for v, view in enumerate(r["views"]):
                masks[v, view["pixels"][view["flip"]]] = True
                fd += float(view["quotient"][~view["flip"]].sum())
            an = float(_analytic(case, masks.reshape(V, Hh, Ww))[r["name"]].reshape(-1)[r["flat"]])
        else:
            fd = r["fd"]
            an = float(base[r["name"]].reshape(-1)[r["flat"]])
        rows.append((r["name"], r["flat"], an, fd, r["flips"]))
        kind_max[r["name"]] = max(kind_max.get(r["name"], 0.0), abs(fd))
    bad, worst = [], {}
    for name, flat, an, fd, flips in rows:
        den = max(abs(fd), FLOOR * kind_max[name])
        err = abs(an - fd) / den
        worst[name] = max(worst.get(name, 0.0), err)
        if err > TOL:
            bad.append((name, flat, an, fd, flips, err))
    print("worst relative error per kind:", {k: f"{v:.2e}" for k, v in worst.items()})
    print("parameters with decision flips excluded pixel-wise:",
          [(n, f, k) for n, f, _, _, k in rows if k])
    assert len(rows) == 8 * 13
    assert not bad, bad
