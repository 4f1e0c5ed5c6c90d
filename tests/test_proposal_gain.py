"""What the trained proposal network gains over the reference's block
initialisation (k-means blocks, identity rotation, fixed size), on seeded
held-out synthetic scenes: the shipped weights (trained on the GPU by the
project's own kernels, partgs_gb300/train_proposal.py) propose
superquadric sets whose surfaces are closer to the truth, and block fits
started from them reach the plain fit's final Chamfer distance sooner."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _weights():
    from partgs_gb300.train_proposal import WEIGHTS
    if not os.path.exists(WEIGHTS):
        pytest.fail(f"trained proposal weights missing: {WEIGHTS}")
    return WEIGHTS


def test_proposal_init_is_closer_than_the_plain_init(sgr_lib):
    from partgs_gb300 import sq_data as D
    from partgs_gb300.proposal import plain_init, predict, set_chamfer
    from partgs_gb300.train_proposal import load_npz
    net = load_npz(_weights())
    b = D.sample_sq_batch(64, torch.Generator().manual_seed(2024))
    pts, _ = D.SceneRenderer(res=96).points(b, seed=2024)
    pred = predict(net, pts, counts=b.counts.tolist())
    cp, cn = [], []
    for s in range(64):
        k = int(b.counts[s])
        tgt = (b.semi[s, :k], b.eps[s, :k], b.quat[s, :k], b.trans[s, :k])
        cp.append(set_chamfer(pred[s], *tgt))
        cn.append(set_chamfer(plain_init(pts[s].float(), k, g=torch.Generator().manual_seed(s)), *tgt))
    cp, cn = np.array(cp), np.array(cn)
    assert cp.mean() < cn.mean(), (cp.mean(), cn.mean())
    assert (cp < cn).mean() >= 0.6, (cp < cn).mean()


def test_block_fit_from_the_proposal_reaches_the_plain_fit_sooner(sgr_lib):
    from partgs_gb300 import sq_data as D
    from partgs_gb300.block_fit import time_to_chamfer
    from partgs_gb300.train_proposal import load_npz
    net = load_npz(_weights())
    b = D.sample_sq_batch(6, torch.Generator().manual_seed(77))
    pts, _ = D.SceneRenderer(res=96).points(b, seed=77)
    res = time_to_chamfer(net, b, pts, iters=150)
    for r in res:
        assert np.isfinite(r["plain_final"]) and r["plain_final"] < r["plain_start"]
    reached = [r for r in res if r["proposal_time"] is not None]
    assert len(reached) >= 4, res
    ratio = np.median([r["proposal_time"] / r["plain_time"] for r in reached])
    assert ratio < 1.0, res
