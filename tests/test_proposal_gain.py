"""What the trained proposal network gains over the reference's block
initialisation (k-means blocks, identity rotation, fixed size), on seeded
held-out synthetic scenes: the shipped weights (trained on the GPU by the
project's own kernels on block-fit labels, partgs_gb300/train_proposal.py)
propose superquadric sets whose surfaces are closer to the truth, and over
the 32 held-out scenes of the committed time-to-Chamfer record
(profiles/time_to_chamfer_32.json: seed 4242, 300 iterations) the block fit
started from them reaches the plain fit's final Chamfer in most scenes,
in about half the plain fit's time in the median scene.  The benchmark spec's
target, a third of the time, is not met; the test asserts the measured
figures (with margin for the run-to-run spread of the fits), not the
target."""
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


def test_time_to_chamfer_over_the_held_out_scenes(sgr_lib):
    """All 32 scenes count: one whose proposal fit never reaches the plain
    fit's level has ratio infinity.  Measured: 23 of 32 reach it, median
    ratio 0.49 (profiles/time_to_chamfer_32.json)."""
    from partgs_gb300 import sq_data as D
    from partgs_gb300.block_fit import summarize, time_to_chamfer
    from partgs_gb300.train_proposal import load_npz
    net = load_npz(_weights())
    b = D.sample_sq_batch(32, torch.Generator().manual_seed(4242))
    pts, _ = D.SceneRenderer(res=96).points(b, seed=4242)
    res = time_to_chamfer(net, b, pts, iters=300)
    for r in res:
        assert np.isfinite(r["plain_final"]) and r["plain_final"] < r["plain_start"]
    s = summarize(res, 300)
    print({k: v for k, v in s.items() if k != "per_scene"})
    assert s["reached"] >= 19, s["reached"]
    assert s["time_ratio_median_all"] is not None and s["time_ratio_median_all"] <= 0.65, s["time_ratio_median_all"]
    assert s["proposal_start_chamfer"] < s["plain_start_chamfer"]
