"""The point-level loss against the reference's own code.

The photometric term: tests/golden/point_loss.npz holds utils/loss_utils.py's l1_loss and
ssim, and train.py:230-231's (1 - lambda_dssim) L1 + lambda_dssim (1 - SSIM)
with its autograd gradient, evaluated one view at a time as the reference's
training loop does (tests/golden/make_golden.py).  The PyTorch statement the
fused loss kernels are checked against (SurfelTrainer.reference_loss, with
the package's ssim) must reproduce it: per view, and for the views batched
as the trainer batches them (the mean over equal-sized views).

The whole loss: tests/golden/render_post.npz holds the reference renderer's
post-processing of given maps and train.py's loss on its outputs (see the
last test).  CPU only."""
import os
import types

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))


def _golden():
    return np.load(os.path.join(HERE, "golden", "point_loss.npz"))


def test_ssim_matches_the_reference_per_view():
    from partgs_gb300.surfel_step import _gaussian_window, ssim
    d = _golden()
    img, gt = torch.from_numpy(d["image"]), torch.from_numpy(d["target"])
    w = _gaussian_window(device="cpu").double()
    for v in range(img.shape[0]):
        s = float(ssim(img[v:v + 1], gt[v:v + 1], w))
        assert abs(s - float(d["ssim"][v])) <= 1e-12, (v, s, float(d["ssim"][v]))
        assert abs(float((img[v] - gt[v]).abs().mean()) - float(d["l1"][v])) <= 1e-15


def test_reference_loss_photometric_term_matches_the_reference():
    from partgs_gb300.surfel_step import SurfelTrainer, _gaussian_window
    d = _golden()
    V, _, H, W = d["image"].shape
    img = torch.from_numpy(d["image"]).clone().requires_grad_(True)
    gt = torch.from_numpy(d["target"])
    # distortion and normal weights 0: the loss is the photometric term alone
    normals = types.SimpleNamespace(view_to_world=torch.eye(3, dtype=torch.float64).expand(V, 3, 3),
                                    normals=lambda depth: torch.zeros(V, 3, H, W, dtype=torch.float64))
    trainer = types.SimpleNamespace(window=_gaussian_window(device="cpu").double(),
                                    lambda_dssim=float(d["lambda_dssim"]), lambda_dist=0.0, lambda_normal=0.0,
                                    depth_ratio=1.0, normals=normals)
    allmap = torch.zeros(V, 7, H, W, dtype=torch.float64)
    loss = SurfelTrainer.reference_loss(trainer, img, allmap, gt)
    loss.backward()
    assert abs(float(loss.detach()) - float(d["loss"].mean())) <= 1e-12
    grad = img.grad.numpy()
    ref = d["grad"] / V
    assert np.abs(grad - ref).max() <= 1e-12 * np.abs(ref).max()


def test_point_loss_on_the_reference_renderers_maps():
    """tests/golden/render_post.npz: the reference's render() post-processing
    (renderer/gaussian_renderer/__init__.py:111-141) of given rasteriser maps
    and train.py:230-249's loss on it (photometric, distortion 1000, normal
    consistency 0.05), per view in float32, at depth ratios 1 and 0.4.  The
    trainer's statement, batched over the views with DepthNormals' precomputed
    rays, gives the mean of the per-view losses and 1/V of each gradient."""
    from partgs_gb300.cameras import orbit_cameras
    from partgs_gb300.surfel_step import DepthNormals, SurfelTrainer, _gaussian_window
    d = np.load(os.path.join(HERE, "golden", "render_post.npz"))
    V, _, H, W = d["image"].shape
    lam, lam_dist, lam_normal = (float(x) for x in d["lambdas"])
    cams = orbit_cameras(V, 3.0, H, W, 55.0, seed=4)
    for tag, ratio in (("r10", 1.0), ("r4", 0.4)):
        trainer = types.SimpleNamespace(window=_gaussian_window(device="cpu"), lambda_dssim=lam, lambda_dist=lam_dist,
                                        lambda_normal=lam_normal, depth_ratio=ratio,
                                        normals=DepthNormals(cams, "cpu"))
        img = torch.from_numpy(d["image"]).clone().requires_grad_(True)
        allmap = torch.from_numpy(d["allmap"]).clone().requires_grad_(True)
        loss = SurfelTrainer.reference_loss(trainer, img, allmap, torch.from_numpy(d["target"]))
        loss.backward()
        ref = float(d[f"{tag}_loss"].mean())
        assert abs(float(loss.detach()) - ref) <= 1e-6 * ref, (tag, float(loss.detach()), ref)
        gi = d[f"{tag}_grad_image"] / V
        assert np.abs(img.grad.numpy() - gi).max() <= 1e-6 * np.abs(gi).max(), tag
        gm = d[f"{tag}_grad_allmap"] / V
        for c in range(gm.shape[1]):
            scale = np.abs(gm[:, c]).max()
            err = np.abs(allmap.grad.numpy()[:, c] - gm[:, c]).max()
            assert err <= 1e-6 * scale if scale > 0 else err == 0, (tag, c, err, scale)
