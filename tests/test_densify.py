"""Densification and PLY interchange against the reference's own
TwoGaussianModel / GaussianModel (tests/golden/densify.npz, made by
tests/golden/make_golden.py): the statistics, clone / split / prune with the
optimiser moments, reset_opacity, and the PLY attribute layout."""
import os

import numpy as np
import pytest
import torch

from oracle import densify_oracle as O
from partgs_gb300 import densify as D
from partgs_gb300 import ply

GOLD = os.path.join(os.path.dirname(__file__), "golden", "densify.npz")


def _gold():
    return np.load(GOLD)


def _params(d, device="cpu"):
    return {k: torch.from_numpy(d[f"in_{k}"]).to(device) for k in D.NAMES}


def _adam(d, device="cpu"):
    return {k: (torch.from_numpy(d[f"in_m_{k}"]).to(device), torch.from_numpy(d[f"in_v_{k}"]).to(device))
            for k in D.NAMES}


def test_stats_oracle_matches_the_reference():
    d = _gold()
    radii, g = d["stats_radii"], d["stats_grad"]
    V, P = radii.shape
    scenes = [(0, P, 0, V)]
    views = [(0, v * P) for v in range(V)]
    mr, acc, den = O.stats(scenes, views, radii.reshape(-1), g.reshape(-1, 3), np.zeros(P, np.float32),
                           np.zeros((P, 1), np.float32)[:, 0], np.zeros(P, np.float32))
    np.testing.assert_array_equal(mr, d["stats_max_radii"])
    np.testing.assert_array_equal(den, d["stats_denom"][:, 0])
    np.testing.assert_allclose(acc, d["stats_accum"][:, 0], rtol=1e-6)


def _densify(d, device):
    thr, min_op, extent, screen, pd = d["densify_args"]
    stats = D.DensifyStats(d["in_xyz"].shape[0], device)
    stats.grad_accum.copy_(torch.from_numpy(d["stats_accum"]))
    stats.denom.copy_(torch.from_numpy(d["stats_denom"]))
    stats.max_radii2D.copy_(torch.from_numpy(d["stats_max_radii"]))
    return D.densify_and_prune(_params(d, device), stats, float(thr), float(min_op), float(extent), float(screen),
                               float(pd), semantic=torch.from_numpy(d["in_semantic"]).to(device),
                               adam=_adam(d, device), split_samples=torch.from_numpy(d["split_samples"]))


def _check_densified(d, params, semantic, adam, stats):
    for k in D.NAMES:
        assert params[k].shape == d[f"out_{k}"].shape, k
        np.testing.assert_allclose(params[k].cpu().numpy(), d[f"out_{k}"], rtol=1e-6, atol=1e-7, err_msg=k)
        np.testing.assert_array_equal(adam[k][0].cpu().numpy(), d[f"out_m_{k}"], err_msg=k)
        np.testing.assert_array_equal(adam[k][1].cpu().numpy(), d[f"out_v_{k}"], err_msg=k)
    np.testing.assert_array_equal(semantic.cpu().numpy(), d["out_semantic"])
    assert stats.num_surfels == d["out_xyz"].shape[0] and float(stats.denom.abs().sum()) == 0


def test_densify_and_prune_matches_the_reference_on_cpu_tensors():
    d = _gold()
    _check_densified(d, *_densify(d, "cpu"))


def test_reset_opacity_matches_the_reference():
    d = _gold()
    params = {k: torch.from_numpy(d[f"out_{k}"]) for k in D.NAMES}
    adam = {k: (torch.from_numpy(d[f"out_m_{k}"]), torch.from_numpy(d[f"out_v_{k}"])) for k in D.NAMES}
    params, adam = D.reset_opacity(params, adam)
    np.testing.assert_allclose(params["opacity"].numpy(), d["reset_opacity"], rtol=1e-6, atol=1e-6)
    np.testing.assert_array_equal(adam["opacity"][0].numpy(), d["reset_m_opacity"])


def test_ply_layout_matches_the_reference(tmp_path):
    d = _gold()
    P = 7
    assert ply.attribute_names(45, 2, 4, 4) == list(d["ply_attrs_two"])
    assert ply.attribute_names(45, 2, 4, 0) == list(d["ply_attrs_plain"])
    g = torch.Generator().manual_seed(0)
    t = dict(xyz=torch.randn(P, 3, generator=g), f_dc=torch.randn(P, 1, 3, generator=g),
             f_rest=torch.randn(P, 15, 3, generator=g), opacity=torch.randn(P, 1, generator=g),
             scaling=torch.randn(P, 2, generator=g), rotation=torch.randn(P, 4, generator=g))
    sem = torch.rand(P, 4, generator=g)
    path = tmp_path / "point_cloud.ply"
    ply.save_ply(path, **t, semantic=sem)
    raw = open(path, "rb").read()
    head, body = raw.split(b"end_header\n", 1)
    names = [ln.split()[-1].decode() for ln in head.split(b"\n") if ln.startswith(b"property")]
    assert names == list(d["ply_attrs_two"])
    assert len(body) == P * 65 * 4
    rows = np.frombuffer(body, "<f4").reshape(P, 65)
    # f_rest is channel-major: f_rest_0..14 are the 15 red coefficients
    np.testing.assert_array_equal(rows[:, 9:24], t["f_rest"][:, :, 0].numpy())
    back = ply.load_ply(path, sh_degree=3)
    for k, v in t.items():
        assert torch.equal(back[k], v), k
    assert torch.equal(back["semantic"], sem)


def test_ply_reads_ascii_and_big_endian(tmp_path):
    names = ply.attribute_names(0, 2, 4)
    P = 3
    vals = np.arange(P * len(names), dtype=np.float32).reshape(P, -1) / 7
    head = ["ply", "", "comment made by hand", f"element vertex {P}"] + [f"property float {n}" for n in names] + \
        ["element face 2", "property list uchar int vertex_indices", "end_header"]
    a = tmp_path / "a.ply"
    head[1] = "format ascii 1.0"
    a.write_text("\n".join(head) + "\n" + "\n".join(" ".join(repr(float(x)) for x in r) for r in vals) +
                 "\n3 0 1 2\n3 0 2 1\n")
    b = tmp_path / "b.ply"
    head[1] = "format binary_big_endian 1.0"
    b.write_bytes(("\n".join(head[:-3] + ["end_header"]) + "\n").encode() + vals.astype(">f4").tobytes())
    for p in (a, b):
        got = ply.load_ply(p, sh_degree=0)
        np.testing.assert_allclose(got["xyz"].numpy(), vals[:, :3], rtol=1e-7)
        np.testing.assert_allclose(got["rotation"].numpy(), vals[:, -4:], rtol=1e-7)


@pytest.mark.gpu
def test_stats_kernel_matches_the_oracle_on_a_multi_scene_batch(sgr_lib):
    from partgs_gb300 import _lib as L
    g = torch.Generator().manual_seed(3)
    sizes, nviews = [1000, 37, 4096], [3, 1, 5]
    scenes, views, so, vo, ro = [], [], 0, 0, 0
    for n, nv in zip(sizes, nviews):
        scenes.append((so, n, vo, nv))
        for _ in range(nv):
            views.append((len(scenes) - 1, ro))
            ro += n
            vo += 1
        so += n
    P, Rn = so, ro
    sct = torch.frombuffer(bytearray(bytes((L.SceneDesc * len(scenes))(*[L.SceneDesc(*s) for s in scenes]))),
                           dtype=torch.uint8).cuda()
    vwt = torch.frombuffer(bytearray(bytes((L.ViewDesc * len(views))(*[L.ViewDesc(s, r, 0.5, 0.5)
                                                                          for s, r in views]))),
                           dtype=torch.uint8).cuda()
    radii = ((torch.rand(Rn, generator=g) * 40).int() * (torch.rand(Rn, generator=g) < 0.6).int())
    grads = torch.randn(Rn, 3, generator=g) * 1e-3
    stats = D.DensifyStats(P)
    stats.max_radii2D.fill_(5.0)
    for step in range(2):
        stats.update((sct, vwt, len(scenes), Rn), radii.cuda(), grads.cuda(), grad_scale=2.0)
    mr, acc, den = np.full(P, 5.0, np.float32), np.zeros(P, np.float32), np.zeros(P, np.float32)
    for _ in range(2):
        mr, acc, den = O.stats(scenes, views, radii.numpy(), grads.numpy(), mr, acc, den, grad_scale=2.0)
    np.testing.assert_array_equal(stats.max_radii2D.cpu().numpy(), mr)
    np.testing.assert_array_equal(stats.denom.cpu().numpy()[:, 0], den)
    np.testing.assert_allclose(stats.grad_accum.cpu().numpy()[:, 0], acc, rtol=2e-6)


@pytest.mark.gpu
def test_densify_and_prune_on_the_device(sgr_lib):
    d = _gold()
    params, semantic, adam, stats = _densify(d, "cuda")
    assert params["xyz"].is_cuda
    _check_densified(d, params, semantic, adam, stats)


@pytest.mark.gpu
def test_trainer_gathers_statistics_and_densifies(sgr_lib):
    """The statistics ride along in every training step (eager and in the
    captured graph); densify_and_prune then resizes the trainer, and a new
    capture trains the new surfels."""
    from partgs_gb300.cameras import orbit_cameras
    from partgs_gb300.scenes import random_surfels
    from partgs_gb300.surfel_step import SurfelTrainer
    scene, cams = random_surfels(3000, seed=5), orbit_cameras(3, 3.0, 64, 80, 55.0, seed=2)
    targets = torch.rand(len(cams), 3, 64, 80, generator=torch.Generator().manual_seed(4)).cuda()
    tr = SurfelTrainer(scene, cams, densify_stats=True)
    V, P = len(cams), scene.P
    mr, acc, den = np.zeros(P, np.float32), np.zeros(P, np.float32), np.zeros(P, np.float32)
    scenes, views = [(0, P, 0, V)], [(0, v * P) for v in range(V)]
    for _ in range(2):
        tr.step(targets)
        torch.cuda.synchronize()
        mr, acc, den = O.stats(scenes, views, tr._radii.cpu().numpy(), tr.raster.last_means2D_grad.cpu().numpy(),
                               mr, acc, den, grad_scale=float(V))
    np.testing.assert_array_equal(tr.stats.denom.cpu().numpy()[:, 0], den)
    np.testing.assert_array_equal(tr.stats.max_radii2D.cpu().numpy(), mr)
    np.testing.assert_allclose(tr.stats.grad_accum.cpu().numpy()[:, 0], acc, rtol=2e-6)
    assert den.max() == 2 * V
    tr.capture(targets, warmup=1)
    before = tr.stats.denom.clone()
    tr.replay()
    torch.cuda.synchronize()
    assert float((tr.stats.denom - before).max()) == V          # the graph carries the statistics kernel
    grads = (tr.stats.grad_accum / tr.stats.denom).nan_to_num(0)
    thr = float(grads.quantile(0.8))
    n = tr.densify_and_prune(thr, 0.005, 3.0, generator=torch.Generator(device="cuda").manual_seed(0))
    assert n != P and tr.xyz.shape[0] == n and tr.stats.num_surfels == n and tr.graph is None
    tr.capture(targets, warmup=1)
    for _ in range(2):
        loss = tr.replay()
    torch.cuda.synchronize()
    assert torch.isfinite(loss)
    tr.reset_opacity()
    assert float(torch.sigmoid(tr.opacity_logit.detach()).max()) <= 0.01 + 1e-6


def test_densify_with_nothing_selected_and_everything_pruned():
    """High thresholds select nothing: the surfels come back unchanged (the
    reference's clone / split of an empty selection); a min opacity above
    every surfel prunes all of them."""
    d = _gold()
    stats = D.DensifyStats(d["in_xyz"].shape[0], "cpu")
    stats.grad_accum.copy_(torch.from_numpy(d["stats_accum"]))
    stats.denom.copy_(torch.from_numpy(d["stats_denom"]))
    params, sem, adam, st = D.densify_and_prune(_params(d), stats, 1e9, 0.0, 1.5, None, 0.01,
                                                semantic=torch.from_numpy(d["in_semantic"]), adam=_adam(d))
    for k in D.NAMES:
        assert torch.equal(params[k], torch.from_numpy(d[f"in_{k}"])), k
        assert torch.equal(adam[k][0], torch.from_numpy(d[f"in_m_{k}"])), k
    assert st.num_surfels == d["in_xyz"].shape[0]
    params, sem, adam, st = D.densify_and_prune(_params(d), stats, 1e9, 1.1, 1.5, None, 0.01,
                                                semantic=torch.from_numpy(d["in_semantic"]), adam=_adam(d))
    assert all(params[k].shape[0] == 0 for k in D.NAMES) and sem.shape[0] == 0 and st.num_surfels == 0
