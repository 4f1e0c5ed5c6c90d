"""The oracle and the host-side code against golden vectors produced by the
reference's own Python (tests/golden/make_golden.py)."""
import os
import types

import numpy as np
import pytest
import torch

from oracle import binding_oracle as B
from oracle import surfel_oracle as O

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_python.npz"))


@pytest.mark.parametrize("deg", [0, 1, 2, 3])
def test_sh_colour_matches_reference_eval_sh(deg):
    """oracle.sh_to_rgb == clamp(eval_sh + 0.5, 0) (utils/sh_utils.py:36-91)."""
    sh = GOLD["sh_coeffs"].transpose(0, 2, 1)        # [P,16,3]
    dirs = GOLD["sh_dirs"]
    rgb, clamped, _ = O.sh_to_rgb(deg, sh, dirs * 2.5, np.zeros(3))
    ref = GOLD[f"sh_eval_deg{deg}"] + 0.5
    np.testing.assert_allclose(rgb, np.maximum(ref, 0), rtol=1e-12, atol=1e-12)
    np.testing.assert_array_equal(clamped, ref < 0)


def test_camera_matrices_match_reference():
    from partgs_gb300.cameras import make_camera
    for row in GOLD["cameras"]:
        R, T, fov = row[:9].reshape(3, 3), row[9:12], row[12:14]
        cam = make_camera(R, T, fov[0], fov[1], 600, 800)
        np.testing.assert_allclose(cam.world_view_transform, row[14:30].reshape(4, 4), rtol=0, atol=1e-6)
        np.testing.assert_allclose(cam.full_proj_transform, row[30:46].reshape(4, 4), rtol=0, atol=1e-6)
        np.testing.assert_allclose(cam.camera_center, row[46:49], rtol=0, atol=1e-5)


def test_rotation_to_quaternion_matches_reference():
    q = B.rot_to_quat(torch.tensor(GOLD["rot_matrices"])).numpy()
    np.testing.assert_allclose(q, GOLD["rot_quats"], rtol=0, atol=1e-12)


def test_depth_normals_match_reference():
    from partgs_gb300.surfel_step import DepthNormals
    row = GOLD["normal_camera"]
    cam = types.SimpleNamespace(width=32, height=24, world_view_transform=row[14:30].reshape(4, 4).astype(np.float32),
                                full_proj_transform=row[30:46].reshape(4, 4).astype(np.float32))
    dn = DepthNormals([cam], device="cpu")
    n = dn.normals(torch.tensor(GOLD["normal_depth"])[None])[0].permute(1, 2, 0).numpy()
    np.testing.assert_allclose(n, GOLD["normal_out"], rtol=0, atol=2e-4)


@pytest.fixture(scope="module")
def bind_case():
    g = {k[len("bind_in_"):]: torch.tensor(GOLD[k]) for k in GOLD.files if k.startswith("bind_in_")}
    Bn = g["sq_s"].shape[0]
    alpha = g["alpha"].reshape(-1, g["alpha"].shape[2], 3)
    return g, Bn, alpha


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_binding_forward_matches_reference(bind_case, dtype):
    g, Bn, alpha = bind_case
    out = B.bind(g["sq_s"].to(dtype), g["sq_r"].to(dtype), g["sq_t"].to(dtype), g["sq_eps"].to(dtype),
                 g["sq_occ"].to(dtype), g["eta"].to(dtype), g["omega"].to(dtype), g["faces"], alpha.to(dtype),
                 g["scale"].to(dtype), 0.25, 0.2)
    tol = 2e-5 if dtype == torch.float32 else 2e-5
    for o, k in zip(out, ["xyz", "scaling", "rotation", "opacity"]):
        np.testing.assert_allclose(o.detach().numpy(), GOLD[f"bind_out_{k}"], rtol=tol, atol=tol, err_msg=k)


def test_binding_gradients_match_reference(bind_case):
    g, Bn, alpha = bind_case
    params = {k: g[k].clone().double().requires_grad_(True) for k in ["sq_s", "sq_r", "sq_t", "sq_eps", "sq_occ"]}
    out = B.bind(params["sq_s"], params["sq_r"], params["sq_t"], params["sq_eps"], params["sq_occ"],
                 g["eta"].double(), g["omega"].double(), g["faces"], alpha.double(), g["scale"].double(), 0.25, 0.2)
    loss = sum((o * torch.tensor(GOLD[f"bind_upstream_{k}"]).double()).sum()
               for o, k in zip(out, ["xyz", "scaling", "rotation", "opacity"]))
    loss.backward()
    for k, p in params.items():
        ref = GOLD[f"bind_grad_{k}"]
        err = np.abs(p.grad.numpy() - ref).max() / max(1e-6, np.abs(ref).max())
        assert err < 2e-4, (k, err)


ICO = np.load(os.path.join(os.path.dirname(__file__), "golden", "bind_icosphere.npz"))


def _ico_inputs(dtype):
    g = {k[len("in_"):]: torch.tensor(ICO[k]) for k in ICO.files if k.startswith("in_")}
    alpha = g["alpha"].reshape(-1, g["alpha"].shape[2], 3)
    return g, alpha.to(dtype)


@pytest.mark.parametrize("dtype,tol", [(torch.float32, 1e-6), (torch.float64, 2e-5)])
def test_binding_on_the_icosphere_matches_reference(dtype, tol):
    """The block model's own topology type: a level-2 icosphere (162
    vertices, 320 faces, vertices at both poles, where cos(eta) is a float32
    rounding residue), 3 splats per face (tests/golden/bind_icosphere.npz)."""
    g, alpha = _ico_inputs(dtype)
    assert int((np.abs(ICO["in_eta"]) > 1.5707).sum()) >= 2                 # the poles
    out = B.bind(*(g[k].to(dtype) for k in ("sq_s", "sq_r", "sq_t", "sq_eps", "sq_occ", "eta", "omega")), g["faces"],
                 alpha, g["scale"].to(dtype), 0.25, 0.2)
    for o, k in zip(out, ["xyz", "scaling", "rotation", "opacity"]):
        np.testing.assert_allclose(o.detach().numpy(), ICO[f"out_{k}"], rtol=tol, atol=tol, err_msg=k)


def test_binding_gradients_on_the_icosphere_match_reference():
    g, alpha = _ico_inputs(torch.float64)
    params = {k: g[k].clone().double().requires_grad_(True) for k in ["sq_s", "sq_r", "sq_t", "sq_eps", "sq_occ"]}
    out = B.bind(params["sq_s"], params["sq_r"], params["sq_t"], params["sq_eps"], params["sq_occ"],
                 g["eta"].double(), g["omega"].double(), g["faces"], alpha, g["scale"].double(), 0.25, 0.2)
    loss = sum((o * torch.tensor(ICO[f"upstream_{k}"]).double()).sum()
               for o, k in zip(out, ["xyz", "scaling", "rotation", "opacity"]))
    loss.backward()
    for k, p in params.items():
        ref = ICO[f"grad_{k}"]
        err = np.abs(p.grad.numpy() - ref).max() / max(1e-6, np.abs(ref).max())
        assert err < 2e-4, (k, err)
