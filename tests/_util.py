"""Helpers shared by the parity tests: conversions to the oracle's inputs and
tolerance checks."""
import numpy as np
import torch

from oracle import surfel_oracle as O


def oracle_camera(cam):
    return O.Camera(np.asarray(cam.world_view_transform, np.float32).reshape(-1),
                    np.asarray(cam.full_proj_transform, np.float32).reshape(-1),
                    np.asarray(cam.camera_center, np.float32), cam.tanfovx, cam.tanfovy, cam.height, cam.width)


def oracle_surfels(scene, colors_precomp=None, transmat=None, semantics=None, sh_degree=3, scale_modifier=1.0):
    n = lambda t: None if t is None else t.detach().cpu().numpy()  # noqa: E731
    use_sh = colors_precomp is None
    return O.Surfels(n(scene.means3D), n(scene.opacities),
                     None if transmat is not None else n(scene.scales),
                     None if transmat is not None else n(scene.rotations),
                     shs=n(scene.shs) if use_sh else None, colors_precomp=n(colors_precomp),
                     transmat_precomp=n(transmat), semantics=n(semantics), sh_degree=sh_degree,
                     scale_modifier=scale_modifier)


def settings(mod, cam, bg, sh_degree=3, device="cuda", scale_modifier=1.0, prefiltered=False):
    return mod.GaussianRasterizationSettings(
        image_height=cam.height, image_width=cam.width, tanfovx=cam.tanfovx, tanfovy=cam.tanfovy,
        bg=torch.as_tensor(bg, dtype=torch.float32, device=device), scale_modifier=scale_modifier,
        viewmatrix=torch.as_tensor(cam.world_view_transform, device=device),
        projmatrix=torch.as_tensor(cam.full_proj_transform, device=device), sh_degree=sh_degree,
        campos=torch.as_tensor(cam.camera_center, device=device), prefiltered=prefiltered, debug=False)


def image_error(gpu, ref, mask=None):
    """Per-channel max |gpu - ref| over unmasked pixels, relative to the
    channel's largest magnitude (at least 1)."""
    gpu = np.asarray(gpu, np.float64)
    ref = np.asarray(ref, np.float64)
    out = []
    for c in range(ref.shape[0]):
        d = np.abs(gpu[c] - ref[c])
        if mask is not None:
            d = d[~mask]
        scale = max(1.0, float(np.abs(ref[c]).max()))
        out.append(float(d.max()) / scale if d.size else 0.0)
    return out


def grad_error(gpu, ref):
    """max |gpu - ref| / max |ref| (a tensor-wide relative error)."""
    gpu = np.asarray(gpu, np.float64)
    ref = np.asarray(ref, np.float64)
    scale = float(np.abs(ref).max())
    if scale == 0:
        return float(np.abs(gpu).max())
    return float(np.abs(gpu - ref).max()) / scale
