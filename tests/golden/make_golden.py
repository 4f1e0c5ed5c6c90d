"""Generates tests/golden/reference_python.npz from the reference's own Python.

Run in a checkout that has the PartGS reference next to it (the path is the
first argument, default /root/reference).  It imports, unmodified:

* utils/sh_utils.py            eval_sh (SH colour)
* utils/graphics_utils.py      getWorld2View2, getProjectionMatrix (camera matrices)
* utils/general_utils.py       rot_to_quat_batch (rotation matrix -> quaternion)
* utils/point_utils.py         depth_to_normal (normals from a depth map)
* games/block_mesh_splatting/scene/block_gaussian_model.py
                               update_alpha / get_verts / prepare_scaling_rot / get_opacity
                               (the superquadric -> surfel binding), differentiated by autograd

Packages the reference imports but this path does not use (open3d, trimesh,
pytorch3d, plyfile, simple_knn, PIL, seaborn, matplotlib, iopath) are stubbed
with inert modules, and ``.cuda()`` placements are redirected to the CPU.
The fixtures are small; the tests compare this repository's oracle and
host-side code against them.
"""
from __future__ import annotations

import math
import os
import sys
import types
from unittest import mock

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


STUB_ROOTS = ("open3d", "trimesh", "pytorch3d", "iopath", "PIL", "plyfile", "simple_knn", "seaborn",
              "matplotlib", "toolz", "kornia", "lpips", "cv2", "imageio", "skimage", "tqdm", "torchvision",
              "tensorboard", "mcubes", "pymeshlab", "natsort", "easydict")


class _StubModule(types.ModuleType):
    __path__ = []

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return mock.MagicMock(name=f"{self.__name__}.{name}")


class _StubFinder:
    """Resolves every module under STUB_ROOTS to an inert stub package."""

    def find_spec(self, fullname, path=None, target=None):
        import importlib.machinery
        if fullname.split(".")[0] in STUB_ROOTS:
            return importlib.machinery.ModuleSpec(fullname, self, is_package=True)
        return None

    def create_module(self, spec):
        return _StubModule(spec.name)

    def exec_module(self, module):
        pass


def _stub_modules():
    sys.meta_path.insert(0, _StubFinder())


def _cpu_only():
    """Redirect the reference's .cuda() / device='cuda' to the CPU."""
    torch.Tensor.cuda = lambda self, *a, **k: self
    real_arange, real_tensor = torch.arange, torch.tensor

    def arange(*a, **k):
        k.pop("device", None)
        return real_arange(*a, **k)
    torch.arange = arange


def main(ref_root="/root/reference"):
    sys.path.insert(0, ref_root)
    _stub_modules()
    _cpu_only()
    torch.set_default_dtype(torch.float32)
    from utils.sh_utils import eval_sh
    from utils.graphics_utils import getWorld2View2, getProjectionMatrix
    from utils.general_utils import rot_to_quat_batch
    from utils.point_utils import depth_to_normal
    import games.block_mesh_splatting.scene.block_gaussian_model as bgm
    sys.path.insert(0, ROOT)
    from oracle.binding_oracle import grid_topology

    out = {}
    g = torch.Generator().manual_seed(0)
    # ---- SH: coefficients [P,3,16] as eval_sh takes them, unit directions
    P = 64
    sh = torch.randn(P, 3, 16, generator=g, dtype=torch.float64) * 0.3
    dirs = torch.randn(P, 3, generator=g, dtype=torch.float64)
    dirs = dirs / dirs.norm(dim=1, keepdim=True)
    out["sh_coeffs"] = sh.numpy()
    out["sh_dirs"] = dirs.numpy()
    for d in range(4):
        out[f"sh_eval_deg{d}"] = eval_sh(d, sh, dirs).numpy()

    # ---- cameras: world-to-view and projection for a few poses
    cams = []
    for k in range(4):
        ang = 0.7 * k + 0.3
        c = np.array([3 * math.cos(ang), 3 * math.sin(ang), 0.5 * k - 0.7])
        fwd = -c / np.linalg.norm(c)
        right = np.cross(fwd, [0, 0, 1.0])
        right /= np.linalg.norm(right)
        down = np.cross(fwd, right)
        R = np.stack([right, down, fwd], 1)
        T = -R.T @ c
        fovx = math.radians(50 + 5 * k)
        fovy = 2 * math.atan(math.tan(fovx / 2) * 0.75)
        wv = torch.tensor(getWorld2View2(R, T)).transpose(0, 1)
        pj = getProjectionMatrix(znear=0.01, zfar=100.0, fovX=fovx, fovY=fovy).transpose(0, 1)
        full = wv.unsqueeze(0).bmm(pj.unsqueeze(0)).squeeze(0)
        center = wv.inverse()[3, :3]
        cams.append(np.concatenate([R.reshape(-1), T, [fovx, fovy], wv.numpy().reshape(-1),
                                    full.numpy().reshape(-1), center.numpy()]))
    out["cameras"] = np.stack(cams)   # R(9) T(3) fov(2) world_view(16) full_proj(16) centre(3)

    # ---- rotation matrix -> quaternion (including near-180-degree rotations)
    q = torch.randn(32, 4, generator=g, dtype=torch.float64)
    q[:4, 0] = 1e-3
    q = q / q.norm(dim=1, keepdim=True)
    w, x, y, z = q.unbind(1)
    Rm = torch.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
                      2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
                      2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], 1).reshape(-1, 3, 3)
    out["rot_matrices"] = Rm.numpy()
    out["rot_quats"] = rot_to_quat_batch(Rm).numpy()

    # ---- normals from a depth map (camera 0 at 32x24)
    W, H = 32, 24
    view = types.SimpleNamespace(image_width=W, image_height=H,
                                 world_view_transform=torch.tensor(cams[0][14:30].reshape(4, 4), dtype=torch.float32),
                                 full_proj_transform=torch.tensor(cams[0][30:46].reshape(4, 4), dtype=torch.float32))
    yy, xx = torch.meshgrid(torch.linspace(-1, 1, H), torch.linspace(-1, 1, W), indexing="ij")
    depth = (3.0 + 0.3 * torch.sin(2 * xx) * torch.cos(3 * yy)).reshape(1, H, W).float()
    out["normal_depth"] = depth.numpy()
    out["normal_camera"] = cams[0]
    out["normal_out"] = depth_to_normal(view, depth).numpy()

    # ---- superquadric binding: 2 superquadrics on a 12x12 grid, 2 surfels per triangle
    B, ne, no_, N = 2, 12, 12, 2
    eta, omega, faces = grid_topology(ne, no_)
    Fn = faces.shape[0]
    model = bgm.BlockGaussianModel.__new__(bgm.BlockGaussianModel)
    model.scaling_activation = torch.exp
    model.rotation_activation = torch.nn.functional.normalize
    model.opacity_activation = torch.sigmoid
    model.ratio_block_scene = 0.25
    model.scale_block_min = 0.2
    model.per_gs_num = Fn * N
    sq_s = torch.log(torch.rand(B, 3, generator=g) * 1.6 + 0.2).requires_grad_(True)
    sq_r = torch.randn(B, 4, generator=g).requires_grad_(True)
    sq_t = (torch.rand(B, 3, generator=g) - 0.5).requires_grad_(True)
    sq_eps = (torch.randn(B, 2, generator=g) * 0.8).requires_grad_(True)
    sq_occ = torch.randn(B, 1, generator=g).requires_grad_(True)
    model.sq_s, model.sq_r, model.sq_t, model.sq_eps, model.sq_occ = sq_s, sq_r, sq_t, sq_eps, sq_occ
    model.sq_eta = torch.tensor(eta, dtype=torch.float32).expand(B, -1).contiguous()
    model.sq_omega = torch.tensor(omega, dtype=torch.float32).expand(B, -1).contiguous()
    model.faces = torch.tensor(faces).expand(B, -1, -1).contiguous()
    model._alpha = torch.rand(B, Fn, N, 3, generator=g)
    model._scale = torch.rand(B, Fn * N, 1, generator=g) * 0.5 + 0.5
    model.update_alpha()
    model.prepare_scaling_rot()
    opac = model.get_opacity
    gx = torch.randn(model._xyz.shape, generator=g)
    gs = torch.randn(model._scaling.shape, generator=g)
    gr = torch.randn(model._rotation.shape, generator=g)
    go = torch.randn(opac.shape, generator=g)
    loss = (model._xyz * gx).sum() + (model._scaling * gs).sum() + (model._rotation * gr).sum() + (opac * go).sum()
    loss.backward()
    for k, v in dict(sq_s=sq_s, sq_r=sq_r, sq_t=sq_t, sq_eps=sq_eps, sq_occ=sq_occ).items():
        out[f"bind_in_{k}"] = v.detach().numpy()
        out[f"bind_grad_{k}"] = v.grad.numpy()
    out["bind_in_eta"] = model.sq_eta.numpy()
    out["bind_in_omega"] = model.sq_omega.numpy()
    out["bind_in_faces"] = model.faces.numpy()
    out["bind_in_alpha"] = model._alpha.numpy()
    out["bind_in_scale"] = model._scale.numpy()
    out["bind_out_xyz"] = model._xyz.detach().numpy()
    out["bind_out_scaling"] = model._scaling.detach().numpy()
    out["bind_out_rotation"] = model._rotation.detach().numpy()
    out["bind_out_opacity"] = opac.detach().numpy()
    for k, v in dict(xyz=gx, scaling=gs, rotation=gr, opacity=go).items():
        out[f"bind_upstream_{k}"] = v.numpy()
    np.savez_compressed(os.path.join(HERE, "reference_python.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_python.npz"), sorted(out))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
