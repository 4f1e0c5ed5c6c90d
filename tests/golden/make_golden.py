"""Generates tests/golden/reference_python.npz from the reference's own Python.

Run with a PartGS checkout: its root is the first argument, or the
PARTGS_REFERENCE environment variable.  It imports, unmodified:

* utils/sh_utils.py            eval_sh (SH colour)
* utils/graphics_utils.py      getWorld2View2, getProjectionMatrix (camera matrices)
* utils/general_utils.py       rot_to_quat_batch (rotation matrix -> quaternion)
* utils/point_utils.py         depth_to_normal (normals from a depth map)
* utils/loss_utils.py          l1_loss, ssim: the photometric term of train.py:230-231, per view,
                               differentiated by autograd (point_loss.npz)
* renderer/gaussian_renderer/__init__.py
                               render()'s post-processing of the rasteriser's maps (world normal,
                               expected / median / surface depth, surface normal), with the
                               rasteriser call answered by given maps; the point loss of
                               train.py:230-249 on its outputs (render_post.npz)
* games/block_mesh_splatting/scene/block_gaussian_model.py
                               update_alpha / get_verts / prepare_scaling_rot / get_opacity
                               (the superquadric -> surfel binding), differentiated by autograd,
                               on a grid and on an icosphere (bind_icosphere.npz);
                               summarize_losses' ray and overlap terms (sq_losses.npz, with
                               scene/cameras.py cast_rays and utils/superquadric.py implicit_sq)

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


def sq_losses(bgm, ref_root):
    """tests/golden/sq_losses.npz: the block-stage losses of summarize_losses
    (ray coverage / uncoverage / occupancy over a 16x12 view's rays, and the
    overlap term with 64 points per block), in float64, and their gradients
    to the block parameters by autograd.  The camera's own cast_rays makes the
    ray samples; torch.randperm / torch.rand / torch.randn_like are fed the
    stored draws."""
    from scene.cameras import Camera
    from utils.graphics_utils import getWorld2View2
    g = torch.Generator().manual_seed(1)
    torch.set_default_dtype(torch.float64)
    N, H, W, P, ratio = 4, 12, 16, 64, 0.25
    S = (torch.rand(N, 3, generator=g) + 0.6).requires_grad_(True)
    q = torch.randn(N, 4, generator=g)
    q = q / q.norm(dim=1, keepdim=True)
    w_, x, y, z = q.unbind(1)
    R = torch.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w_ * z), 2 * (x * z + w_ * y),
                     2 * (x * y + w_ * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w_ * x),
                     2 * (x * z - w_ * y), 2 * (y * z + w_ * x), 1 - 2 * (x * x + y * y)], 1)
    R = R.reshape(N, 3, 3).detach().requires_grad_(True)
    T = ((torch.rand(N, 3, generator=g) - 0.5) * 0.3).requires_grad_(True)
    eps1 = (torch.rand(N, 1, generator=g) * 1.6 + 0.2).requires_grad_(True)
    eps2 = (torch.rand(N, 1, generator=g) * 1.6 + 0.2).requires_grad_(True)
    sq_occ = (torch.randn(N, 1, generator=g) * 0.5 + 3.0).requires_grad_(True)   # overlapping, opaque blocks
    perm = torch.randperm(H * W, generator=g)
    jitter = torch.rand(H * W, 128, 1, generator=g)
    unit01 = torch.rand(N, P, 3, generator=g)
    noise = torch.randn(N, 1, generator=g)
    mask = (torch.rand(H, W, generator=g) < 0.5).double()

    ang = 0.4
    c = np.array([3 * math.sin(ang), 0.3, 3 * math.cos(ang)])
    fwd = -c / np.linalg.norm(c)
    right = np.cross([0, 1.0, 0], fwd)
    right /= np.linalg.norm(right)
    down = np.cross(fwd, right)
    Rc = np.stack([right, down, fwd], 1)
    Tc = -Rc.T @ c
    fovx = math.radians(50)
    fovy = 2 * math.atan(math.tan(fovx / 2) * H / W)
    K = torch.zeros((3, 3), dtype=torch.float32)
    K[0, 0] = (W / 2.0) / math.tan(fovx / 2.0)
    K[1, 1] = (H / 2.0) / math.tan(fovy / 2.0)
    K[0, 2] = W / 2.0
    K[1, 2] = H / 2.0
    K[2, 2] = 1.0
    wv = torch.tensor(getWorld2View2(Rc, Tc)).transpose(0, 1).float()
    recorded = {}
    cam = types.SimpleNamespace(image_height=H, image_width=W, data_device="cpu", K=K, world_view_transform=wv,
                                original_mask=mask)
    cam.invert = types.MethodType(Camera.invert, cam)
    cam.cam2world = types.MethodType(Camera.cam2world, cam)

    def cast_rays(**kw):
        pts, idx = Camera.cast_rays(cam, **kw)
        recorded["points"] = pts
        return pts, idx
    cam.cast_rays = cast_rays

    real_rand, real_randperm, real_randn_like = torch.rand, torch.randperm, torch.randn_like

    def rand(*shape, **k):
        shape = tuple(shape[0]) if len(shape) == 1 and isinstance(shape[0], (tuple, list)) else shape
        if shape == (H * W, 128, 1):
            return jitter.clone()
        if shape == (N, P, 3):
            return unit01.clone()
        raise AssertionError(f"unexpected torch.rand{shape}")

    model = bgm.BlockGaussianModel.__new__(bgm.BlockGaussianModel)
    model.n_blocks = N
    model.ratio_block_scene = ratio
    model.coarse_learning = True
    model.opacity_activation = torch.sigmoid
    model.sq_occ = sq_occ
    model._blocks_SRT = (S, R, T)
    model._blocks_eps = (eps1, eps2)
    opt = types.SimpleNamespace(rgb_weight=1.0, lambda_dssim=0.2, primtive_scale_weight=0.0, parsimony_weight=0.0,
                                data_type="blender", ray_coverage_weigth=10.0, ray_uncoverage_weigth=100.0,
                                occupancy_weight=0.02, overlap_weight=2.0)
    image = torch.rand(3, H, W, generator=g)
    n_points = bgm.OVERLAP_N_POINTS
    bgm.OVERLAP_N_POINTS = P
    torch.rand, torch.randperm, torch.randn_like = rand, (lambda *a, **k: perm.clone()), (lambda t: noise.clone())
    try:
        _, loss, parts = model.summarize_losses(image, image.clone(), cam, opt)
    finally:
        torch.rand, torch.randperm, torch.randn_like = real_rand, real_randperm, real_randn_like
        bgm.OVERLAP_N_POINTS = n_points
    loss.backward()
    out = dict(S=S, R=R, T=T, eps1=eps1, eps2=eps2, sq_occ=sq_occ)
    res = {f"in_{k}": v.detach().numpy() for k, v in out.items()}
    res.update({f"grad_{k}": v.grad.numpy() for k, v in out.items()})
    res.update(K=K.numpy(), world_view=wv.numpy(), height=H, width=W, ratio=ratio, near=2.0, far=5.0,
               ray_idx=perm.numpy(), jitter=jitter[..., 0].numpy(), mask=mask.numpy(), unit01=unit01.numpy(),
               noise=noise[:, 0].numpy(), weights=np.array([10.0, 100.0, 0.02, 2.0]),
               points_head=recorded["points"][:, :8].detach().numpy(),
               losses=np.array([float(parts[k].detach()) for k in ("ray_in_mask", "ray_out_mask", "primitive_opacity",
                                                          "overlap")]))
    torch.set_default_dtype(torch.float32)
    np.savez_compressed(os.path.join(HERE, "sq_losses.npz"), **res)
    print("wrote", os.path.join(HERE, "sq_losses.npz"), res["losses"])


def main(ref_root):
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


def icosphere(level: int):
    """Unit icosphere: the icosahedron (vertices the cyclic permutations of
    (0, +-1, +-phi), faces the vertex triples at mutual edge length 2,
    wound outward), each level splitting every triangle into four at its
    normalised edge midpoints.  Level 2: 162 vertices, 320 faces, with
    vertices at the poles (0, +-1, 0)."""
    phi = (1.0 + 5.0 ** 0.5) / 2.0
    v = []
    for a in (-1.0, 1.0):
        for b in (-phi, phi):
            v += [(0.0, a, b), (a, b, 0.0), (b, 0.0, a)]
    v = np.array(v)
    faces = []
    n = len(v)
    for i in range(n):
        for j in range(i + 1, n):
            for k in range(j + 1, n):
                d = [np.linalg.norm(v[i] - v[j]), np.linalg.norm(v[j] - v[k]), np.linalg.norm(v[i] - v[k])]
                if np.allclose(d, 2.0):
                    f = [i, j, k]
                    if np.dot(np.cross(v[j] - v[i], v[k] - v[i]), v[i] + v[j] + v[k]) < 0:
                        f = [i, k, j]
                    faces.append(f)
    verts = list(v / np.linalg.norm(v, axis=1, keepdims=True))
    for _ in range(level):
        mid, out = {}, []

        def m(a, b):
            key = (min(a, b), max(a, b))
            if key not in mid:
                c = verts[a] + verts[b]
                verts.append(c / np.linalg.norm(c))
                mid[key] = len(verts) - 1
            return mid[key]
        for a, b, c in faces:
            ab, bc, ca = m(a, b), m(b, c), m(c, a)
            out += [[a, ab, ca], [b, bc, ab], [c, ca, bc], [ab, bc, ca]]
        faces = out
    return np.array(verts), np.array(faces, dtype=np.int64)


def bind_icosphere(bgm):
    """tests/golden/bind_icosphere.npz: the binding on the block model's own
    topology type, a level-2 icosphere (dataset_readers.py:130, with eta =
    asin(y) and omega = atan2(x, z) as :141-142), poles included, 3 splats
    per face, 2 blocks; prepare_scaling_rot and its autograd gradients in the
    reference's float32."""
    g = torch.Generator().manual_seed(21)
    verts, faces = icosphere(2)
    vt = torch.tensor(verts, dtype=torch.float32)
    eta, omega = torch.asin(vt[:, 1].clamp(-1, 1)), torch.atan2(vt[:, 0], vt[:, 2])
    B, N, Fn = 2, 3, faces.shape[0]
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
    model.sq_eta = eta.expand(B, -1).contiguous()
    model.sq_omega = omega.expand(B, -1).contiguous()
    model.faces = torch.tensor(faces).expand(B, -1, -1).contiguous()
    model._alpha = torch.rand(B, Fn, N, 3, generator=g)
    model._scale = torch.rand(B, Fn * N, 1, generator=g) * 0.5 + 0.5
    model.update_alpha()
    model.prepare_scaling_rot()
    opac = model.get_opacity
    ups = {k: torch.randn(t.shape, generator=g) for k, t in
           dict(xyz=model._xyz, scaling=model._scaling, rotation=model._rotation, opacity=opac).items()}
    loss = sum((t * ups[k]).sum() for k, t in
               dict(xyz=model._xyz, scaling=model._scaling, rotation=model._rotation, opacity=opac).items())
    loss.backward()
    out = {}
    for k, v in dict(sq_s=sq_s, sq_r=sq_r, sq_t=sq_t, sq_eps=sq_eps, sq_occ=sq_occ).items():
        out[f"in_{k}"] = v.detach().numpy()
        out[f"grad_{k}"] = v.grad.numpy()
    out.update(in_eta=model.sq_eta.numpy(), in_omega=model.sq_omega.numpy(), in_faces=model.faces.numpy(),
               in_alpha=model._alpha.numpy(), in_scale=model._scale.numpy(), out_xyz=model._xyz.detach().numpy(),
               out_scaling=model._scaling.detach().numpy(), out_rotation=model._rotation.detach().numpy(),
               out_opacity=opac.detach().numpy(), **{f"upstream_{k}": v.numpy() for k, v in ups.items()})
    np.savez_compressed(os.path.join(HERE, "bind_icosphere.npz"), **out)
    print("wrote", os.path.join(HERE, "bind_icosphere.npz"), "vertices", len(verts), "faces", Fn,
          "poles", int((np.abs(verts[:, 1]) > 1 - 1e-12).sum()))


def main_bind_ico(ref_root):
    sys.path.insert(0, ref_root)
    _stub_modules()
    _cpu_only()
    torch.set_default_dtype(torch.float32)
    import games.block_mesh_splatting.scene.block_gaussian_model as bgm
    bind_icosphere(bgm)


def densify(ref_root):
    """tests/golden/densify.npz: TwoGaussianModel's densify_and_prune (clone,
    split with the stored normal draws, prune, optimiser state surgery) and
    reset_opacity on 400 surfels, the statistics of train.py:293-297 over
    three iterations, and both models' PLY attribute lists."""
    import games.block_mesh_splatting.scene.two_gaussian_model as tgm
    import scene.gaussian_model as gm
    from utils import general_utils
    g = torch.Generator().manual_seed(2)
    P, M = 400, 16
    real_zeros, real_normal = torch.zeros, torch.normal

    def zeros(*a, **k):
        k.pop("device", None)
        return real_zeros(*a, **k)

    model = tgm.TwoGaussianModel.__new__(tgm.TwoGaussianModel)
    gm.GaussianModel.setup_functions(model) if hasattr(gm.GaussianModel, "setup_functions") else None
    model.scaling_activation, model.scaling_inverse_activation = torch.exp, torch.log
    model.opacity_activation, model.inverse_opacity_activation = torch.sigmoid, general_utils.inverse_sigmoid
    model.rotation_activation = torch.nn.functional.normalize
    model.percent_dense = 0.01
    model.max_sh_degree = 3
    raw = {"xyz": torch.randn(P, 3, generator=g), "f_dc": torch.randn(P, 1, 3, generator=g),
           "f_rest": torch.randn(P, M - 1, 3, generator=g) * 0.1,
           "opacity": torch.randn(P, 1, generator=g) * 2 - 1,
           "scaling": torch.log(torch.rand(P, 2, generator=g) * 0.05 + 0.005),
           "rotation": torch.randn(P, 4, generator=g)}
    attr = {"xyz": "_xyz", "f_dc": "_features_dc", "f_rest": "_features_rest", "opacity": "_opacity",
            "scaling": "_scaling", "rotation": "_rotation"}
    for k, v in raw.items():
        setattr(model, attr[k], torch.nn.Parameter(v.clone()))
    model._semantic = torch.rand(P, 4, generator=g)
    model.optimizer = torch.optim.Adam([{"params": [getattr(model, attr[k])], "lr": 0.01, "name": k} for k in raw],
                                       lr=0.0, eps=1e-15)
    for k in raw:   # one step so every parameter has Adam moments to carry
        getattr(model, attr[k]).grad = torch.randn(raw[k].shape, generator=g)
    model.optimizer.step()
    out = {f"in_{k}": getattr(model, attr[k]).detach().numpy().copy() for k in raw}
    for k in raw:
        st = model.optimizer.state[getattr(model, attr[k])]
        out[f"in_m_{k}"], out[f"in_v_{k}"] = st["exp_avg"].numpy().copy(), st["exp_avg_sq"].numpy().copy()
    out["in_semantic"] = model._semantic.numpy().copy()
    # statistics: three views' radii and screen-space gradients
    model.xyz_gradient_accum = torch.zeros(P, 1)
    model.denom = torch.zeros(P, 1)
    model.max_radii2D = torch.zeros(P)
    radii = (torch.rand(3, P, generator=g) * 30).int() * (torch.rand(3, P, generator=g) < 0.7).int()
    g2d = torch.randn(3, P, 3, generator=g) * 2e-4
    for it in range(3):
        vis = radii[it] > 0
        model.max_radii2D[vis] = torch.max(model.max_radii2D[vis], radii[it][vis])
        vp = types.SimpleNamespace(grad=g2d[it])
        model.add_densification_stats(vp, vis)
    out.update(stats_radii=radii.numpy(), stats_grad=g2d.numpy(), stats_accum=model.xyz_gradient_accum.numpy().copy(),
               stats_denom=model.denom.numpy().copy(), stats_max_radii=model.max_radii2D.numpy().copy())
    # densify and prune with grad threshold 2e-4, min opacity 0.05, extent 1.5, screen size 20
    grads = model.xyz_gradient_accum / model.denom
    grads[grads.isnan()] = 0.0
    n_split = None
    draws = {}

    def normal(mean, std, *a, **k):
        x = real_normal(torch.zeros_like(mean), torch.ones_like(std), generator=g) * std + mean
        draws["split"] = x.detach().clone()
        return x
    torch.zeros, torch.normal = zeros, normal
    general_utils.torch.zeros = zeros
    try:
        model.densify_and_prune(2e-4, 0.05, 1.5, 20)
    finally:
        torch.zeros, torch.normal = real_zeros, real_normal
    out["split_samples"] = draws["split"].numpy()
    for k in raw:
        t = getattr(model, attr[k])
        out[f"out_{k}"] = t.detach().numpy()
        st = model.optimizer.state[t]
        out[f"out_m_{k}"], out[f"out_v_{k}"] = st["exp_avg"].detach().numpy(), st["exp_avg_sq"].detach().numpy()
    out["out_semantic"] = model._semantic.detach().numpy()
    out["densify_args"] = np.array([2e-4, 0.05, 1.5, 20, 0.01])
    # reset_opacity on the densified set
    torch.zeros = zeros
    try:
        model.reset_opacity()
    finally:
        torch.zeros = real_zeros
    t = model._opacity
    out["reset_opacity"] = t.detach().numpy()
    out["reset_m_opacity"] = model.optimizer.state[t]["exp_avg"].detach().numpy()
    # PLY attribute lists (construct_list_of_attributes of both models)
    out["ply_attrs_two"] = np.array(tgm.TwoGaussianModel.construct_list_of_attributes(model))
    out["ply_attrs_plain"] = np.array(gm.GaussianModel.construct_list_of_attributes(model))
    np.savez_compressed(os.path.join(HERE, "densify.npz"), **out)
    print("wrote", os.path.join(HERE, "densify.npz"), P, "->", out["out_xyz"].shape[0])


def point_loss(ref_root):
    """The reference's photometric loss, (1 - lambda_dssim) L1 + lambda_dssim
    (1 - SSIM) (train.py:230-231, utils/loss_utils.py:6-7, 24-54), evaluated
    one view at a time as its training loop does, in float64, with the
    gradient w.r.t. the rendered image from autograd."""
    from utils.loss_utils import l1_loss, ssim
    g = torch.Generator().manual_seed(11)
    V, H, W, lam = 2, 24, 40, 0.2
    yy, xx = torch.meshgrid(torch.linspace(0, 1, H, dtype=torch.float64),
                            torch.linspace(0, 1, W, dtype=torch.float64), indexing="ij")
    base = 0.5 + 0.4 * torch.sin(7 * xx + 3 * yy)[None, None] * torch.rand(V, 3, 1, 1, generator=g, dtype=torch.float64)
    target = (base + 0.05 * torch.rand(V, 3, H, W, generator=g, dtype=torch.float64)).clamp(0, 1)
    image = (target + 0.1 * torch.randn(V, 3, H, W, generator=g, dtype=torch.float64)).clamp(0, 1)
    out = dict(image=image.numpy(), target=target.numpy(), lambda_dssim=np.float64(lam))
    l1s, ssims, losses, grads = [], [], [], []
    for v in range(V):
        img = image[v].clone().requires_grad_(True)
        l1 = l1_loss(img, target[v])
        s = ssim(img, target[v])
        loss = (1.0 - lam) * l1 + lam * (1.0 - s)
        loss.backward()
        l1s.append(float(l1.detach()))
        ssims.append(float(s.detach()))
        losses.append(float(loss.detach()))
        grads.append(img.grad.numpy())
    out.update(l1=np.array(l1s), ssim=np.array(ssims), loss=np.array(losses), grad=np.stack(grads))
    np.savez_compressed(os.path.join(HERE, "point_loss.npz"), **out)
    print("wrote", os.path.join(HERE, "point_loss.npz"), "ssim", ssims)


def render_post(ref_root):
    """The reference renderer's post-processing and the point loss on it.

    render() (renderer/gaussian_renderer/__init__.py:9-141) runs unmodified;
    its rasteriser (diff_surfel_rasterization) is replaced by a stand-in that
    returns a given image and allmap, so what is exercised is the code after
    the call (:111-141: normal view -> world, expected depth with
    nan_to_num, median depth, surf_depth by depth_ratio, surf_normal from
    utils/point_utils.py depth_to_normal times the detached alpha).  The
    loss on its outputs is train.py:230-231 (photometric, through
    utils/loss_utils.py) plus :244-249 (normal consistency and distortion,
    both weights active), in the reference's float32, with autograd
    gradients w.r.t. the image and the allmap.  Two views, two depth ratios."""
    sys.path.insert(0, ROOT)
    from partgs_gb300.cameras import orbit_cameras
    slot = {}

    class _Rasterizer:
        def __init__(self, raster_settings):
            self.raster_settings = raster_settings

        def __call__(self, **kw):
            return slot["image"], torch.zeros(kw["means3D"].shape[0], dtype=torch.int32), slot["allmap"]

    stub = types.ModuleType("diff_surfel_rasterization")
    stub.GaussianRasterizationSettings = lambda **kw: types.SimpleNamespace(**kw)
    stub.GaussianRasterizer = _Rasterizer
    sys.modules["diff_surfel_rasterization"] = stub
    real_zeros_like = torch.zeros_like

    def zeros_like(*a, **k):
        k.pop("device", None)
        return real_zeros_like(*a, **k)
    torch.zeros_like = zeros_like
    from renderer.gaussian_renderer import render
    from utils.loss_utils import l1_loss, ssim

    V, H, W, lam, lam_dist, lam_normal = 2, 24, 32, 0.2, 1000.0, 0.05
    cams = orbit_cameras(V, 3.0, H, W, 55.0, seed=4)
    g = torch.Generator().manual_seed(12)
    yy, xx = torch.meshgrid(torch.linspace(-1, 1, H), torch.linspace(-1, 1, W), indexing="ij")
    image = torch.rand(V, 3, H, W, generator=g)
    target = torch.rand(V, 3, H, W, generator=g)
    alpha = 0.2 + 0.8 * torch.rand(V, 1, H, W, generator=g)
    median = 2.5 + 0.3 * torch.sin(3 * xx + 1) * torch.cos(2 * yy) + 0.01 * torch.rand(V, 1, H, W, generator=g)
    expected = median * alpha * (1 + 0.05 * torch.rand(V, 1, H, W, generator=g))
    normal = torch.nn.functional.normalize(torch.randn(V, 3, H, W, generator=g), dim=1) * alpha
    dist = 1e-3 * torch.rand(V, 1, H, W, generator=g)
    allmap = torch.cat([expected, alpha, normal, median, dist], 1)
    pc = types.SimpleNamespace(get_xyz=torch.zeros(4, 3), get_opacity=torch.ones(4, 1),
                               get_scaling=torch.ones(4, 2), get_rotation=torch.ones(4, 4),
                               get_features=torch.zeros(4, 16, 3), active_sh_degree=3, max_sh_degree=3)
    out = dict(image=image.numpy(), target=target.numpy(), allmap=allmap.numpy(),
               lambdas=np.array([lam, lam_dist, lam_normal]))
    for ratio in (1.0, 0.4):
        pipe = types.SimpleNamespace(compute_cov3D_python=False, convert_SHs_python=False, depth_ratio=ratio,
                                     debug=False)
        tag = f"r{int(ratio * 10)}"
        losses, g_img, g_map = [], [], []
        for v, c in enumerate(cams):
            cam = types.SimpleNamespace(FoVx=c.fovx, FoVy=c.fovy, image_height=H, image_width=W,
                                        world_view_transform=torch.as_tensor(c.world_view_transform),
                                        full_proj_transform=torch.as_tensor(c.full_proj_transform),
                                        camera_center=torch.as_tensor(c.camera_center), znear=0.01, zfar=100.0)
            img = image[v].clone().requires_grad_(True)
            am = allmap[v].clone().requires_grad_(True)
            slot.update(image=img, allmap=am)
            pkg = render(cam, pc, pipe, torch.zeros(3))
            loss = (1.0 - lam) * l1_loss(pkg["render"], target[v]) + lam * (1.0 - ssim(pkg["render"], target[v]))
            normal_error = (1 - (pkg["rend_normal"] * pkg["surf_normal"]).sum(dim=0))[None]
            loss = loss + lam_dist * pkg["rend_dist"].mean() + lam_normal * normal_error.mean()
            loss.backward()
            losses.append(float(loss.detach()))
            g_img.append(img.grad.numpy())
            g_map.append(am.grad.numpy())
        out.update({f"{tag}_loss": np.array(losses), f"{tag}_grad_image": np.stack(g_img),
                    f"{tag}_grad_allmap": np.stack(g_map)})
    torch.zeros_like = real_zeros_like
    np.savez_compressed(os.path.join(HERE, "render_post.npz"), **out)
    print("wrote", os.path.join(HERE, "render_post.npz"), {k: v for k, v in out.items() if k.endswith("_loss")})


def main_loss(ref_root):
    sys.path.insert(0, ref_root)
    _stub_modules()
    _cpu_only()
    point_loss(ref_root)
    render_post(ref_root)


def main_sq(ref_root):
    sys.path.insert(0, ref_root)
    _stub_modules()
    _cpu_only()
    import games.block_mesh_splatting.scene.block_gaussian_model as bgm
    sq_losses(bgm, ref_root)


def main_densify(ref_root):
    sys.path.insert(0, ref_root)
    _stub_modules()
    _cpu_only()
    densify(ref_root)


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    root = args[0] if args else os.environ.get("PARTGS_REFERENCE")
    if not root:
        raise SystemExit("usage: make_golden.py <PartGS checkout> [--sq|--densify|--loss|--bind-ico] "
                         "(or set PARTGS_REFERENCE)")
    if "--sq" in sys.argv:   # only the superquadric-loss fixture
        main_sq(root)
    elif "--densify" in sys.argv:   # only the densification fixture
        main_densify(root)
    elif "--loss" in sys.argv:   # only the photometric-loss fixture
        main_loss(root)
    elif "--bind-ico" in sys.argv:   # only the icosphere binding fixture
        main_bind_ico(root)
    else:
        main(root)
        main_sq(root)
        main_densify(root)
        main_loss(root)
        main_bind_ico(root)
