"""The CUDA superquadric binding and its hand-written adjoint against the
float64 restatement (autograd) at the block-level workload's size: 8
superquadrics, 2,500 surfels each on a 50x50 (eta, omega) grid; plus the
float64 finite-difference check of the composite binding + rasteriser
gradient of the superquadric parameters."""
import numpy as np
import pytest
import torch

from oracle import binding_oracle as B

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def inputs(sgr_lib):
    return B.random_binding_inputs(B=8, n_eta=50, n_omega=50, N=1, seed=0)


def _cuda_binding(inp):
    from partgs_gb300.binding import SuperquadricBinding
    return SuperquadricBinding(inp["eta"].cuda(), inp["omega"].cuda(), inp["faces"].cuda(),
                               inp["alpha_raw"].cuda(), inp["scale"].cuda(), inp["ratio_block_scene"],
                               inp["scale_block_min"])


NAMES = ["sq_s", "sq_r", "sq_t", "sq_eps", "sq_occ"]


def _restated(inp, dtype, requires_grad=False):
    ps = [inp[k].to(dtype).clone().requires_grad_(requires_grad) for k in NAMES]
    out = B.bind(*ps, inp["eta"].to(dtype), inp["omega"].to(dtype), inp["faces"], inp["alpha_raw"].to(dtype),
                 inp["scale"].to(dtype), inp["ratio_block_scene"], inp["scale_block_min"])
    return ps, out


def test_binding_forward(inputs):
    """Within 5e-5 of the float64 restatement, or within twice the float32
    restatement's own distance to it (thin triangles near the poles make the
    Gram-Schmidt tangent, hence its log scale, ill-conditioned in FP32)."""
    bind = _cuda_binding(inputs)
    out = bind(*(inputs[k].float().cuda() for k in NAMES))
    _, ref = _restated(inputs, torch.float64)
    _, ref32 = _restated(inputs, torch.float32)
    assert out[0].shape == (20000, 3)
    for o, r, r32, k in zip(out, ref, ref32, ["xyz", "log_scaling", "rotation", "opacity"]):
        err = float((o.double().cpu() - r).abs().max())
        floor = float((r32.double() - r).abs().max())
        assert err < max(5e-5, 2 * floor), (k, err, floor)


def test_binding_adjoint(inputs):
    bind = _cuda_binding(inputs)
    p_cuda = [inputs[k].float().cuda().requires_grad_(True) for k in NAMES]
    out = bind(*p_cuda)
    p64, ref = _restated(inputs, torch.float64, True)
    p32, ref32 = _restated(inputs, torch.float32, True)
    g = torch.Generator().manual_seed(1)
    ups = [torch.randn(r.shape, generator=g, dtype=torch.float64) for r in ref]
    sum((o * u.float().cuda()).sum() for o, u in zip(out, ups)).backward()
    sum((r * u).sum() for r, u in zip(ref, ups)).backward()
    sum((r * u.float()).sum() for r, u in zip(ref32, ups)).backward()
    for k, pc, pr, p3 in zip(NAMES, p_cuda, p64, p32):
        scale = float(pr.grad.abs().max())
        err = float((pc.grad.double().cpu() - pr.grad).abs().max()) / scale
        floor = float((p3.grad.double() - pr.grad).abs().max()) / scale
        assert err < max(1e-4, 2 * floor), (k, err, floor)


def test_binding_then_rasterise_gradient_fd():
    """d(loss)/d(superquadric parameters) through binding + rasteriser on the
    GPU against float64 central differences of the oracle chain (binding
    restatement + rasteriser oracle) on a small case."""
    from oracle import surfel_oracle as O
    from partgs_gb300.batched import MultiViewRasterizer
    from partgs_gb300.cameras import orbit_cameras
    inp = B.random_binding_inputs(B=2, n_eta=10, n_omega=12, N=1, seed=3)
    cams = orbit_cameras(2, 2.2, 40, 48, 55.0, seed=4)
    names = ["sq_s", "sq_r", "sq_t", "sq_eps", "sq_occ"]
    P = inp["faces"].shape[0] * inp["faces"].shape[1]
    shs = torch.randn(P, 16, 3, generator=torch.Generator().manual_seed(5), dtype=torch.float64) * 0.2
    g = np.random.default_rng(6)
    wts = [g.standard_normal((3, 40, 48)) for _ in cams]

    def oracle_loss(params):
        xyz, ls, rot, op = B.bind(*params, inp["eta"], inp["omega"], inp["faces"], inp["alpha_raw"], inp["scale"],
                                  inp["ratio_block_scene"], inp["scale_block_min"])
        s = O.Surfels(xyz.numpy(), op.numpy(), np.exp(ls.numpy()), rot.numpy(), shs=shs.numpy(), sh_degree=3)
        tot = 0.0
        for cam, w in zip(cams, wts):
            oc = O.Camera(cam.world_view_transform.reshape(-1), cam.full_proj_transform.reshape(-1),
                          cam.camera_center, cam.tanfovx, cam.tanfovy, cam.height, cam.width)
            tot += float((O.forward_view(s, oc, np.zeros(3), O.PLAIN, np.float64).color * w).sum())
        return tot

    bind = _cuda_binding(inp)
    mv = MultiViewRasterizer(cams, [0, 0, 0], 3, num_surfels=P)
    pc = [inp[k].float().cuda().requires_grad_(True) for k in names]
    xyz, ls, rot, op = bind(*pc)
    img, _, _, _ = mv(xyz, op, shs.float().cuda(), torch.exp(ls), torch.nn.functional.normalize(rot))
    (img * torch.tensor(np.stack(wts), dtype=torch.float32).cuda()).sum().backward()
    eps = 1e-6
    for k_i, k in enumerate(names[:3]):
        base = [inp[n].clone() for n in names]
        fd = torch.zeros_like(base[k_i])
        for idx in np.ndindex(*base[k_i].shape):
            vals = []
            for sgn in (1, -1):
                pp = [t.clone() for t in base]
                pp[k_i][idx] += sgn * eps
                vals.append(oracle_loss(pp))
            fd[idx] = (vals[0] - vals[1]) / (2 * eps)
        an = pc[k_i].grad.double().cpu()
        err = float((an - fd).abs().max() / fd.abs().max())
        assert err < 2e-3, (k, err)
