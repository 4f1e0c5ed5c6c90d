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


def ours_render(variant, cam, bg, means3D, opacities, shs=None, colors_precomp=None, scales=None, rotations=None,
                transmat_precomp=None, semantics=None, sh_degree=3, scale_modifier=1.0, upstream=None):
    """The same call as ``oracle.ref_cuda.render`` through this library's
    drop-in ``GaussianRasterizer`` (images, radii, leaf gradients), plus the
    core's per-pixel and per-tile state of the same forward (contributor
    counts, final T planes, tile ranges and lists)."""
    from partgs_gb300 import _lib as L
    from partgs_gb300 import raster
    if variant == "part":
        import partgs_gb300.diff_surfel_rasterization_part as mod
    else:
        import partgs_gb300.diff_surfel_rasterization as mod
    rs = settings(mod, cam, bg, sh_degree=sh_degree, scale_modifier=scale_modifier)
    leaf = {}

    def lf(name, t):
        if t is None:
            return None
        t = t.detach().float().cuda().contiguous().requires_grad_(upstream is not None)
        leaf[name] = t
        return t

    m3 = lf("means3D", means3D)
    m2 = torch.zeros_like(m3, requires_grad=upstream is not None)
    leaf["means2D"] = m2
    kw = dict(means3D=m3, means2D=m2, opacities=lf("opacity", opacities), shs=lf("sh", shs),
              colors_precomp=lf("colors", colors_precomp), scales=lf("scales", scales),
              rotations=lf("rotations", rotations), cov3D_precomp=lf("transmat", transmat_precomp))
    rast = mod.GaussianRasterizer(rs)
    semantic = None
    if variant == "part":
        kw["semantics"] = lf("semantics", semantics)
        color, semantic, radii, allmap = rast(**kw)
    else:
        color, radii, allmap = rast(**kw)
    out = dict(color=color.detach().cpu().numpy(), allmap=allmap.detach().cpu().numpy(),
               radii=radii.cpu().numpy().astype(np.int64))
    if semantic is not None:
        out["semantic"] = semantic.detach().cpu().numpy()
    if upstream is not None:
        dcol, doth, dsem = upstream
        loss = (color * torch.as_tensor(dcol, device="cuda")).sum() + \
            (allmap * torch.as_tensor(doth, device="cuda")).sum()
        if semantic is not None and dsem is not None:
            loss = loss + (semantic * torch.as_tensor(dsem, device="cuda")).sum()
        loss.backward()
        torch.cuda.synchronize()
        for k, t in leaf.items():
            if t is not None and t.grad is not None:
                out["dL_d" + k] = t.grad.detach().cpu().numpy()
    # the core's internal state for the same inputs
    v = L.SGR_VARIANT_PART if variant == "part" else L.SGR_VARIANT_PLAIN
    vs = raster.ViewSet(rs.viewmatrix.reshape(1, 16), rs.projmatrix.reshape(1, 16), rs.campos.reshape(1, 3),
                        [(cam.tanfovx, cam.tanfovy)], cam.height, cam.width)
    with torch.no_grad():
        c = lambda t: None if t is None else t.detach().float().cuda().contiguous()  # noqa: E731
        _, _, _, _, state = raster.forward(v, c(means3D), c(opacities), c(shs), c(colors_precomp), c(scales),
                                           c(rotations), c(transmat_precomp), c(semantics), vs, rs.bg, sh_degree,
                                           scale_modifier)
        dbg = raster.debug_state(state)
    out["tiles_touched"] = dbg["tiles_touched"].cpu().numpy().astype(np.int64)
    out["final_T"] = dbg["final_T"][0].cpu().numpy()
    out["n_contrib"] = dbg["n_contrib"][0].cpu().numpy().astype(np.int64)
    out["ranges"] = dbg["ranges"].cpu().numpy().astype(np.int64)
    out["point_list"] = dbg["point_list"].cpu().numpy().astype(np.int64)
    out["num_rendered"] = int(dbg["num_keys"])
    return out



# Gradients that run through the splat-to-pixel matrix adjoint: its FP32
# evaluation cancels per-fragment terms weighted by pixel coordinates, so
# single elements carry more rounding than the tensor as a whole (the
# reference's own CUDA lands up to ~1e-4 from FP64 on them, max-norm).
GEOMETRY_GRADS = ("dL_dmeans3D", "dL_dmeans2D", "dL_drotations", "dL_dtransmat")
GRAD_TOL = 1e-4             # max |a - b| / max |b|, and |a - b|_2 / |b|_2
GRAD_TOL_GEOMETRY = 3e-4    # max-norm bar of GEOMETRY_GRADS
GRAD_L2_TOL_GEOMETRY = 2e-4  # their L2 bar: the part variant's lands at 1.2e-4 to 1.7e-4 from FP64 (its AABB-centre
                             # adjoint cancels too), the reference binary's own up to 2.1e-4 (max-norm) on the same case


def ill_conditioned(st, cam, s, bg, variant, img_tol=1e-5, aux_tol=3e-5):
    """Pixels where rounding every surfel's splat-to-pixel matrix and screen
    centre by one FP32 unit moves the FP64 result by more than half the
    tolerance (oracle.fp32_sensitivity): nearly edge-on splats, whose value
    and gradients two FP32 implementations cannot agree on to the bars.
    Their upstream gradients are zeroed and they are left out of the image
    comparisons, like the oracle's rounding-ambiguous pixels."""
    from oracle import surfel_oracle as O
    sens = O.fp32_sensitivity(st, cam, s, np.asarray(bg, np.float64), variant)
    return (sens[:3].max(0) > 0.5 * img_tol) | (sens[3:].max(0) > 0.5 * aux_tol)


def l2_error(gpu, ref):
    """|gpu - ref|_2 / |ref|_2."""
    gpu = np.asarray(gpu, np.float64).reshape(-1)
    ref = np.asarray(ref, np.float64).reshape(-1)
    n = float(np.linalg.norm(ref))
    return float(np.linalg.norm(gpu - ref)) / n if n else float(np.linalg.norm(gpu))


def grad_check(got, ref, names=None):
    """Gradient tensors against reference ones: every tensor within GRAD_TOL
    relative in the L2 norm (GRAD_L2_TOL_GEOMETRY for GEOMETRY_GRADS), and
    its largest element error within GRAD_TOL (GRAD_TOL_GEOMETRY) of its
    largest magnitude.
    Returns ({name: (max-norm error, L2 error)}, {name: errors} of misses)."""
    errs, bad = {}, {}
    for k in (names or got.keys()):
        a = np.asarray(got[k], np.float64)
        b = np.asarray(ref[k], np.float64).reshape(a.shape)
        e = (grad_error(a, b), l2_error(a, b))
        errs[k] = e
        geo = k in GEOMETRY_GRADS
        if e[0] > (GRAD_TOL_GEOMETRY if geo else GRAD_TOL) or e[1] > (GRAD_L2_TOL_GEOMETRY if geo else GRAD_TOL):
            bad[k] = e
    return errs, bad
