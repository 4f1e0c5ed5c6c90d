"""Float64 central finite differences of the superquadric binding followed by
the plain rasteriser, for checking the hand-written adjoint chain
(``sgr_bind_backward`` after ``sgr_backward``) parameter by parameter.

TEST INFRASTRUCTURE ONLY.

The chain is the oracle's: ``binding_oracle.bind`` (prepare_scaling_rot,
games/block_mesh_splatting/scene/block_gaussian_model.py:198-256), the
model's quaternion normalisation, then ``surfel_oracle.forward_view`` (the
rasteriser), all in float64.  The loss
is a fixed weighted sum of the rendered colour and the seven auxiliary maps
of every view.

A parameter of block b moves only block b's surfels, so each evaluation
blends only the tiles those surfels' rectangles cover (one tile of margin);
every other pixel is unchanged by construction.

The chain orders each tile's surfels by their FP64 depth, not by the FP32
depth bits the reference sorts on: neighbouring surfels that tie in FP32
would otherwise trade places under perturbations far below any step.
Discrete decisions (the alpha cut-off, the stop test, the 3D/2D branch, the
median switch, the normal's orientation, two surfels crossing in depth, a
rectangle's rounding) make the loss jump.  Each evaluation
returns the oracle's per-pixel decision signature; a pixel whose signature
differs between any of the evaluations (+h, -h, +h/2, -h/2 and the
unperturbed one) is a "flip", and the checks leave such pixels out of both the difference and the
analytic gradient (the loss restricted to the other pixels is smooth over
[-h, +h], on the branch the analytic gradient is taken on).

Evaluations run in a ``spawn`` process pool.
"""
from __future__ import annotations

import multiprocessing as mp
import os

import numpy as np

NAMES = ["sq_s", "sq_r", "sq_t", "sq_eps", "sq_occ"]

_W = {}


def make_case(B=8, n_eta=50, n_omega=50, views=(0,), height=300, width=400, fovx=50.0, seed=0, channels=None):
    """The block-level workload's layout: B superquadrics with n_eta x n_omega
    surfels each, cameras on a radius-3 sphere; seeded SH colours and loss
    weights (``channels``: the loss channels kept, 0-2 the colour and 3-9 the
    auxiliary maps; all by default).  Returns a dict of numpy / torch inputs
    (float64)."""
    import torch
    from oracle import binding_oracle as Bo
    from partgs_gb300.cameras import orbit_cameras
    inp = Bo.random_binding_inputs(B=B, n_eta=n_eta, n_omega=n_omega, N=1, seed=seed)
    cams_all = orbit_cameras(8, 3.0, height, width, fovx, seed=seed)
    cams = [cams_all[v] for v in views]
    P = inp["faces"].shape[0] * inp["faces"].shape[1]
    shs = torch.randn(P, 16, 3, generator=torch.Generator().manual_seed(seed + 5), dtype=torch.float64) * 0.2
    g = np.random.default_rng(seed + 6)
    w_col = [g.standard_normal((3, height, width)) for _ in cams]
    w_oth = [g.standard_normal((7, height, width)) * 0.1 for _ in cams]
    if channels is not None:
        keep = np.isin(np.arange(10), channels).astype(np.float64)
        w_col = [w * keep[:3, None, None] for w in w_col]
        w_oth = [w * keep[3:, None, None] for w in w_oth]
    return dict(inp=inp, cams=cams, shs=shs, w_col=w_col, w_oth=w_oth, B=B)


def _camera(cam):
    from oracle import surfel_oracle as O
    return O.Camera(np.asarray(cam.world_view_transform, np.float64).reshape(-1),
                    np.asarray(cam.full_proj_transform, np.float64).reshape(-1),
                    np.asarray(cam.camera_center, np.float64), cam.tanfovx, cam.tanfovy, cam.height, cam.width)


def _bind(case, params):
    """The binding, then the model's rotation activation: the block model
    inherits GaussianModel.get_rotation (scene/gaussian_model.py:65, 203-205),
    torch.nn.functional.normalize.  The quaternions the binding makes are
    not unit (down to 0.992 here), and the rasteriser's quaternion adjoint
    (quat_to_rotmat_vjp, P0/cr/auxiliary.h:239) is the gradient with
    respect to the normalised quaternion, so the chain needs the
    normalisation's own Jacobian, which autograd supplies."""
    import torch
    from oracle import binding_oracle as Bo
    inp = case["inp"]
    xyz, ls, rot, op = Bo.bind(*params, inp["eta"], inp["omega"], inp["faces"], inp["alpha_raw"], inp["scale"],
                               inp["ratio_block_scene"], inp["scale_block_min"])
    return xyz, ls, torch.nn.functional.normalize(rot, dim=-1), op


def _surfels(case, params):
    from oracle import surfel_oracle as O
    xyz, ls, rot, op = (t.detach() for t in _bind(case, params))
    return O.Surfels(xyz.numpy(), op.numpy(), np.exp(ls.numpy()), rot.numpy(), shs=case["shs"].numpy(), sh_degree=3)


def block_tiles(case, block):
    """Per view, the tiles block `block`'s visible surfels cover, with one
    tile of margin (sorted tile indices)."""
    from oracle import surfel_oracle as O
    inp = case["inp"]
    s = _surfels(case, [inp[k] for k in NAMES])
    per_block = inp["faces"].shape[1] * inp["alpha_raw"].shape[1]
    out = []
    for cam in case["cams"]:
        pre = O.preprocess(s, _camera(cam), O.PLAIN, np.float64)
        gx, gy = pre["grid"]
        xmin, ymin, xmax, ymax = pre["rect"]
        mask = np.zeros((gy, gx), bool)
        for i in range(block * per_block, (block + 1) * per_block):
            if pre["radii"][i] > 0:
                mask[max(0, ymin[i] - 1):min(gy, ymax[i] + 1), max(0, xmin[i] - 1):min(gx, xmax[i] + 1)] = True
        out.append(np.nonzero(mask.reshape(-1))[0])
    return out


def pixel_values(case, params, tiles_per_view):
    """Per view: (weighted per-pixel loss contributions [H,W], decision
    signature [H,W], pixel mask of the blended tiles [H,W])."""
    from oracle import surfel_oracle as O
    s = _surfels(case, params)
    res = []
    for v, cam in enumerate(case["cams"]):
        st = O.forward_view(s, _camera(cam), np.zeros(3), O.PLAIN, np.float64, tiles=tiles_per_view[v],
                            exact_depth=True)
        val = (case["w_col"][v] * st.color).sum(0) + (case["w_oth"][v] * st.others).sum(0)
        gx = (cam.width + 15) // 16
        tmask = np.zeros(((cam.height + 15) // 16) * gx, bool)
        tmask[tiles_per_view[v]] = True
        yy, xx = np.mgrid[0:cam.height, 0:cam.width]
        pmask = tmask[(yy // 16) * gx + (xx // 16)]
        res.append((np.where(pmask, val, 0.0), st.extra["signature"], pmask))
    return res


def _init(case_kwargs):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    if root not in sys.path:
        sys.path.insert(0, root)
    import torch
    torch.set_num_threads(1)
    case = make_case(**case_kwargs)
    _W["case"] = case
    _W["tiles"] = {}


def _eval(job):
    """job = (name, flat index, signed step): per view (values, signature)
    on block b's tiles."""
    case = _W["case"]
    name, flat, delta = job
    inp = case["inp"]
    params = [inp[k].clone() for k in NAMES]
    k = NAMES.index(name)
    block = int(np.unravel_index(flat, params[k].shape)[0])
    if block not in _W["tiles"]:
        _W["tiles"][block] = block_tiles(case, block)
    params[k].view(-1)[flat] += delta
    res = pixel_values(case, params, _W["tiles"][block])
    out = []
    for val, sig, pm in res:
        idx = np.flatnonzero(pm)
        out.append((idx.astype(np.int32), val.reshape(-1)[idx], sig.reshape(-1)[idx]))
    return out


def _surfel_grads(case, v, wc, wo, tiles=None, exact=True):
    """FP64 oracle adjoint of sum(wc * colour + wo * others) of view v at the
    case's parameters: per-surfel gradients (means3D, scales, rotations,
    opacity) -- the rasteriser half of the chain.  ``exact``: tiles ordered
    by FP64 depth (the chain the differences see); else by the FP32 depth
    bits, as the reference and the library sort."""
    from oracle import surfel_oracle as O
    cache = _W.setdefault("forward", {})
    if (v, exact) not in cache:      # the forward at the case's parameters, once per view and process
        inp = case["inp"]
        s = _surfels(case, [inp[k] for k in NAMES])
        cam = _camera(case["cams"][v])
        cache[(v, exact)] = (s, cam, O.forward_view(s, cam, np.zeros(3), O.PLAIN, np.float64, exact_depth=exact))
    s, cam, st = cache[(v, exact)]
    g = O.backward_view(st, cam, s, np.zeros(3), wc, wo, variant=O.PLAIN, dtype=np.float64, tiles=tiles)
    return [np.asarray(g[k], np.float64) for k in ("dL_dmeans3D", "dL_dscales", "dL_drotations", "dL_dopacity")]


def _eval_grads(job):
    """job = (key, view, flat pixel indices or None[, exact]): the surfel
    gradients of the loss restricted to those pixels (all pixels with None)."""
    case = _W["case"]
    key, v, pix = job[:3]
    exact = job[3] if len(job) > 3 else True
    wc, wo = case["w_col"][v], case["w_oth"][v]
    tiles = None
    if pix is not None:
        cam = case["cams"][v]
        keep = np.zeros(cam.height * cam.width, bool)
        keep[pix] = True
        keep = keep.reshape(cam.height, cam.width)
        wc, wo = wc * keep, wo * keep
        gx = (cam.width + 15) // 16
        tiles = np.unique((pix // cam.width) // 16 * gx + (pix % cam.width) // 16)
    return key, _surfel_grads(case, v, wc, wo, tiles, exact)


def chain_to_parameters(case, surfel_grads):
    """FP64 vector-Jacobian product of the binding (binding_oracle.bind,
    autograd) for per-surfel gradients [means3D, scales, rotations,
    opacity]: {name: gradient of each block parameter}."""
    import torch
    inp = case["inp"]
    ps = [inp[k].clone().requires_grad_(True) for k in NAMES]
    xyz, ls, rot, op = _bind(case, ps)
    gx, gs, gr, go = surfel_grads
    scales = np.exp(ls.detach().numpy())      # the rasteriser takes exp(log_scaling)
    loss = (xyz * torch.tensor(gx)).sum() + (ls * torch.tensor(gs * scales)).sum() + \
        (rot * torch.tensor(gr)).sum() + (op * torch.tensor(go.reshape(-1, 1))).sum()
    loss.backward()
    return {k: p.grad.numpy().reshape(-1).copy() for k, p in zip(NAMES, ps)}


def check(case_kwargs, params, h=1e-6, procs=None, richardson=True):
    """Central differences of every parameter in ``params`` and the FP64
    analytic gradient of the same (flip-masked) loss: the oracle's adjoint
    of the rasteriser, then the binding's autograd.  Returns the
    finite_differences records, each with ``an64`` (the analytic value of
    the loss its ``fd`` differentiates, flip pixels left out) and
    ``masks`` (per view, the flat pixel indices left out), and ``an64_ref``:
    the same analytic gradient with each tile's surfels in the reference's
    order (FP32 depth bits, then index), the one to hold an FP32
    implementation of the reference's algorithm against.

    With ``richardson`` the difference is extrapolated from the steps h and
    h/2, (4 D(h/2) - D(h)) / 3, which cancels the truncation term (h^2 / 6
    times the third derivative): pixels of nearly edge-on splats are smooth
    over the step but steep and curved (third derivatives near 1e11 per
    unit translation), which leaves plain central differences 1e-4 off."""
    procs = procs or min(16, os.cpu_count() or 1)
    case = make_case(**case_kwargs)
    V = len(case["cams"])
    steps = (h, h / 2) if richardson else (h,)
    per = 2 * len(steps)
    jobs = [(n, f, sgn * d) for n, f in params for d in steps for sgn in (1, -1)]
    # the unperturbed signature of each block's tiles: a pixel whose +h and
    # -h decisions agree but differ from the base point's (a near-tie that
    # rounding breaks one way at the base and the other way at both steps)
    # is a flip too, since the analytic gradient is taken at the base
    block_of = {}
    for n, f in params:
        b = int(np.unravel_index(f, case["inp"][n].shape)[0])
        block_of[(n, f)] = b
        if b not in block_of:
            block_of[b] = len(jobs)
            jobs.append((n, f, 0.0))
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs, initializer=_init, initargs=(case_kwargs,)) as pool:
        full = pool.map_async(_eval_grads, [(("full", v, ex), v, None, ex) for v in range(V) for ex in (True, False)],
                              chunksize=1)
        res = pool.map(_eval, jobs, chunksize=1)
        out = []
        corr_jobs = []
        for i, (n, f) in enumerate(params):
            evals = res[per * i:per * (i + 1)]
            base = res[block_of[block_of[(n, f)]]]
            views, fd, flips, masks = [], 0.0, 0, []
            for v in range(V):
                idx, _, s0 = base[v]
                flip = np.zeros(len(idx), bool)
                qs = []
                for k, d in enumerate(steps):
                    (_, vp, sp), (_, vm, sm) = evals[2 * k][v], evals[2 * k + 1][v]
                    qs.append((vp - vm) / (2 * d))
                    flip |= (sp != s0) | (sm != s0)
                q = (4 * qs[1] - qs[0]) / 3 if richardson else qs[0]
                views.append(dict(pixels=idx, quotient=q, flip=flip))
                fd += float(q[~flip].sum())
                flips += int(flip.sum())
                masks.append(idx[flip])
                if flip.any():
                    corr_jobs += [((i, v, ex), v, idx[flip], ex) for ex in (True, False)]
            out.append(dict(name=n, flat=f, fd=fd, views=views, flips=flips, masks=masks))
        corr = dict(pool.map(_eval_grads, corr_jobs, chunksize=1))
        full = dict(full.get())
    for ex, key in ((True, "an64"), (False, "an64_ref")):
        g_full = [sum(full[("full", v, ex)][k] for v in range(V)) for k in range(4)]
        base = chain_to_parameters(case, g_full)
        for i, r in enumerate(out):
            a = float(base[r["name"]][r["flat"]])
            for v in range(V):
                if (i, v, ex) in corr:
                    a -= float(chain_to_parameters(case, corr[(i, v, ex)])[r["name"]][r["flat"]])
            r[key] = a
    return case, out


def parameter_list(case, blocks_full=None):
    """(name, flat index) of every parameter (or every parameter of the
    blocks in ``blocks_full`` plus the exponents and occupancy of all)."""
    inp = case["inp"]
    out = []
    for name in NAMES:
        t = inp[name]
        per = t.numel() // case["B"]
        for flat in range(t.numel()):
            b = flat // per
            if blocks_full is None or b in blocks_full or name in ("sq_eps", "sq_occ"):
                out.append((name, flat))
    return out


def finite_differences(case_kwargs, params, h=1e-6, procs=None):
    """Central differences of the loss for each (name, flat index) in
    ``params``.  Returns a list of dicts: fd (all pixels), flips (their
    count), and per view the flat indices of the pixels the block's tiles
    cover, their difference quotients, and the flip mask (pixels whose
    decisions differ between +h and -h)."""
    procs = procs or min(16, os.cpu_count() or 1)
    jobs = [(n, f, s * h) for n, f in params for s in (1, -1)]
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs, initializer=_init, initargs=(case_kwargs,)) as pool:
        res = pool.map(_eval, jobs, chunksize=1)
    out = []
    for i, (n, f) in enumerate(params):
        plus, minus = res[2 * i], res[2 * i + 1]
        views = []
        total = 0.0
        for (idx, vp, sp), (_, vm, sm) in zip(plus, minus):
            q = (vp - vm) / (2 * h)
            views.append(dict(pixels=idx, quotient=q, flip=sp != sm))
            total += float(q.sum())
        out.append(dict(name=n, flat=f, fd=total, views=views, flips=int(sum(v["flip"].sum() for v in views))))
    return out
