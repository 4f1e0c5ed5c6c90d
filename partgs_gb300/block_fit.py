"""Block-level superquadric fit and the time-to-Chamfer comparison of its two
initialisations.

The fit optimises each superquadric's log semi-axes, exponent logits,
rotation and centre (the block model's sq_s, sq_eps, sq_r, sq_t with the
reference's learning rates 5e-3 / 1e-3 / 5e-3 / 5e-3 and Adam eps 1e-15,
games/block_mesh_splatting/scene/block_gaussian_model.py:430-442) through
the CUDA binding and rasteriser, so that the union's silhouettes and median
depth maps match those of the target scene from V orbit cameras.  (The
reference fits RGB images with photometric losses; the synthetic scenes
here carry geometry only, so the geometric maps stand in for them.)

``time_to_chamfer`` runs the fit from the reference's initialisation
(k-means blocks, ``proposal.plain_init``) and from the proposal network's,
and reports how long each takes to reach the Chamfer distance the plain fit
ends at.
"""
from __future__ import annotations

import os
import time

import torch

from . import _lib as L
from .batched import MultiViewRasterizer
from .binding import SuperquadricBinding
from .cameras import orbit_cameras
from .optim import SurfelAdam
from .proposal import chamfer
from .sq_data import RATIO, SMIN, grid_topology, surface_samples, to_binding_params

LR = {"sq_s": 5e-3, "sq_eps": 1e-3, "sq_r": 5e-3, "sq_t": 5e-3}


class BlockFit:
    def __init__(self, target, views: int = 8, res: int = 96, n_eta: int = 30, n_omega: int = 30, seed: int = 0,
                 device="cuda"):
        """target: (semi [K,3], eps [K,2], quat [K,4], trans [K,3])."""
        self.dev = torch.device(device)
        self.cams = orbit_cameras(views, 3.0, res, res, 50.0, seed=seed)
        eta, omega, faces = grid_topology(n_eta, n_omega)
        self.eta = torch.tensor(eta, dtype=torch.float32, device=self.dev)
        self.omega = torch.tensor(omega, dtype=torch.float32, device=self.dev)
        self.faces = torch.tensor(faces, dtype=torch.int32, device=self.dev)
        self.F = faces.shape[0]
        self.seed = seed
        self._rasters, self._bindings = {}, {}
        g = torch.Generator().manual_seed(seed)
        self.target = [t.float() for t in target]
        self.target_pts = surface_samples(*self.target, 256, g).reshape(-1, 3)
        with torch.no_grad():
            others = self.render(*(t.to(self.dev) for t in to_binding_params(*self.target)))
        self.alpha_t = others[:, 1].detach()
        self.depth_t = others[:, 5].detach()
        self.mask_t = (self.alpha_t > 0.5).float()

    def _parts(self, K):
        """The binding topology and the rasteriser of K superquadrics (built once)."""
        if K not in self._bindings:
            g = torch.Generator().manual_seed(self.seed + 7)
            alpha = torch.rand(K * self.F, 1, 3, generator=g).to(self.dev)
            self._bindings[K] = SuperquadricBinding(self.eta.expand(K, -1), self.omega.expand(K, -1),
                                                    self.faces.expand(K, -1, -1).contiguous(), alpha,
                                                    torch.ones(K, self.F, 1, device=self.dev), RATIO, SMIN)
            self._rasters[K] = MultiViewRasterizer(self.cams, [0.0, 0.0, 0.0], 0, num_surfels=K * self.F,
                                                   device=self.dev)
        return self._bindings[K], self._rasters[K]

    def render(self, sq_s, sq_eps, sq_r, sq_t):
        K = sq_s.shape[0]
        bind, raster = self._parts(K)
        occ = torch.full((K, 1), 4.6, device=self.dev)
        xyz, log_s, rot, op = bind(sq_s, sq_r, sq_t, sq_eps, occ)
        _, others, _, _ = raster(xyz, op, None, torch.exp(log_s), rot, colors_precomp=torch.ones_like(xyz))
        return others

    def fit(self, init, iters: int = 300, eval_every: int = 10, reg: bool = False):
        """Runs the fit from init (semi, eps, quat, trans); returns
        [(fit seconds so far, Chamfer distance to the target)].  With ``reg``
        the block model's regularisers are added as summarize_losses adds
        them (block_gaussian_model.py:584-648): ray coverage and uncoverage,
        occupancy BCE and overlap against the target silhouettes, one view's
        2048 rays x 128 samples per iteration, with the reference's weights."""
        raw = [t.detach().float().to(self.dev).clone().contiguous() for t in to_binding_params(*init)]
        sq_s, sq_eps, sq_r, sq_t = (t.requires_grad_(True) for t in raw)
        opt = SurfelAdam([{"params": [sq_s], "lr": LR["sq_s"]}, {"params": [sq_eps], "lr": LR["sq_eps"]},
                          {"params": [sq_r], "lr": LR["sq_r"]}, {"params": [sq_t], "lr": LR["sq_t"]}], eps=1e-15)
        hist = [(0.0, self.chamfer_of(sq_s, sq_eps, sq_r, sq_t))]
        elapsed = 0.0
        self.last_reg = None
        if reg:
            from . import sq_losses as Q
            gen = torch.Generator(device=self.dev).manual_seed(self.seed + 23)
            occ = torch.full((sq_s.shape[0],), 4.6, device=self.dev)   # the fit's fixed block opacity logit
            weights = torch.tensor([10.0, 100.0, 0.02, 2.0], device=self.dev)
            Ks = [Q.intrinsics(c.height, c.width, c.fovx, c.fovy, self.dev) for c in self.cams]
            wvs = [torch.as_tensor(c.world_view_transform, device=self.dev) for c in self.cams]
        it = 0
        for it0 in range(0, iters, eval_every):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(min(eval_every, iters - it0)):
                others = self.render(sq_s, sq_eps, sq_r, sq_t)
                loss = (others[:, 1] - self.alpha_t).abs().mean() + \
                    (self.mask_t * (others[:, 5] - self.depth_t).abs()).mean()
                if reg:
                    v = it % len(self.cams)
                    c = self.cams[v]
                    rays = Q.cast_rays(Ks[v], wvs[v], c.height, c.width, self.mask_t[v], *Q.NEAR_FAR["blender"],
                                       generator=gen)
                    ovl = Q.overlap_samples(sq_s.shape[0], device=self.dev, generator=gen)
                    S, R, T, e1, e2 = Q.block_frames(sq_s, sq_r, sq_t, sq_eps, SMIN)
                    terms = Q.sq_losses(S, R, T, e1, e2, occ, RATIO, rays, ovl)
                    loss = loss + (weights * terms.nan_to_num(0.0)).sum()
                    self.last_reg = terms.detach()
                it += 1
                loss.backward()
                opt.step()
            torch.cuda.synchronize()
            elapsed += time.perf_counter() - t0
            hist.append((elapsed, self.chamfer_of(sq_s, sq_eps, sq_r, sq_t)))
        self.last_params = [t.detach() for t in (sq_s, sq_eps, sq_r, sq_t)]
        return hist

    def chamfer_of(self, sq_s, sq_eps, sq_r, sq_t):
        with torch.no_grad():
            semi = RATIO * (torch.exp(sq_s) + SMIN)
            eps = torch.sigmoid(sq_eps) * 1.8 + 0.1
            quat = torch.nn.functional.normalize(sq_r, dim=-1)
            g = torch.Generator().manual_seed(self.seed + 11)
            pts = surface_samples(semi.cpu(), eps.cpu(), quat.cpu(), sq_t.detach().cpu(), 256, g).reshape(-1, 3)
        return chamfer(pts, self.target_pts)


class BatchFit:
    """The block-level fit of many scenes at once.  Every scene's blocks are
    bound in one binding call and all scenes' views are rasterised in one
    multi-scene launch sequence per iteration (the uneven-batch path of the
    rasteriser: scene s carries K_s x F surfels and its own V cameras).  A
    scene's loss is exactly BlockFit's (silhouette and masked median-depth L1,
    each a mean over its views' pixels), the scenes' losses are summed, and
    Adam is element-wise, so every scene follows the trajectory its own
    BlockFit (same seed, views and resolution) would, up to the FP32 order
    of the gradient atomics.

    targets: a list of (semi [K,3], eps [K,2], quat [K,4], trans [K,3]), one
    per scene; seeds: the per-scene seeds BlockFit would take (cameras and
    surfel barycentres)."""

    def __init__(self, targets, seeds, views: int = 8, res: int = 96, n_eta: int = 30, n_omega: int = 30,
                 device="cuda"):
        self.dev = torch.device(device)
        self.S = len(targets)
        self.K = [int(t[0].shape[0]) for t in targets]
        self.views = views
        eta, omega, faces = grid_topology(n_eta, n_omega)
        F = faces.shape[0]
        B = sum(self.K)
        alpha = torch.cat([torch.rand(k * F, 1, 3, generator=torch.Generator().manual_seed(int(sd) + 7))
                           for k, sd in zip(self.K, seeds)]).to(self.dev)
        self.bind = SuperquadricBinding(torch.tensor(eta, dtype=torch.float32, device=self.dev).expand(B, -1),
                                        torch.tensor(omega, dtype=torch.float32, device=self.dev).expand(B, -1),
                                        torch.tensor(faces, dtype=torch.int32, device=self.dev).expand(B, -1, -1)
                                        .contiguous(), alpha, torch.ones(B, F, 1, device=self.dev), RATIO, SMIN)
        cams = [c for sd in seeds for c in orbit_cameras(views, 3.0, res, res, 50.0, seed=int(sd))]
        self.raster = MultiViewRasterizer(cams, [0.0, 0.0, 0.0], 0, scene_sizes=[k * F for k in self.K],
                                          scene_views=[views] * self.S, device=self.dev)
        self.occ = torch.full((B, 1), 4.6, device=self.dev)
        with torch.no_grad():
            others = self.render(*self.raw(targets))
        self.alpha_t = others[:, 1].detach()
        self.depth_t = others[:, 5].detach()
        self.mask_t = (self.alpha_t > 0.5).float()

    def raw(self, sets):
        """Concatenated block-model parameters (sq_s, sq_eps, sq_r, sq_t) of
        per-scene (semi, eps, quat, trans) sets."""
        parts = [to_binding_params(*(t.float() for t in st)) for st in sets]
        return [torch.cat([p[i] for p in parts]).to(self.dev).contiguous() for i in range(4)]

    def render(self, sq_s, sq_eps, sq_r, sq_t):
        xyz, log_s, rot, op = self.bind(sq_s, sq_r, sq_t, sq_eps, self.occ)
        _, others, _, _ = self.raster(xyz, op, None, torch.exp(log_s), rot, colors_precomp=torch.ones_like(xyz))
        return others

    def loss(self, others):
        """Per scene: BlockFit's loss; [S]."""
        la = (others[:, 1] - self.alpha_t).abs().mean(dim=(1, 2))
        ld = (self.mask_t * (others[:, 5] - self.depth_t).abs()).mean(dim=(1, 2))
        return (la + ld).reshape(self.S, self.views).mean(1)

    def fit(self, init, iters: int, capture: bool = False, headroom: float = 1.5):
        """Runs the fit from per-scene init sets; returns the fitted sets
        [(semi, eps, quat, trans)] (quaternions normalised, w >= 0) and the
        per-scene loss of the last iteration.  With ``capture`` one iteration
        (binding, rasteriser, loss, backward, Adam) is captured in a CUDA
        graph after an eager first iteration has sized the cell lists
        (``headroom`` times its entry count), and replayed; if a replay
        overflowed the lists, the fit runs again eagerly from the start."""
        raw = [t.detach().clone() for t in self.raw(init)]

        def run(graphed):
            params = [t.clone().requires_grad_(True) for t in raw]
            sq_s, sq_eps, sq_r, sq_t = params
            opt = SurfelAdam([{"params": [sq_s], "lr": LR["sq_s"]}, {"params": [sq_eps], "lr": LR["sq_eps"]},
                              {"params": [sq_r], "lr": LR["sq_r"]}, {"params": [sq_t], "lr": LR["sq_t"]}],
                             eps=1e-15)

            def step():
                per_scene = self.loss(self.render(*params))
                per_scene.sum().backward()
                opt.step()
                return per_scene.detach()

            if not graphed:
                self.raster.set_capacity(None)
                last = None
                for _ in range(iters):
                    last = step()
                return params, last, True
            side = torch.cuda.Stream()
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(side):
                self.raster.set_capacity(None)
                last = step()                       # iteration 1, eager: sizes the lists
                side.synchronize()
                most = self.raster.counts()[2]
            torch.cuda.current_stream().wait_stream(side)
            self.raster.set_capacity(int(most * headroom) + 4096)
            graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(graph):
                out = step()
            self.raster.sticky_counts(reset=True)
            for _ in range(iters - 1):
                graph.replay()
            flags, _ = self.raster.sticky_counts(reset=True)
            self.raster.set_capacity(None)
            return params, out.clone(), not (flags & L.SGR_FLAG_BIN_OVERFLOW)

        params, last, ok = run(capture and iters > 1)
        if not ok:
            params, last, ok = run(False)
        sq_s, sq_eps, sq_r, sq_t = params
        with torch.no_grad():
            semi = RATIO * (torch.exp(sq_s) + SMIN)
            eps = torch.sigmoid(sq_eps) * 1.8 + 0.1
            quat = torch.nn.functional.normalize(sq_r, dim=-1)
            quat = torch.where(quat[:, :1] < 0, -quat, quat)
            out, o = [], 0
            for k in self.K:
                out.append((semi[o:o + k], eps[o:o + k], quat[o:o + k], sq_t.detach()[o:o + k]))
                o += k
        return out, last


def time_to_reach(hist, level):
    """Fit seconds until the Chamfer distance first reaches ``level`` (None if never)."""
    for t, c in hist:
        if c <= level:
            return t
    return None


def time_to_chamfer(net, batch, points, iters: int = 300, views: int = 8, res: int = 96):
    """Per scene of ``batch`` (an SQBatch with its ``points`` [S, 2048, 3]):
    plain-init and proposal-init fits with the same, configured number of
    blocks (the reference's block stage is given it; k-means uses it, the
    proposal keeps its k most likely slots); the plain fit's final Chamfer is
    the level both are timed to.  The proposal's time includes its network
    forward.  Returns a list of dicts."""
    from .proposal import plain_init, predict
    out = []
    for s in range(points.shape[0]):
        k = int(batch.counts[s])
        target = (batch.semi[s, :k], batch.eps[s, :k], batch.quat[s, :k], batch.trans[s, :k])
        fit = BlockFit(target, views=views, res=res, seed=s)
        plain = plain_init(points[s].float(), k, g=torch.Generator().manual_seed(s))
        h_plain = fit.fit(plain, iters)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        prop = predict(net, points[s:s + 1].contiguous(), counts=[k])[0]
        torch.cuda.synchronize()
        t_net = time.perf_counter() - t0
        h_prop = fit.fit(prop, iters)
        level = h_plain[-1][1]
        t_prop = time_to_reach(h_prop, level)
        out.append(dict(k=k, k_proposed=int(prop[0].shape[0]), plain_final=level, plain_time=h_plain[-1][0],
                        proposal_start=h_prop[0][1], plain_start=h_plain[0][1], proposal_final=h_prop[-1][1],
                        proposal_time=None if t_prop is None else t_prop + t_net, network_s=t_net))
    return out


def summarize(res, budget_iters: int):
    """Population figures of time_to_chamfer results.  A scene whose
    proposal-initialised fit never reaches the plain fit's final Chamfer
    within the same iteration budget counts with ratio infinity (a failure),
    so the median and p90 are over every scene; ``target_met`` says whether
    the median ratio is at most 1/3."""
    import math

    import numpy as np
    ratios = [r["proposal_time"] / r["plain_time"] if r["proposal_time"] is not None else math.inf for r in res]
    srt = np.sort(np.array(ratios))
    med = float(np.median(srt))
    p90 = float(np.percentile(srt, 90, method="higher"))
    fin = lambda x: x if math.isfinite(x) else None  # noqa: E731
    return {
        "scenes": len(res), "iters": budget_iters,
        "reached": int(sum(r["proposal_time"] is not None for r in res)),
        "time_ratio_median_all": fin(med), "time_ratio_p90_all": fin(p90),
        "scenes_at_most_one_third": int(sum(x <= 1 / 3 for x in ratios)),
        "target_met": bool(med <= 1 / 3),
        "plain_start_chamfer": float(np.mean([r["plain_start"] for r in res])),
        "proposal_start_chamfer": float(np.mean([r["proposal_start"] for r in res])),
        "plain_final_chamfer": float(np.mean([r["plain_final"] for r in res])),
        "proposal_final_chamfer": float(np.mean([r["proposal_final"] for r in res])),
        "proposal_final_below_plain": int(sum(r["proposal_final"] <= r["plain_final"] for r in res)),
        "plain_fit_s": float(np.mean([r["plain_time"] for r in res])),
        "network_s": float(np.mean([r["network_s"] for r in res])),
        "per_scene": [{"k": r["k"], "ratio": fin(x), "plain_final": round(r["plain_final"], 5),
                       "proposal_final": round(r["proposal_final"], 5)} for r, x in zip(res, ratios)]}


def main():
    """python -m partgs_gb300.block_fit --scenes 32 --iters 300 [--out F]:
    time to the plain fit's final Chamfer distance, proposal init against
    plain init, on seeded held-out scenes; prints (and writes) one JSON
    record with the population figures (``summarize``)."""
    import argparse
    import json

    from . import sq_data as D
    from .train_proposal import WEIGHTS, load_npz
    ap = argparse.ArgumentParser()
    ap.add_argument("--scenes", type=int, default=32)
    ap.add_argument("--iters", type=int, default=300)
    ap.add_argument("--seed", type=int, default=4242)
    ap.add_argument("--weights", default=WEIGHTS)
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
    net = load_npz(a.weights)
    b = D.sample_sq_batch(a.scenes, torch.Generator().manual_seed(a.seed))
    pts, _ = D.SceneRenderer(res=96).points(b, seed=a.seed)
    time_to_chamfer(net, b, pts[:1], iters=20)                     # warm-up (library load, first launches)
    res = time_to_chamfer(net, b, pts, iters=a.iters)
    rec = dict(summarize(res, a.iters), seed=a.seed, weights=os.path.basename(a.weights),
               command=f"python -m partgs_gb300.block_fit --scenes {a.scenes} --iters {a.iters} --seed {a.seed}")
    line = json.dumps(rec)
    print(line)
    if a.out:
        with open(a.out, "w") as f:
            f.write(json.dumps(rec, indent=1) + "\n")


if __name__ == "__main__":
    main()
