"""Point-set proposal network for the block-level stage (BF16 tensor-core
MLP, trained with the project's own kernels).

From 2,048 points back-projected from a rendered median depth map
(``sq_data.SceneRenderer``) the network proposes up to eight superquadrics
to initialise the block-level fit:

    per point   3 -> 64 -> 128 -> 256   (shared weights, ReLU)
    max-pool over the points
    head        256 -> 256 (ReLU) -> 8 x 13

Each slot's 13 outputs are semi-axes (3; 0.1 + 0.4 sigmoid), exponents
(2; 0.2 + 1.6 sigmoid), a quaternion (4; normalised), a centre (3) and an
existence logit (1).  Every layer, forward and backward, runs on the tcgen05
GEMM of ``proposal_gemm`` (BF16 operands, FP32 accumulation, fused bias /
ReLU / ReLU-mask epilogues, split-K atomics for the weight gradients); the
max-pool and its backward are CUDA kernels of the same library; the weights
are FP32 masters updated by the one-launch Adam (``optim.SurfelAdam``) with
BF16 copies refreshed after each step.  The loss and its gradient on the
8 x 13 outputs are small PyTorch operations.

The method without the network is the reference's initialisation
(games/block_mesh_splatting/scene/dataset_readers.py:137-150,
utils/superquadric.py:112-120): k-means clusters of the points, one
superquadric per cluster at the cluster mean with identity rotation,
exponents 1 (sq_eps = 0) and sq_s = log(ratio), i.e. semi-axes
ratio * (ratio + scale_block_min) = 0.1125.
"""
from __future__ import annotations

import ctypes as C
import math

import torch
import torch.nn.functional as F

from . import _lib as L
from . import proposal_gemm as G
from .optim import SurfelAdam
from .sq_data import MAX_SQ, RATIO, SMIN, SQBatch, surface_samples

IN_PAD = 16                       # the 3 coordinates, padded to the MMA's K step
SLOT = 13
LAYERS = ((IN_PAD, 64), (64, 128), (128, 256), (256, 256), (256, SLOT * MAX_SQ))
SPLIT_K = 8192                    # point rows per CTA in the weight-gradient GEMMs


def _pool_lib():
    lib = L.load()
    lib.sgr_mlp_maxpool.restype = C.c_int
    lib.sgr_mlp_maxpool.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.c_void_p]
    lib.sgr_mlp_maxpool_backward.restype = C.c_int
    lib.sgr_mlp_maxpool_backward.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32,
                                             C.c_void_p, C.c_void_p]
    return lib


class ProposalNet:
    def __init__(self, device="cuda", seed: int = 0):
        self.dev = torch.device(device)
        g = torch.Generator().manual_seed(seed)
        self.W, self.b = [], []
        for i, (fin, fout) in enumerate(LAYERS):
            real_in = 3 if i == 0 else fin
            bound = 1.0 / math.sqrt(real_in)
            W = (torch.rand(fout, fin, generator=g) * 2 - 1) * bound
            if i == 0:
                W[:, 3:] = 0.0
            b = (torch.rand(fout, generator=g) * 2 - 1) * bound
            self.W.append(W.to(self.dev).requires_grad_(True))
            self.b.append(b.to(self.dev).requires_grad_(True))
        for t in self.W + self.b:
            t.grad = torch.zeros_like(t)
        self.refresh()

    def parameters(self):
        return self.W + self.b

    def refresh(self):
        """BF16 copies of the weights, [out, in] and [in, out]."""
        with torch.no_grad():
            self.Wb = [W.detach().to(torch.bfloat16).contiguous() for W in self.W]
            self.WTb = [W.detach().t().contiguous().to(torch.bfloat16) for W in self.W]

    def state_dict(self):
        return {"W": [w.detach().cpu() for w in self.W], "b": [b.detach().cpu() for b in self.b]}

    def load_state_dict(self, sd):
        with torch.no_grad():
            for dst, src in zip(self.W + self.b, sd["W"] + sd["b"]):
                dst.copy_(src)
        self.refresh()

    def forward(self, pts: torch.Tensor):
        """pts [S, P, 3] -> raw outputs [S, 104] (fp32) and the saved
        activations for ``backward``."""
        S, P, _ = pts.shape
        M = S * P
        bf = torch.bfloat16
        x0 = torch.zeros(M, IN_PAD, dtype=bf, device=self.dev)
        x0[:, :3] = pts.reshape(M, 3).to(bf)
        h1 = torch.empty(M, 64, dtype=bf, device=self.dev)
        h2 = torch.empty(M, 128, dtype=bf, device=self.dev)
        h3 = torch.empty(M, 256, dtype=bf, device=self.dev)
        G.gemm(x0, self.Wb[0], h1, G.RELU_BF16, bias=self.b[0].detach())
        G.gemm(h1, self.Wb[1], h2, G.RELU_BF16, bias=self.b[1].detach())
        G.gemm(h2, self.Wb[2], h3, G.RELU_BF16, bias=self.b[2].detach())
        g = torch.empty(S, 256, device=self.dev)
        gb = torch.empty(S, 256, dtype=bf, device=self.dev)
        arg = torch.empty(S, 256, dtype=torch.int32, device=self.dev)
        L.check(_pool_lib().sgr_mlp_maxpool(h3.data_ptr(), S, P, 256, g.data_ptr(), gb.data_ptr(), arg.data_ptr(),
                                            torch.cuda.current_stream().cuda_stream), "sgr_mlp_maxpool")
        h4 = torch.empty(S, 256, dtype=bf, device=self.dev)
        G.gemm(gb, self.Wb[3], h4, G.RELU_BF16, bias=self.b[3].detach())
        out = torch.empty(S, SLOT * MAX_SQ, device=self.dev)
        G.gemm(h4, self.Wb[4], out, G.STORE_F32, bias=self.b[4].detach())
        return out, (S, P, x0, h1, h2, h3, g, gb, arg, h4)

    def backward(self, cache, dout: torch.Tensor):
        """Adds the weight and bias gradients of dout [S, 104] to the
        parameters' ``.grad`` buffers (the optimiser clears them)."""
        S, P, x0, h1, h2, h3, g, gb, arg, h4 = cache
        M = S * P
        bf = torch.bfloat16
        gW = [w.grad for w in self.W]
        gB = [b.grad for b in self.b]
        d5 = dout.to(bf).contiguous()
        G.gemm(d5, h4, gW[4], G.ADD_F32, trans=True)
        gB[4] += dout.sum(0)
        dz4 = torch.empty(S, 256, dtype=bf, device=self.dev)
        G.gemm(d5, self.WTb[4], dz4, G.MASK_BF16, mask=h4)
        G.gemm(dz4, gb, gW[3], G.ADD_F32, trans=True)
        gB[3] += dz4.float().sum(0)
        dg = torch.empty(S, 256, device=self.dev)
        G.gemm(dz4, self.WTb[3], dg, G.STORE_F32)
        dz3 = torch.empty(M, 256, dtype=bf, device=self.dev)
        L.check(_pool_lib().sgr_mlp_maxpool_backward(dg.data_ptr(), g.data_ptr(), arg.data_ptr(), S, P, 256,
                                                     dz3.data_ptr(), torch.cuda.current_stream().cuda_stream),
                "sgr_mlp_maxpool_backward")
        G.gemm(dz3, h2, gW[2], G.ADD_F32, trans=True, split_k=SPLIT_K)
        gB[2] += dz3.float().sum(0)
        dz2 = torch.empty(M, 128, dtype=bf, device=self.dev)
        G.gemm(dz3, self.WTb[2], dz2, G.MASK_BF16, mask=h2)
        G.gemm(dz2, h1, gW[1], G.ADD_F32, trans=True, split_k=SPLIT_K)
        gB[1] += dz2.float().sum(0)
        dz1 = torch.empty(M, 64, dtype=bf, device=self.dev)
        G.gemm(dz2, self.WTb[1], dz1, G.MASK_BF16, mask=h1)
        G.gemm(dz1, x0, gW[0], G.ADD_F32, trans=True, split_k=SPLIT_K)
        gB[0] += dz1.float().sum(0)


def decode(out: torch.Tensor):
    """Raw outputs [S, 104] -> (semi [S,8,3], eps [S,8,2], quat [S,8,4],
    trans [S,8,3], exist logit [S,8])."""
    r = out.reshape(out.shape[0], MAX_SQ, SLOT)
    semi = 0.1 + 0.4 * torch.sigmoid(r[..., 0:3])
    eps = 0.2 + 1.6 * torch.sigmoid(r[..., 3:5])
    quat = F.normalize(r[..., 5:9], dim=-1)
    return semi, eps, quat, r[..., 9:12], r[..., 12]


def _pair_costs(semi, eps, quat, trans, t):
    """[S, 8 predicted, 8 target] costs of assigning slots to superquadrics."""
    d = lambda a, b: ((a[:, :, None, :] - b[:, None, :, :]) ** 2).sum(-1)  # noqa: E731
    return (4.0 * d(semi, t[0]) + 0.5 * d(eps, t[1]) +
            (1.0 - (quat[:, :, None, :] * t[2][:, None, :, :]).sum(-1).abs()) + 4.0 * d(trans, t[3]))


def slot_loss(out: torch.Tensor, target: SQBatch):
    """Set loss: per scene the predicted slots are matched to the target's
    superquadrics by minimum total cost (Hungarian assignment); matched slots
    should exist and carry the weighted squared errors of semi-axes,
    exponents and centres and 1 - |<q, q*>| of the rotation; the others
    should not exist."""
    from scipy.optimize import linear_sum_assignment
    semi, eps, quat, trans, logit = decode(out)
    t = [x.to(out.device) for x in (target.semi, target.eps, target.quat, target.trans, target.exist)]
    cost = _pair_costs(semi, eps, quat, trans, t)
    cost_host = cost.detach().cpu().numpy()
    counts = target.exist.sum(1).long().tolist()
    S = out.shape[0]
    rows, cols, scene = [], [], []
    for s in range(S):
        k = counts[s]
        r, c = linear_sum_assignment(cost_host[s, :, :k])
        rows += r.tolist()
        cols += c.tolist()
        scene += [s] * len(r)
    scene_t = torch.tensor(scene, device=out.device)
    rows_t = torch.tensor(rows, device=out.device)
    cols_t = torch.tensor(cols, device=out.device)
    exist = torch.zeros_like(logit)
    exist[scene_t, rows_t] = 1.0
    l_exist = F.binary_cross_entropy_with_logits(logit, exist)
    return l_exist + cost[scene_t, rows_t, cols_t].sum() / max(1, len(rows))


class Trainer:
    """Adam (one launch) on the network's FP32 master weights."""

    def __init__(self, net: ProposalNet, lr: float = 1e-3):
        self.net = net
        self.opt = SurfelAdam([{"params": [p], "lr": lr} for p in net.parameters()], eps=1e-8)

    def step(self, pts: torch.Tensor, target: SQBatch) -> float:
        """One training step; raises if a tensor-core GEMM of its forward or
        backward ran out of time (before the optimiser uses its gradients)."""
        out, cache = self.net.forward(pts)
        o = out.detach().requires_grad_(True)
        loss = slot_loss(o, target)
        (dout,) = torch.autograd.grad(loss, o)
        self.net.backward(cache, dout.contiguous())
        G.check_status(pts.device)
        self.opt.step()
        self.net.refresh()
        return loss.detach()


def predict(net: ProposalNet, pts: torch.Tensor, threshold: float = 0.5, counts=None):
    """Per scene, the proposed superquadrics: a list of (semi, eps, quat,
    trans) tensors [k, .].  With ``counts`` (the configured number of blocks
    per scene, as the reference's block stage is given) the k most likely
    slots; otherwise the slots with existence probability above
    ``threshold`` (at least one)."""
    out, _ = net.forward(pts)
    G.check_status(pts.device)          # raises if a GEMM's wait ran out
    semi, eps, quat, trans, logit = decode(out)
    res = []
    for s in range(out.shape[0]):
        if counts is not None:
            keep = logit[s].argsort(descending=True)[:int(counts[s])]
        else:
            keep = torch.sigmoid(logit[s]) > threshold
            if not bool(keep.any()):
                keep = logit[s] == logit[s].max()
        res.append((semi[s][keep], eps[s][keep], quat[s][keep], trans[s][keep]))
    return res


def kmeans(points: torch.Tensor, k: int, iters: int = 20, g: torch.Generator | None = None):
    """Cluster centres of points [n, 3] (k-means++ seeding, Lloyd steps)."""
    n = points.shape[0]
    g = g or torch.Generator().manual_seed(0)
    first = int(torch.randint(n, (1,), generator=g))
    centres = [points[first]]
    for _ in range(1, k):
        d = torch.cdist(points, torch.stack(centres)).min(dim=1).values ** 2
        w = (d / d.sum().clamp(min=1e-12)).cpu()
        centres.append(points[int(torch.multinomial(w, 1, generator=g))])
    c = torch.stack(centres)
    for _ in range(iters):
        lab = torch.cdist(points, c).argmin(dim=1)
        for j in range(k):
            sel = lab == j
            if bool(sel.any()):
                c[j] = points[sel].mean(0)
    return c


def kmeans_batch(points: torch.Tensor, counts, iters: int = 20, seed: int = 0):
    """Per scene s of points [S, n, 3], counts[s] k-means centres (k-means++
    seeding, Lloyd steps), all scenes at once on the device: [S, 8, 3], the
    slots past counts[s] zero."""
    S, n, _ = points.shape
    dev = points.device
    K = MAX_SQ
    k = torch.as_tensor(counts, device=dev).long()
    g = torch.Generator(device=dev).manual_seed(seed)
    ar = torch.arange(S, device=dev)
    pts = points.float()
    centres = torch.zeros(S, K, 3, device=dev)
    first = torch.randint(n, (S,), generator=g, device=dev)
    centres[:, 0] = pts[ar, first]
    d = ((pts - centres[:, :1]) ** 2).sum(-1)
    for j in range(1, K):
        w = d / d.sum(1, keepdim=True).clamp(min=1e-12)
        w = torch.where(w.sum(1, keepdim=True) > 0, w, torch.ones_like(w))
        pick = torch.multinomial(w, 1, generator=g).squeeze(1)
        centres[:, j] = pts[ar, pick]
        d = torch.minimum(d, ((pts - centres[:, j:j + 1]) ** 2).sum(-1))
    slot_on = torch.arange(K, device=dev)[None, :] < k[:, None]             # [S, K]
    for _ in range(iters):
        dist = torch.cdist(pts, centres)                                      # [S, n, K]
        dist = dist.masked_fill(~slot_on[:, None, :], float("inf"))
        onehot = torch.nn.functional.one_hot(dist.argmin(-1), K).float()     # [S, n, K]
        num = onehot.sum(1)                                                   # [S, K]
        sums = onehot.transpose(1, 2) @ pts                                   # [S, K, 3]
        centres = torch.where((num > 0)[..., None], sums / num.clamp(min=1)[..., None], centres)
    return centres * slot_on[..., None]


def plain_init_batch(points: torch.Tensor, counts, seed: int = 0):
    """plain_init for every scene of points [S, n, 3] at once (the k-means
    of kmeans_batch): a list of (semi, eps, quat, trans) per scene."""
    c = kmeans_batch(points, counts, seed=seed)
    out = []
    for s, k in enumerate(counts):
        k = int(k)
        semi = torch.full((k, 3), RATIO * (RATIO + SMIN), device=points.device)
        eps = torch.ones(k, 2, device=points.device)
        quat = torch.tensor([1.0, 0.0, 0.0, 0.0], device=points.device).expand(k, 4)
        out.append((semi, eps, quat, c[s, :k]))
    return out


def plain_init(points: torch.Tensor, k: int, g: torch.Generator | None = None):
    """The reference's block initialisation for k blocks (utils/superquadric.py:
    112-120): k-means centres, identity rotation, sq_eps = 0 (exponents 1.0)
    and sq_s = log(ratio), i.e. semi-axes ratio * (ratio + scale_block_min)."""
    c = kmeans(points, k, g=g)
    semi = torch.full((k, 3), RATIO * (RATIO + SMIN), device=points.device)
    eps = torch.ones(k, 2, device=points.device)
    quat = torch.tensor([1.0, 0.0, 0.0, 0.0], device=points.device).expand(k, 4)
    return semi, eps, quat, c


def chamfer(a: torch.Tensor, b: torch.Tensor) -> float:
    """Symmetric mean nearest-neighbour distance between point sets."""
    d = torch.cdist(a, b)
    return float(0.5 * (d.min(dim=1).values.mean() + d.min(dim=0).values.mean()))


def set_chamfer(pred, target_semi, target_eps, target_quat, target_trans, n: int = 256, seed: int = 0):
    """Chamfer distance between the surfaces of a predicted and a target set
    of superquadrics (n samples per superquadric)."""
    g = torch.Generator().manual_seed(seed)
    semi, eps, quat, trans = (t.detach().float().cpu() for t in pred)
    pa = surface_samples(semi, eps, quat, trans, n, g).reshape(-1, 3)
    pb = surface_samples(target_semi.float().cpu(), target_eps.float().cpu(), target_quat.float().cpu(),
                         target_trans.float().cpu(), n, g).reshape(-1, 3)
    return chamfer(pa, pb)
