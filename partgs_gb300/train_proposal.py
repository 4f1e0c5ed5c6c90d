"""Trains the superquadric proposal network on synthetic scenes labelled by
the block-level fit, and writes its weights (``.npz``: W0..W4, b0..b4,
float32).

    python -m partgs_gb300.train_proposal --scenes 200000 --batch 256 --steps 12000 \
        --label-iters 300 --label-views 4 --out partgs_gb300/weights/proposal_sq8.npz

Scenes are drawn, rendered and back-projected on the GPU in chunks of 256
(``sq_data``).  Each chunk is then labelled by the block-level optimisation
itself (``label_chunk``): from the reference's initialisation (k-means
blocks of the scene's own points), ``block_fit.BatchFit`` fits all 256
scenes at once (one multi-scene rasteriser launch sequence per iteration)
for ``label_iters`` iterations against the scenes' silhouettes and median
depth from ``label_views`` views at 64x64 (a 20 x 20 surfel grid per block),
and the fitted blocks are the labels.  Training runs
the network's tensor-core forward and backward and the one-launch Adam
(``proposal.Trainer``).
"""
from __future__ import annotations

import argparse
import os
import time

import numpy as np
import torch

from . import sq_data as D
from .proposal import LAYERS, ProposalNet, Trainer

WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "proposal_sq8.npz")


def label_chunk(b: D.SQBatch, points: torch.Tensor, seeds, iters: int, res: int = 64, grid: int = 20,
                views: int = 8):
    """Replaces the chunk's labels (in place) by what the block-level fit
    reaches from the reference's initialisation: every scene starts from
    k-means blocks of its own points (proposal.plain_init_batch) and is
    fitted for ``iters`` iterations against its silhouettes and median depth
    (block_fit.BatchFit, all scenes at once); the fitted blocks, clamped into
    the ranges the network's outputs can take, are the labels.  Returns the
    mean absolute difference of the labels from the generating parameters
    (semi-axes, exponents, centres) and the mean final loss."""
    from .block_fit import BatchFit
    from .proposal import plain_init_batch
    counts = b.counts.tolist()
    targets = [(b.semi[s, :k], b.eps[s, :k], b.quat[s, :k], b.trans[s, :k]) for s, k in enumerate(counts)]
    init = plain_init_batch(points, counts, seed=int(seeds[0]))
    fit = BatchFit(targets, seeds, views=views, res=res, n_eta=grid, n_omega=grid)
    fitted, last = fit.fit(init, iters, capture=True)
    moved = []
    for s, (k, (semi, eps, quat, trans)) in enumerate(zip(counts, fitted)):
        semi, eps = semi.cpu().clamp(0.1001, 0.4999), eps.cpu().clamp(0.2001, 1.7999)
        quat, trans = quat.cpu(), trans.cpu()
        moved.append(torch.cat([(semi - b.semi[s, :k]).abs().reshape(-1), (eps - b.eps[s, :k]).abs().reshape(-1),
                                (trans - b.trans[s, :k]).abs().reshape(-1)]).mean())
        b.semi[s, :k], b.eps[s, :k], b.quat[s, :k], b.trans[s, :k] = semi, eps, quat, trans
    return float(torch.stack(moved).mean()), float(last.mean())


def make_dataset(num_scenes: int, seed: int = 0, res: int = 96, chunk: int = 256, label_iters: int = 0, log=None,
                 label_views: int = 4):
    """(points [N, 2048, 3] on the GPU, labels SQBatch on the host).  With
    ``label_iters`` > 0 the labels are block-level fits (``label_chunk``),
    else the generating parameters."""
    g = torch.Generator().manual_seed(seed)
    ren = D.SceneRenderer(res=res)
    pts, labels = [], []
    t0 = time.time()
    for i in range((num_scenes + chunk - 1) // chunk):
        b = D.sample_sq_batch(min(chunk, num_scenes - i * chunk), g)
        p, _ = ren.points(b, seed=seed * 100003 + i)
        if label_iters > 0:
            seeds = [seed * 1000003 + i * chunk + s for s in range(b.exist.shape[0])]
            moved, loss = label_chunk(b, p, seeds, label_iters, views=label_views)
            if log and (i % 64 == 0):
                log(f"labelled {i * chunk + b.exist.shape[0]} scenes: labels moved {moved:.4f} from the "
                    f"generating parameters, fit loss {loss:.4f}, {time.time() - t0:.0f}s")
        pts.append(p)
        labels.append(b)
    lab = D.SQBatch(*(torch.cat([getattr(x, f) for x in labels]) for f in ("semi", "eps", "quat", "trans", "exist")))
    return torch.cat(pts), lab


def train(num_scenes: int = 16384, steps: int = 8000, batch: int = 64, lr: float = 1e-3, seed: int = 0,
          log_every: int = 500, log=print, label_iters: int = 0, label_views: int = 4):
    pts, lab = make_dataset(num_scenes, seed, label_iters=label_iters, log=log, label_views=label_views)
    net = ProposalNet(seed=seed)
    tr = Trainer(net, lr=lr)
    g = torch.Generator().manual_seed(seed + 1)
    hist = []
    t0 = time.time()
    for it in range(steps):
        sel = torch.randint(0, pts.shape[0], (batch,), generator=g)
        sub = D.SQBatch(*(t[sel] for t in (lab.semi, lab.eps, lab.quat, lab.trans, lab.exist)))
        hist.append(tr.step(pts[sel.to(pts.device)].contiguous(), sub))
        if log and (it % log_every == 0 or it == steps - 1):
            recent = torch.stack(hist[-log_every:]).mean()
            log(f"step {it} loss {float(recent):.4f} {time.time() - t0:.1f}s")
    return net, [float(h) for h in hist]


def save_npz(net: ProposalNet, path: str):
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    arrays = {f"W{i}": w.detach().cpu().numpy() for i, w in enumerate(net.W)}
    arrays.update({f"b{i}": b.detach().cpu().numpy() for i, b in enumerate(net.b)})
    np.savez(path, **arrays)


def load_npz(path: str = WEIGHTS, device="cuda") -> ProposalNet:
    z = np.load(path)
    net = ProposalNet(device=device)
    net.load_state_dict({"W": [torch.from_numpy(z[f"W{i}"]) for i in range(len(LAYERS))],
                         "b": [torch.from_numpy(z[f"b{i}"]) for i in range(len(LAYERS))]})
    return net


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--scenes", type=int, default=200000)
    ap.add_argument("--steps", type=int, default=12000)
    ap.add_argument("--batch", type=int, default=256)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--label-iters", type=int, default=300,
                    help="block-level fit iterations per label (0: the generating parameters)")
    ap.add_argument("--label-views", type=int, default=4, help="views of each labelling fit (64x64)")
    ap.add_argument("--out", default=WEIGHTS)
    a = ap.parse_args()
    t0 = time.time()
    net, _ = train(a.scenes, a.steps, a.batch, a.lr, a.seed, label_iters=a.label_iters, label_views=a.label_views)
    print(f"trained in {time.time() - t0:.0f}s")
    save_npz(net, a.out)
    print("wrote", a.out)


if __name__ == "__main__":
    main()
