"""Trains the superquadric proposal network on synthetic scenes labelled by
the block-level fit, and writes its weights (``.npz``: W0..W4, b0..b4,
float32).

    python -m partgs_gb300.train_proposal --scenes 200000 --batch 256 --steps 12000 \
        --label-iters 50 --out partgs_gb300/weights/proposal_sq8.npz

Scenes are drawn, rendered and back-projected on the GPU in chunks of 256
(``sq_data``).  Each chunk is then labelled by the block-level optimisation
itself: ``block_fit.BatchFit`` fits all 256 scenes at once (one multi-scene
rasteriser launch sequence per iteration) for ``label_iters`` iterations,
from the generating parameters, against the scenes' own silhouettes and
median depth from 8 views, and the labels are the fitted blocks -- the
optimum the block stage settles at for that scene, which the silhouettes
and depths leave free to differ from the generating parameters.  Training
runs the network's tensor-core forward and backward and the one-launch Adam
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


def label_chunk(b: D.SQBatch, seeds, iters: int, res: int = 96, views: int = 8):
    """Replaces the chunk's labels by the block-level fit of each scene (in
    place), clamped into the ranges the network's outputs can take; returns
    the mean absolute change of (semi, eps, trans) and the mean final loss."""
    from .block_fit import BatchFit
    counts = b.counts.tolist()
    targets = [(b.semi[s, :k], b.eps[s, :k], b.quat[s, :k], b.trans[s, :k]) for s, k in enumerate(counts)]
    fit = BatchFit(targets, seeds, views=views, res=res)
    fitted, last = fit.fit(targets, iters)
    moved = []
    for s, (k, (semi, eps, quat, trans)) in enumerate(zip(counts, fitted)):
        semi, eps = semi.cpu().clamp(0.1001, 0.4999), eps.cpu().clamp(0.2001, 1.7999)
        quat, trans = quat.cpu(), trans.cpu()
        moved.append(torch.cat([(semi - b.semi[s, :k]).abs().reshape(-1), (eps - b.eps[s, :k]).abs().reshape(-1),
                                (trans - b.trans[s, :k]).abs().reshape(-1)]).mean())
        b.semi[s, :k], b.eps[s, :k], b.quat[s, :k], b.trans[s, :k] = semi, eps, quat, trans
    return float(torch.stack(moved).mean()), float(last.mean())


def make_dataset(num_scenes: int, seed: int = 0, res: int = 96, chunk: int = 256, label_iters: int = 0, log=None):
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
            moved, loss = label_chunk(b, seeds, label_iters, res=res)
            if log and (i % 64 == 0):
                log(f"labelled {i * chunk + b.exist.shape[0]} scenes: labels moved {moved:.4f} from the "
                    f"generating parameters, fit loss {loss:.4f}, {time.time() - t0:.0f}s")
        pts.append(p)
        labels.append(b)
    lab = D.SQBatch(*(torch.cat([getattr(x, f) for x in labels]) for f in ("semi", "eps", "quat", "trans", "exist")))
    return torch.cat(pts), lab


def train(num_scenes: int = 16384, steps: int = 8000, batch: int = 64, lr: float = 1e-3, seed: int = 0,
          log_every: int = 500, log=print, label_iters: int = 0):
    pts, lab = make_dataset(num_scenes, seed, label_iters=label_iters, log=log)
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
    ap.add_argument("--label-iters", type=int, default=50,
                    help="block-level fit iterations per label (0: the generating parameters)")
    ap.add_argument("--out", default=WEIGHTS)
    a = ap.parse_args()
    t0 = time.time()
    net, _ = train(a.scenes, a.steps, a.batch, a.lr, a.seed, label_iters=a.label_iters)
    print(f"trained in {time.time() - t0:.0f}s")
    save_npz(net, a.out)
    print("wrote", a.out)


if __name__ == "__main__":
    main()
