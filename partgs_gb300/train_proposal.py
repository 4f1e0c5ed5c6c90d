"""Trains the superquadric proposal network on synthetic scenes and writes its
weights (``.npz``: W0..W4, b0..b4, float32).

    python -m partgs_gb300.train_proposal --scenes 65536 --steps 20000 --batch 128 \
        --out partgs_gb300/weights/proposal_sq8.npz

Scenes are drawn, rendered and back-projected on the GPU in batches of 256
(``sq_data``); training runs the network's tensor-core forward and backward
and the one-launch Adam (``proposal.Trainer``).
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


def make_dataset(num_scenes: int, seed: int = 0, res: int = 96, chunk: int = 256):
    """(points [N, 2048, 3] on the GPU, labels SQBatch on the host)."""
    g = torch.Generator().manual_seed(seed)
    ren = D.SceneRenderer(res=res)
    pts, labels = [], []
    for i in range((num_scenes + chunk - 1) // chunk):
        b = D.sample_sq_batch(min(chunk, num_scenes - i * chunk), g)
        p, _ = ren.points(b, seed=seed * 100003 + i)
        pts.append(p)
        labels.append(b)
    lab = D.SQBatch(*(torch.cat([getattr(x, f) for x in labels]) for f in ("semi", "eps", "quat", "trans", "exist")))
    return torch.cat(pts), lab


def train(num_scenes: int = 16384, steps: int = 8000, batch: int = 64, lr: float = 1e-3, seed: int = 0,
          log_every: int = 500, log=print):
    pts, lab = make_dataset(num_scenes, seed)
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
    ap.add_argument("--scenes", type=int, default=16384)
    ap.add_argument("--steps", type=int, default=8000)
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=WEIGHTS)
    a = ap.parse_args()
    net, _ = train(a.scenes, a.steps, a.batch, a.lr, a.seed)
    save_npz(net, a.out)
    print("wrote", a.out)


if __name__ == "__main__":
    main()
