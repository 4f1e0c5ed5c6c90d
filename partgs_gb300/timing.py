"""Per-phase timing of the rasteriser alone (forward + backward through
autograd, no loss kernels or optimiser) for either variant:

  python -m partgs_gb300.timing [--workload sq500k_16x800x600] [--semantics 8] [--steps 5]

Prints one JSON line per variant with the library's CUDA-event phase times
(ms per call).  The part variant gets ``--semantics`` channels of seeded
softmax weights; the loss is the sum of every output, so every pixel
carries a gradient.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json

import torch

from . import _lib as L
from .batched import MultiViewRasterizer
from .scenes import workload


def time_variant(scene, cams, variant, semantics=None, steps=5, warmup=3, cell_tiles=0):
    dev = torch.device("cuda")
    lib = L.load()
    P = scene.P
    means, op = scene.means3D.to(dev), scene.opacities.to(dev)
    shs, sc, rot = scene.shs.to(dev), scene.scales.to(dev), scene.rotations.to(dev)
    r = MultiViewRasterizer(cams, [0, 0, 0], scene.sh_degree, variant=variant, num_surfels=P, device=dev,
                            cell_tiles=cell_tiles)

    def step():
        m = means.clone().requires_grad_(True)
        s_ = semantics.clone().requires_grad_(True) if semantics is not None else None
        col, oth, se, _ = r(m, op, shs, sc, rot, semantics=s_)
        loss = col.sum() + oth.sum() + (se.sum() if se is not None else 0)
        loss.backward()

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    lib.sgr_profile_enable(1)
    for _ in range(steps):
        step()
    torch.cuda.synchronize()
    ms, cnt = (C.c_float * len(L.PHASES))(), (C.c_int32 * len(L.PHASES))()
    lib.sgr_profile_read(ms, cnt)
    lib.sgr_profile_enable(0)
    return {L.PHASES[i]: round(ms[i] / max(1, cnt[i]), 3) for i in range(len(L.PHASES))}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="sq500k_16x800x600")
    ap.add_argument("--semantics", type=int, default=8)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--cell-tiles", type=int, default=0)
    a = ap.parse_args(argv)
    scene, cams = workload(a.workload, 0)
    g = torch.Generator().manual_seed(1)
    sem = torch.softmax(torch.randn(scene.P, a.semantics, generator=g) * 3, -1).cuda()
    for variant, name, s in ((L.SGR_VARIANT_PLAIN, "plain", None), (L.SGR_VARIANT_PART, "part", sem)):
        ph = time_variant(scene, cams, variant, s, a.steps, cell_tiles=a.cell_tiles)
        print(json.dumps({"variant": name, "workload": a.workload, "semantics": a.semantics if s is not None else 0,
                          "phase_ms": ph}), flush=True)


if __name__ == "__main__":
    main()
