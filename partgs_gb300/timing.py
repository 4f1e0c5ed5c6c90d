"""Per-phase timing of the rasteriser alone (forward + backward through
autograd, no loss kernels or optimiser) for either variant:

  python -m partgs_gb300.timing [--workload sq500k_16x800x600] [--semantics 8] [--steps 5]
                                [--cell-tiles 2] [--blend-shape 0] [--tile-schedule 1] [--stage-entries 128]

Prints one JSON line per variant with the library's CUDA-event phase times
(ms per call).  The part variant gets ``--semantics`` channels of seeded
softmax weights; the loss is the sum of every output, so every pixel
carries a gradient.

  python -m partgs_gb300.timing --multi-scene [--scenes 32] [--steps 5]

times an uneven multi-scene batch: 32 scenes of log-uniform surfel counts in
[20k, 400k] (superquadric surfaces as in the 500k workload), 8 views each at
400x300, forward + backward of all of them in one batched call against one
call per scene, each at its best cell size.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import time

import torch

from . import _lib as L
from .batched import MultiViewRasterizer
from .scenes import workload


def time_variant(scene, cams, variant, semantics=None, steps=5, warmup=3, cell_tiles=0, blend_shape=0,
                 tile_schedule=0, stage_entries=0):
    dev = torch.device("cuda")
    lib = L.load()
    P = scene.P
    means, op = scene.means3D.to(dev), scene.opacities.to(dev)
    shs, sc, rot = scene.shs.to(dev), scene.scales.to(dev), scene.rotations.to(dev)
    r = MultiViewRasterizer(cams, [0, 0, 0], scene.sh_degree, variant=variant, num_surfels=P, device=dev,
                            cell_tiles=cell_tiles, blend_shape=blend_shape, tile_schedule=tile_schedule,
                            stage_entries=stage_entries)

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


def multi_scene(n_scenes=32, steps=5, seed=0, lo=20_000, hi=400_000, views=8, height=300, width=400):
    """Wall time per fwd+bwd (CUDA-synchronised) of the batched call and of
    the per-scene calls, each at the best of the cell sizes 2, 4, 8."""
    from .scenes import scene_cameras, superquadric_surfels
    dev = torch.device("cuda")
    g = torch.Generator().manual_seed(seed)
    sizes = [int(math.exp(math.log(lo) + (math.log(hi) - math.log(lo)) * float(torch.rand(1, generator=g))))
             for _ in range(n_scenes)]
    scenes = [superquadric_surfels(n, 16, seed + s) for s, n in enumerate(sizes)]
    cams = [scene_cameras(views, height, width, 50.0, seed=seed + s) for s in range(n_scenes)]
    cat = lambda name: torch.cat([getattr(sc, name) for sc in scenes]).to(dev)  # noqa: E731
    means, op, shs, sc, rot = cat("means3D"), cat("opacities"), cat("shs"), cat("scales"), cat("rotations")
    offs = [0]
    for n in sizes:
        offs.append(offs[-1] + n)

    def run(rasters, parts):
        for r, (a, b) in zip(rasters, parts):
            m = means[a:b].clone().requires_grad_(True)
            col, oth, _, _ = r(m, op[a:b], shs[a:b], sc[a:b], rot[a:b])
            (col.sum() + oth.sum()).backward()

    def timed(make, parts):
        best = None
        for cell in (2, 4, 8):
            rasters = make(cell)
            for _ in range(2):
                run(rasters, parts)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(steps):
                run(rasters, parts)
            torch.cuda.synchronize()
            dt = (time.perf_counter() - t0) / steps
            best = (dt, cell) if best is None or dt < best[0] else best
            del rasters
            torch.cuda.empty_cache()
        return best

    all_cams = [c for cs in cams for c in cs]
    batched = timed(lambda cell: [MultiViewRasterizer(all_cams, [0, 0, 0], 3, scene_sizes=sizes,
                                                      scene_views=[views] * n_scenes, device=dev,
                                                      cell_tiles=cell)], [(0, offs[-1])])
    per_scene = timed(lambda cell: [MultiViewRasterizer(cams[s], [0, 0, 0], 3, num_surfels=sizes[s], device=dev,
                                                        cell_tiles=cell) for s in range(n_scenes)],
                      [(offs[s], offs[s + 1]) for s in range(n_scenes)])
    return {"scenes": n_scenes, "surfels": offs[-1], "views_per_scene": views, "image": [height, width],
            "batched_ms": round(batched[0] * 1e3, 2), "batched_cell_tiles": batched[1],
            "per_scene_ms": round(per_scene[0] * 1e3, 2), "per_scene_cell_tiles": per_scene[1],
            "speedup": round(per_scene[0] / batched[0], 2)}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="sq500k_16x800x600")
    ap.add_argument("--semantics", type=int, default=8)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--cell-tiles", type=int, default=0)
    ap.add_argument("--blend-shape", type=int, default=0, help="0: 16-wide warp strips, 1: 8-wide patches")
    ap.add_argument("--tile-schedule", type=int, default=0, help="0: a CTA per tile, 1: persistent tile queue")
    ap.add_argument("--stage-entries", type=int, default=0,
                    help="list entries per staged batch: 0 (the library's choice), 256, 128 or 64")
    ap.add_argument("--multi-scene", action="store_true")
    ap.add_argument("--scenes", type=int, default=32)
    a = ap.parse_args(argv)
    if a.multi_scene:
        print(json.dumps(multi_scene(a.scenes, a.steps)), flush=True)
        return
    scene, cams = workload(a.workload, 0)
    g = torch.Generator().manual_seed(1)
    sem = torch.softmax(torch.randn(scene.P, a.semantics, generator=g) * 3, -1).cuda()
    for variant, name, s in ((L.SGR_VARIANT_PLAIN, "plain", None), (L.SGR_VARIANT_PART, "part", sem)):
        ph = time_variant(scene, cams, variant, s, a.steps, cell_tiles=a.cell_tiles, blend_shape=a.blend_shape,
                          tile_schedule=a.tile_schedule, stage_entries=a.stage_entries)
        print(json.dumps({"variant": name, "workload": a.workload, "semantics": a.semantics if s is not None else 0,
                          "phase_ms": ph}), flush=True)


if __name__ == "__main__":
    main()
