"""Writes golden vectors of the reference's own CUDA rasterisers (plain and
part), compiled unmodified for sm_103a by ``oracle/ref_build.py``, for the
CPU tests that pin the oracle (``tests/test_ref_cuda_golden.py``).

Needs a GPU and the built reference extension; run from the repository root:

    python oracle/ref_build.py --ref <PartGS checkout>   # stage + build
    python tests/golden/make_ref_cuda_golden.py [out_dir]

Each case stores its inputs (surfels, camera, background), the upstream
gradients (seeded; zeroed where the FP64 oracle finds a decision within
FP32 rounding or the pixel ill-conditioned in FP32, the masks stored too),
and the reference's outputs: images,
radii, per-pixel final T and contributor counts, tile ranges and lists, and
the gradients of every input.
"""
from __future__ import annotations

import os
import sys

import numpy as np
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref_cuda  # noqa: E402
from oracle import surfel_oracle as O  # noqa: E402
from partgs_gb300.cameras import orbit_cameras  # noqa: E402
from partgs_gb300.scenes import random_surfels  # noqa: E402
from tests._util import oracle_camera, oracle_surfels  # noqa: E402

CASES = {
    # name: (variant, surfels, seed, height, width, fovx, cam seed, bg, semantic channels, colours precomputed)
    "plain_sh3_80x96": ("plain", 1536, 101, 80, 96, 60.0, 31, (0.1, 0.2, 0.3), 0, False),
    "part_sh3_S4_64x80": ("part", 1200, 102, 64, 80, 55.0, 32, (0.3, 0.1, 0.2), 4, False),
    "part_colors_S4_64x80": ("part", 1500, 51, 64, 80, 55.0, 23, (0.1, 0.5, 0.3), 4, True),
}


def make(name):
    variant, P, seed, H, W, fov, cseed, bg, S, precomp = CASES[name]
    scene = random_surfels(P, seed=seed)
    cam = orbit_cameras(1, 3.0, H, W, fov, seed=cseed)[0]
    g = torch.Generator()
    sem = torch.rand(P, S, generator=g.manual_seed(seed + 1)) if S else None
    cols = torch.rand(P, 3, generator=g.manual_seed(seed + 2)) if precomp else None
    osf = oracle_surfels(scene, colors_precomp=cols, semantics=sem)
    v = O.PART if variant == "part" else O.PLAIN
    st = O.forward_view(osf, oracle_camera(cam), np.array(bg), v, np.float64)
    sens = O.fp32_sensitivity(st, oracle_camera(cam), osf, np.array(bg), v)
    ill = (sens[:3].max(0) > 5e-6) | (sens[3:].max(0) > 1.5e-5)
    amb_pixel = st.amb_pixel | ill
    rng = np.random.default_rng(seed + 3)
    dcol = rng.standard_normal(st.color.shape).astype(np.float32)
    doth = (rng.standard_normal(st.others.shape) * 0.1).astype(np.float32)
    dsem = rng.standard_normal(st.semantic.shape).astype(np.float32) if S else None
    for a in (dcol, doth, dsem):
        if a is not None:
            a[:, amb_pixel] = 0
    kw = dict(means3D=scene.means3D, opacities=scene.opacities, scales=scene.scales, rotations=scene.rotations,
              semantics=sem)
    if precomp:
        kw["colors_precomp"] = cols
    else:
        kw["shs"] = scene.shs
    out = ref_cuda.render(variant, cam, list(bg), upstream=(dcol, doth, dsem), **kw)
    rec = dict(variant=np.array(variant), means3D=scene.means3D.numpy(), opacities=scene.opacities.numpy(),
               scales=scene.scales.numpy(), rotations=scene.rotations.numpy(), bg=np.array(bg, np.float32),
               viewmatrix=np.asarray(cam.world_view_transform, np.float32),
               projmatrix=np.asarray(cam.full_proj_transform, np.float32),
               campos=np.asarray(cam.camera_center, np.float32), tanfov=np.array([cam.tanfovx, cam.tanfovy]),
               hw=np.array([H, W]), amb_pixel=amb_pixel, amb_count_pixel=st.extra["amb_count_pixel"] | ill,
               amb_surfel=st.amb_surfel,
               amb_tiles=st.extra["amb_tiles"], dL_dcolor_in=dcol, dL_dothers_in=doth)
    if precomp:
        rec["colors_precomp"] = cols.numpy()
    else:
        rec["shs"] = scene.shs.numpy()
    if S:
        rec["semantics"] = sem.numpy()
        rec["dL_dsemantic_in"] = dsem
    for key, val in out.items():
        rec["ref_" + key] = np.asarray(val)
    return rec


def main(out_dir=None):
    out_dir = out_dir or os.path.join(ROOT, "tests", "golden")
    os.makedirs(out_dir, exist_ok=True)
    for name in CASES:
        rec = make(name)
        path = os.path.join(out_dir, f"ref_cuda_{name}.npz")
        np.savez_compressed(path, **rec)
        print(path, os.path.getsize(path))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
