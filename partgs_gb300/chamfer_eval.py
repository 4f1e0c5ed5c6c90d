"""Chamfer evaluation of a mesh against a ground-truth point set on the GPU,
the reference's evaluate_mesh (utils/blender_eval.py:25-111):

1. the mesh is sampled: its vertices plus, per triangle of non-zero area, a
   grid of (i + 0.5) / n1, (j + 0.5) / n2 barycentric steps inside it, with
   n1, n2 = floor(edge / (density * sqrt(l1 l2 / |v1 x v2|))) (float64, as
   numpy computes them);
2. the samples are shuffled (here with a seeded permutation; the reference
   draws an unseeded one);
3. they are thinned by the radius-`density` greedy suppression in that order
   (``sgr_radius_downsample``);
4. accuracy = mean of the nearest-GT distances of all samples below
   MAX_DIST, completeness = mean of the GT points' nearest-sample distances
   (to the thinned set) below MAX_DIST (exact nearest neighbours:
   ``sgr_nn_search_grid`` for large sets, ``sgr_nn_search`` for small);
5. the score is their average.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib as L

MAX_DIST = 1.0
DOWNSAMPLE_DENSITY = 0.005
_p = C.c_void_p


def _lib():
    lib = L.load()
    lib.sgr_nn_search.restype = C.c_int
    lib.sgr_nn_search.argtypes = [_p, C.c_int64, _p, C.c_int64, _p, _p, _p]
    f3 = C.POINTER(C.c_float)
    lib.sgr_nn_grid_scratch_bytes.restype = C.c_size_t
    lib.sgr_nn_grid_scratch_bytes.argtypes = [C.c_int64, C.c_int64, f3, f3]
    lib.sgr_nn_search_grid.restype = C.c_int
    lib.sgr_nn_search_grid.argtypes = [_p, C.c_int64, _p, C.c_int64, f3, f3, _p, _p, _p, C.c_size_t, _p]
    lib.sgr_downsample_scratch_bytes.restype = C.c_size_t
    lib.sgr_downsample_scratch_bytes.argtypes = [C.c_int64]
    lib.sgr_radius_downsample.restype = C.c_int
    lib.sgr_radius_downsample.argtypes = [_p, C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_double,
                                          _p, _p, C.c_size_t, C.POINTER(C.c_int32), _p]
    return lib


GRID_MIN_PAIRS = 1 << 24     # below this many (query, point) pairs the brute-force scan is as fast


def nn_distance(q: torch.Tensor, r: torch.Tensor, with_index: bool = False, method: str = "auto"):
    """Nearest-neighbour distances (and indices) in r of every point of q.

    method: "brute" (sgr_nn_search), "grid" (sgr_nn_search_grid, which
    gives the same results bit for bit) or "auto" (the grid for large sets;
    it reads r's bounding box on the host)."""
    if method not in ("auto", "brute", "grid"):
        raise ValueError(f"unknown method {method!r}")
    lib = _lib()
    q = q.float().contiguous()
    r = r.float().contiguous()
    n, m = q.shape[0], r.shape[0]
    dist = torch.empty(n, device=q.device)
    idx = torch.empty(n, dtype=torch.int32, device=q.device) if with_index else None
    ip = idx.data_ptr() if idx is not None else None
    stream = torch.cuda.current_stream().cuda_stream
    grid = method == "grid" or (method == "auto" and n * m >= GRID_MIN_PAIRS)
    if grid and n > 0 and m > 0:
        lo_t, hi_t = torch.aminmax(r, dim=0)
        lo = (C.c_float * 3)(*lo_t.tolist())
        hi = (C.c_float * 3)(*hi_t.tolist())
        scratch = torch.empty(lib.sgr_nn_grid_scratch_bytes(n, m, lo, hi), dtype=torch.uint8, device=q.device)
        L.check(lib.sgr_nn_search_grid(q.data_ptr(), n, r.data_ptr(), m, lo, hi, dist.data_ptr(), ip,
                                       scratch.data_ptr(), scratch.numel(), stream), "sgr_nn_search_grid")
    else:
        L.check(lib.sgr_nn_search(q.data_ptr(), n, r.data_ptr(), m, dist.data_ptr(), ip, stream), "sgr_nn_search")
    return (dist, idx) if with_index else dist


def radius_downsample(pts: torch.Tensor, radius: float = DOWNSAMPLE_DENSITY):
    """Keep mask of the in-order greedy radius suppression (fp64), and the
    number of parallel rounds it took."""
    lib = _lib()
    pts = pts.double().contiguous()
    n = pts.shape[0]
    if n == 0:
        return torch.zeros(0, dtype=torch.bool, device=pts.device), 0
    lo = (C.c_double * 3)(*pts.min(dim=0).values.tolist())
    hi = (C.c_double * 3)(*pts.max(dim=0).values.tolist())
    state = torch.empty(n, dtype=torch.uint8, device=pts.device)
    scratch = torch.empty(lib.sgr_downsample_scratch_bytes(n), dtype=torch.uint8, device=pts.device)
    rounds = C.c_int32(0)
    L.check(lib.sgr_radius_downsample(pts.data_ptr(), n, lo, hi, radius, state.data_ptr(), scratch.data_ptr(),
                                      scratch.numel(), C.byref(rounds), torch.cuda.current_stream().cuda_stream),
            "sgr_radius_downsample")
    return state == 1, int(rounds.value)


def _norm(x):
    # numpy's order: ((x0^2 + x1^2) + x2^2), each step rounded
    return torch.sqrt((x[:, 0] * x[:, 0] + x[:, 1] * x[:, 1]) + x[:, 2] * x[:, 2])


def _cross(a, b):
    return torch.stack([a[:, 1] * b[:, 2] - a[:, 2] * b[:, 1], a[:, 2] * b[:, 0] - a[:, 0] * b[:, 2],
                        a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]], -1)


def drop_unreferenced(vertices, triangles):
    """Open3D's remove_unreferenced_vertices: referenced vertices in their order, triangles re-indexed."""
    v = np.asarray(vertices)
    f = np.asarray(triangles)
    used = np.zeros(v.shape[0], dtype=bool)
    used[f.reshape(-1)] = True
    remap = np.cumsum(used) - 1
    return v[used], remap[f]


def sample_mesh(vertices, triangles, density: float = DOWNSAMPLE_DENSITY, device="cuda") -> torch.Tensor:
    """The reference's mesh samples (vertices first, then each triangle's grid
    points in its row-major (i, j) order), float64, with every arithmetic
    step in numpy's order so the samples are the reference's bit for bit."""
    v = torch.as_tensor(np.asarray(vertices), dtype=torch.float64, device=device)
    f = torch.as_tensor(np.asarray(triangles), dtype=torch.long, device=device)
    tv = v[f]
    v1, v2 = tv[:, 1] - tv[:, 0], tv[:, 2] - tv[:, 0]
    l1, l2 = _norm(v1), _norm(v2)
    area2 = _norm(_cross(v1, v2))
    nz = area2 > 0
    v1, v2, l1, l2, area2, t0 = v1[nz], v2[nz], l1[nz], l2[nz], area2[nz], tv[nz, 0]
    thr = density * torch.sqrt(l1 * l2 / area2)
    n1, n2 = torch.floor(l1 / thr), torch.floor(l2 / thr)
    g1, g2 = (n1 + 1).long(), (n2 + 1).long()
    count = g1 * g2
    tri = torch.repeat_interleave(torch.arange(count.shape[0], device=device), count)
    start = torch.cumsum(count, 0) - count
    local = torch.arange(int(count.sum()), device=device) - start[tri]
    i = torch.div(local, g2[tri], rounding_mode="floor")
    j = local - i * g2[tri]
    c0 = (i.double() + 0.5) / torch.clamp(n1[tri], min=1e-7)
    c1 = (j.double() + 0.5) / torch.clamp(n2[tri], min=1e-7)
    inside = (c0 + c1) < 1
    tri, c0, c1 = tri[inside], c0[inside], c1[inside]
    q = v1[tri] * c0[:, None] + v2[tri] * c1[:, None] + t0[tri]
    return torch.cat([v, q], 0)


def evaluate(vertices, triangles, gt_points, max_dist: float = MAX_DIST, density: float = DOWNSAMPLE_DENSITY,
             seed: int = 0, device="cuda"):
    """(accuracy, completeness, average) of a mesh against GT points.  The
    mesh's unreferenced vertices are dropped first, as the reference does."""
    vertices, triangles = drop_unreferenced(vertices, triangles)
    pcd = sample_mesh(vertices, triangles, density, device)
    perm = torch.randperm(pcd.shape[0], generator=torch.Generator().manual_seed(seed)).to(device)
    pcd = pcd[perm]
    keep, _ = radius_downsample(pcd, density)
    down = pcd[keep]
    stl = torch.as_tensor(np.asarray(gt_points), dtype=torch.float32, device=device)
    d2s = nn_distance(pcd, stl)
    s2d = nn_distance(stl, down)
    acc = float(d2s[d2s < max_dist].double().mean())
    comp = float(s2d[s2d < max_dist].double().mean())
    return acc, comp, (acc + comp) / 2


def write_scores(eval_dir, acc: float, comp: float, avg: float, suffix: str = "", step="-1", num_mesh: int = 1):
    """The reference's score file, blender_scores{suffix}_{step}.tsv."""
    import os
    os.makedirs(eval_dir, exist_ok=True)
    path = os.path.join(eval_dir, f"blender_scores{suffix}_{step}.tsv")
    with open(path, "w") as fh:
        fh.write("acc\tcomp\tavg\n")
        fh.write(f"{acc}\t{comp}\t{avg}\n")
        fh.write("num_mesh\n")
        fh.write(f"{num_mesh}")
    return path


def main(argv=None):
    """Times the evaluation of a dense superquadric mesh against a jittered
    sample of it: python -m partgs_gb300.chamfer_eval [--grid 400] [--gt 1000000]"""
    import argparse
    import time

    from . import sq_data as D
    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", type=int, default=400)
    ap.add_argument("--gt", type=int, default=1_000_000)
    a = ap.parse_args(argv)
    g = torch.Generator().manual_seed(0)
    eta, omega, faces = D.grid_topology(a.grid, a.grid)
    e, semi = (0.6, 1.3), np.array([0.6, 0.4, 0.5])
    sp = lambda t, x: np.sign(t) * np.abs(t) ** x  # noqa: E731
    verts = np.stack([sp(np.cos(eta), e[0]) * sp(np.sin(omega), e[1]), sp(np.sin(eta), e[0]),
                      sp(np.cos(eta), e[0]) * sp(np.cos(omega), e[1])], -1) * semi
    gt = D.surface_samples(torch.tensor(semi[None], dtype=torch.float32), torch.tensor([e]), torch.tensor([[1.0, 0, 0, 0]]),
                           torch.zeros(1, 3), a.gt, g).reshape(-1, 3)
    gt = (gt + 0.002 * torch.randn(gt.shape, generator=g)).numpy()
    evaluate(verts, faces, gt)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pcd = sample_mesh(*drop_unreferenced(verts, faces))
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    keep, rounds = radius_downsample(pcd[torch.randperm(pcd.shape[0], device=pcd.device)])
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    acc, comp, avg = evaluate(verts, faces, gt)
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    print(f"samples {pcd.shape[0]} kept {int(keep.sum())} gt {gt.shape[0]} rounds {rounds}")
    print(f"sample {1e3 * (t1 - t0):.1f} ms, downsample {1e3 * (t2 - t1):.1f} ms, whole evaluation "
          f"{1e3 * (t3 - t2):.1f} ms; acc {acc:.6f} comp {comp:.6f} avg {avg:.6f}")
    # the two searches of the evaluation, brute force against the grid
    stl = torch.as_tensor(gt, dtype=torch.float32, device=pcd.device)
    down = pcd[keep]
    for name, q, r in (("samples->gt", pcd, stl), ("gt->kept", stl, down)):
        res, ms = {}, {}
        for method in ("brute", "grid"):
            nn_distance(q, r, True, method)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            res[method] = nn_distance(q, r, True, method)
            torch.cuda.synchronize()
            ms[method] = 1e3 * (time.perf_counter() - t0)
        same = all(torch.equal(x, y) for x, y in zip(res["brute"], res["grid"]))
        print(f"nearest neighbours {name} ({q.shape[0]} x {r.shape[0]}): brute {ms['brute']:.2f} ms, "
              f"grid {ms['grid']:.2f} ms, identical {same}")


if __name__ == "__main__":
    main()
