"""CPU baseline: the oracle's restatement of the rasteriser timed on the host.

TEST / MEASUREMENT INFRASTRUCTURE ONLY (used by ``bench.py``'s
``cpu_baseline`` field and its ``--impl reference`` arm; never by the
product path).

The reference rasteriser itself cannot run on a CPU (it is CUDA code), so
the baseline is the oracle port
(``kind: "port"``): numpy FP32, the reference's per-pixel algorithm.  A full
step of the 500k-surfel / 16-view / 800x600 workload would take hours on the
host, so one bounded sample is timed and scaled:

* per view, the per-surfel phases (preprocess, key binning, preprocess
  backward) are timed in full on one view;
* the per-pixel phases (blend forward + backward) are estimated for every
  tile of that view from a seeded sample of tiles drawn with probability
  proportional to their list length, each timed alone in a ``spawn``
  process pool (Horvitz-Thompson), and divided over the host cores;
* the step time is that per-view estimate times the number of views.
"""
from __future__ import annotations

import multiprocessing as mp
import os
import time

import numpy as np

_W = {}


def _setup(workload_name, seed, view, dtype_name):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    if root not in sys.path:
        sys.path.insert(0, root)
    from oracle import surfel_oracle as O
    from partgs_gb300.scenes import workload
    scene, cams = workload(workload_name, seed)
    cam = cams[view]
    ocam = O.Camera(cam.world_view_transform.reshape(-1), cam.full_proj_transform.reshape(-1), cam.camera_center,
                    cam.tanfovx, cam.tanfovy, cam.height, cam.width)
    osf = O.Surfels(scene.means3D.numpy(), scene.opacities.numpy(), scene.scales.numpy(), scene.rotations.numpy(),
                    shs=scene.shs.numpy(), sh_degree=scene.sh_degree)
    dt = np.dtype(dtype_name).type
    pre = O.preprocess(osf, ocam, O.PLAIN, dt)
    pl, ranges, keys = O.bin_tiles(pre)
    _W.update(O=O, ocam=ocam, osf=osf, pre=pre, pl=pl, ranges=ranges, dt=dt)


def _render_tiles(tiles):
    """Blend forward + backward of a tile subset; returns its compute seconds."""
    O = _W["O"]
    ocam, osf, pre, dt = _W["ocam"], _W["osf"], _W["pre"], _W["dt"]
    t0 = time.perf_counter()
    rf = O.render_forward(pre, _W["pl"], _W["ranges"], ocam, osf, np.zeros(3), O.PLAIN, dt, tiles=tiles)
    st = O.ViewState(radii=pre["radii"], tiles_touched=pre["tiles_touched"], means2D=pre["means2D"],
                     depths=pre["depths"], transmat=pre["transmat"], normal_opacity=pre["normal_opacity"],
                     rgb=pre["rgb"], clamped=pre["clamped"], point_list=_W["pl"], ranges=_W["ranges"],
                     keys=np.zeros(0), final_T=rf["final_T"], n_contrib=rf["n_contrib"], color=rf["color"],
                     others=rf["others"], semantic=None, amb_surfel=pre["amb"], amb_pixel=rf["amb_pixel"])
    st.extra["pre"] = pre
    dcol = np.full(rf["color"].shape, 1e-3, dt)
    doth = np.full(rf["others"].shape, 1e-4, dt)
    O.render_backward(st, ocam, osf, np.zeros(3), dcol, doth, None, O.PLAIN, dt, tiles=tiles)
    return time.perf_counter() - t0, int(rf["fragments"])


def sample_tiles(ranges, k, rng):
    """k tiles drawn with replacement, with probability proportional to their
    list length (the blend's work grows with it), and those probabilities."""
    lens = (ranges[:, 1] - ranges[:, 0]).astype(np.float64)
    p = lens / lens.sum()
    tiles = rng.choice(len(lens), size=k, replace=True, p=p)
    return tiles, p[tiles]


def blend_estimate(pool, ranges, k, rng):
    """Single-core seconds of the blend forward + backward of every tile of
    the view, estimated from k length-weighted tiles timed one per job
    (Horvitz-Thompson: the mean of cost / probability), and the sampled
    fragments."""
    tiles, p = sample_tiles(ranges, k, rng)
    res = pool.map(_render_tiles, [np.array([t]) for t in tiles], chunksize=1)
    cost = np.array([r[0] for r in res])
    return float(np.mean(cost / p)), int(sum(r[1] for r in res))


def time_step(workload_name="sq500k_16x800x600", seed=0, sample_tiles=None, procs=None, dtype_name="float32"):
    """Estimated seconds per step of the oracle on ``procs`` host processes,
    with the sample description.

    Per view: the per-surfel phases (preprocess, binning, preprocess
    backward) timed in full on one core; the blend forward + backward of
    every tile estimated from a length-weighted sample of tiles (each timed
    alone) and divided over the processes, as a tile-parallel host
    implementation would run it; times the number of views."""
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    if root not in sys.path:
        sys.path.insert(0, root)
    from oracle import surfel_oracle as O
    from partgs_gb300.scenes import workload
    procs = procs or os.cpu_count() or 1
    scene, cams = workload(workload_name, seed)
    V = len(cams)
    t0 = time.perf_counter()
    _setup(workload_name, seed, 0, dtype_name)
    t_setup = time.perf_counter() - t0          # preprocess + binning of one view (plus scene build)
    pre, ranges = _W["pre"], _W["ranges"]
    ocam, osf, dt = _W["ocam"], _W["osf"], _W["dt"]
    t0 = time.perf_counter()
    rb = dict(dL_dtransmat=np.zeros((osf.P, 9), dt), dL_dmean2D=np.zeros((osf.P, 2), dt),
              dL_dnormal=np.zeros((osf.P, 3), dt), dL_dopacity=np.zeros(osf.P, dt),
              dL_dcolor=np.zeros((osf.P, 3), dt), dL_dsemantics=np.zeros((osf.P, 0), dt))
    st = O.ViewState(radii=pre["radii"], tiles_touched=pre["tiles_touched"], means2D=pre["means2D"],
                     depths=pre["depths"], transmat=pre["transmat"], normal_opacity=pre["normal_opacity"],
                     rgb=pre["rgb"], clamped=pre["clamped"], point_list=_W["pl"], ranges=ranges, keys=np.zeros(0),
                     final_T=None, n_contrib=None, color=None, others=None, semantic=None, amb_surfel=pre["amb"],
                     amb_pixel=None)
    O.preprocess_backward(st, rb, ocam, osf, O.PLAIN, dt)
    t_prebwd = time.perf_counter() - t0
    ntiles = ranges.shape[0]
    k = sample_tiles or max(2 * procs, int(round(0.1 * ntiles)))   # default: a tenth of the tiles
    rng = np.random.default_rng(seed)
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs, initializer=_setup, initargs=(workload_name, seed, 0, dtype_name)) as pool:
        nonempty = np.nonzero(ranges[:, 1] > ranges[:, 0])[0]
        pool.map(_render_tiles, [nonempty[i:i + 1] for i in range(procs)], chunksize=1)   # warm-up
        blend_core_s, frags = blend_estimate(pool, ranges, k, rng)
    per_view = t_setup + t_prebwd + blend_core_s / procs
    step = per_view * V
    sample = (f"view 0 of {V}: preprocess, binning and preprocess backward in full (1 core); blend forward + "
              f"backward of all {ntiles} tiles estimated from {k} tiles drawn by list length (each timed alone, "
              f"{frags} fragments; Horvitz-Thompson), divided over {procs} processes; times {V} views")
    return step, sample, procs, dict(t_setup=t_setup, t_prebwd=t_prebwd, blend_core_s=blend_core_s,
                                     tiles_sampled=k, tiles=ntiles)


if __name__ == "__main__":
    s, desc, cores, d = time_step(sample_tiles=16)
    print(s, desc, cores, d)
