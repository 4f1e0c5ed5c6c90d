"""Benchmark: point-level surfel training steps per second.

Workload (default ``sq500k_16x800x600``): 500,000 surfels on a seeded union
of 16 superquadric surfaces, 16 cameras at 800x600 (fovx 50 deg), one step =
rasterise all 16 views, photometric (L1 + D-SSIM) + distortion (weight 1000)
+ normal-consistency loss, backward, Adam; the whole step is captured in one
CUDA graph.  Targets are seeded uniform images (no dataset is available).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line.  ``--impl reference`` times the CPU restatement of the
reference rasteriser (the oracle) on a bounded sample of the same workload.
Under torchrun each rank runs an independent replica (the step needs no
exchange between GPUs); the reported value is the whole-job rate.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "fwd+bwd train steps/s (500k surfels, 16x800x600)"
UNIT = "steps/s"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float, device=None) -> float:
    """Largest value of ``x`` over the ranks of the default process group
    (``x`` itself without one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _workload_config(name):
    if name == "sq500k_16x800x600":
        return {"workload": name, "surfels": 500_000, "views": 16, "height": 600, "width": 800, "fovx_deg": 50,
                "sh_degree": 3, "loss": "0.8 L1 + 0.2 D-SSIM + 1000 distortion + 0.05 normal consistency",
                "optimizer": "Adam (fused, capturable)", "cuda_graph": True,
                "l2": "per-step working set (per-view records, cell lists, images, gradients) far larger than the 129 MB L2"}
    return {"workload": name}


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons (200 ms)."""

    def __init__(self, index=0):
        self.f = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.f.name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def run_reference(args):
    """CPU restatement timed on the host (rank 0 only): per step, the
    per-surfel phases of one view (timed once) plus the blend of every tile
    estimated from a fresh length-weighted sample of tiles, times the views."""
    ws, rank, _ = _dist()
    if rank != 0:
        return
    import numpy as np
    from oracle import cpu_baseline as CB
    procs = os.cpu_count() or 1
    t0 = time.perf_counter()
    est, desc, cores, d = CB.time_step(args.workload, 0, sample_tiles=procs, procs=procs)
    per_surfel = d["t_setup"] + d["t_prebwd"]
    ests = []
    import multiprocessing as mp
    CB._setup(args.workload, 0, 0, "float32")
    ranges = CB._W["ranges"]
    views = _workload_config(args.workload).get("views", 16)
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs, initializer=CB._setup, initargs=(args.workload, 0, 0, "float32")) as pool:
        nonempty = np.nonzero(ranges[:, 1] > ranges[:, 0])[0]
        pool.map(CB._render_tiles, [nonempty[i:i + 1] for i in range(procs)], chunksize=1)
        for step in range(args.warmup + args.steps):
            rng = np.random.default_rng(1000 + step)
            core_s, _ = CB.blend_estimate(pool, ranges, procs, rng)
            if step >= args.warmup:
                ests.append((per_surfel + core_s / procs) * views)
    step_s = statistics.mean(ests)
    value = 1.0 / step_s
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": _workload_config(args.workload),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": "port",
                             "sample": desc + f"; {args.steps} timed samples of {procs} tiles each"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": time.perf_counter() - t0}
    print(json.dumps(line), flush=True)


# FP32 operations per visited fragment of the reference's blend loops
# (P0/cr/forward.cu:349-412: 77; P0/cr/backward.cu:290-437: 195)
FLOPS_PER_FRAGMENT = {"blend_fwd": 77, "blend_bwd": 195}


def roofline_report(workload, phases, dom, tr, P, V, H, W, keys, nbins, dev):
    """Per-phase rooflines of the eager step whose CUDA-event phase times are
    ``phases`` (ms).  The blends are bound by instruction issue: warp
    instructions per launch (one ncu count of this workload, committed under
    profiles/) over the live launch time, against one warp instruction per
    scheduler per SM clock; beside that, the effective FP32 rate of the
    reference's algorithm (FLOPS_PER_FRAGMENT x the fragments counted on the
    device) against the FP32 peak.  The other phases are bound by HBM:
    algorithmic bytes per launch over the launch time, against the measured
    copy bandwidth."""
    import torch
    from partgs_gb300 import _lib as L
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    props = torch.cuda.get_device_properties(dev)
    sms = props.multi_processor_count
    clock_mhz = float(peaks.get("sm_max_mhz", 2070.0))
    issue_peak = sms * 4 * clock_mhz * 1e6                 # warp instructions / s
    fp32_peak = sms * 128 * 2 * clock_mhz * 1e6            # FMA = 2 operations, 128 lanes per SM
    frag_fwd = tr.raster.fragments()
    st = tr.raster.last_state
    s = st.sizes
    HW = H * W
    nc = st.geom[s.off_n_contrib:s.off_n_contrib + V * 2 * HW * 4].view(torch.int32).reshape(V, 2, HW)
    frag_bwd = int(nc[:, 0].sum().item())
    R = P * V
    tj = {}
    try:
        tj = json.load(open(os.path.join(ROOT, "profiles", "roofline_traffic.json"))).get(workload, {})
    except (OSError, ValueError):
        pass
    alg_bytes = {
        "preprocess": 232 * P + 87 * R + 96 * R,     # parameters once; per record: outputs + the 96-B record
        "depth_order": 24 * R + 20 * R,              # sort of 12-B (key, index) pairs; rectangle gather
        "binning": 3 * 8 * R + 4 * nbins,            # rectangles read by three passes; one 4-B id per entry
        "preprocess_bwd": 583 * R,
    }
    per = {}
    for name, ms in phases.items():
        t = ms * 1e-3
        e = {"ms": round(ms, 4)}
        if name in FLOPS_PER_FRAGMENT:
            frags = frag_fwd if name == "blend_fwd" else frag_bwd
            # warp instructions per launch: ncu's count per fragment on a smaller case of the same scene
            # distribution (profiles/roofline_traffic.json) times this run's device-counted fragments
            ipf = tj.get(name + "_warp_inst_per_fragment")
            inst = ipf * frags if ipf else tj.get(name + "_warp_inst")
            e.update(bound="issue", fragments=int(frags),
                     fp32_effective={"achieved": round(FLOPS_PER_FRAGMENT[name] * frags / t / 1e12, 3),
                                     "peak": round(fp32_peak / 1e12, 2), "unit": "TFLOP/s",
                                     "frac": round(FLOPS_PER_FRAGMENT[name] * frags / t / fp32_peak, 4)})
            if inst:
                e.update(achieved=round(inst / t / 1e12, 4), peak=round(issue_peak / 1e12, 4), unit="Twarp-inst/s",
                         frac=round(inst / t / issue_peak, 4), warp_inst_per_launch=int(inst))
        else:
            b = alg_bytes[name]
            e.update(bound="hbm", achieved=round(b / t / 1e9, 1), peak=hbm_peak, unit="GB/s",
                     frac=round(b / t / 1e9 / hbm_peak, 4), algorithmic_bytes=int(b))
        traffic = tj.get(name)
        if traffic:
            e["traffic"] = int(traffic)
            e["dram_gbs"] = round(traffic / t / 1e9, 1)
        per[name] = e
    top = dict(per[dom])
    out = {"kernel": dom, "bound": top.get("bound"), "achieved": top.get("achieved"), "peak": top.get("peak"),
           "unit": top.get("unit"), "frac": top.get("frac"), "traffic": top.get("traffic"),
           "launch_ms": top["ms"], "peak_source": "measured" if "hbm_gbs" in peaks else "fallback",
           "fragments_fwd": int(frag_fwd), "fragments_bwd": int(frag_bwd), "phases": per}
    if "fp32_effective" in top:
        out["fp32_effective"] = top["fp32_effective"]
    return out


def time_reference_cuda(workload_name, steps=3, warmup=1, device=None):
    """The reference's own CUDA rasteriser (compiled unmodified for sm_103a by
    ``oracle/ref_build.py``) on the same workload, the way the reference
    trains: per view, the activations (scene/gaussian_model.py:198-218), its
    ``GaussianRasterizer`` forward, the same loss in PyTorch operations
    (L1 + D-SSIM, distortion, normal consistency, as train.py:229-250 /
    ``SurfelTrainer.reference_loss``) divided by the view count, backward;
    after all views, ``torch.optim.Adam`` (eps 1e-15, fused) and zero_grad.
    Also times the rasteriser alone (forward + backward of every view
    against fixed upstream gradients).  Returns a dict of per-step ms, or
    None when the reference was not built."""
    import torch
    from oracle import ref_build, ref_cuda
    if not ref_cuda.available():
        try:
            ref_build.build()
        except Exception:
            return None
        if not ref_cuda.available():
            return None
    from partgs_gb300.scenes import workload
    from partgs_gb300.surfel_step import DepthNormals, _gaussian_window, ssim
    dev = device or torch.device("cuda")
    mod = ref_cuda.load("plain")
    scene, cams = workload(workload_name, 0)
    V = len(cams)
    g = torch.Generator().manual_seed(7)
    targets = torch.rand(V, 3, cams[0].height, cams[0].width, generator=g).to(dev)
    sets = [ref_cuda.settings(mod, c, [0.0, 0.0, 0.0], scene.sh_degree) for c in cams]
    normals = [DepthNormals([c], dev) for c in cams]
    window = _gaussian_window(device=dev)
    xyz = scene.means3D.to(dev).clone().requires_grad_(True)
    log_s = torch.log(scene.scales).to(dev).clone().requires_grad_(True)
    rot = scene.rotations.to(dev).clone().requires_grad_(True)
    op = scene.opacities.clamp(1e-4, 1 - 1e-4)
    op_l = torch.log(op / (1 - op)).to(dev).clone().requires_grad_(True)
    f_dc = scene.shs[:, :1].to(dev).clone().requires_grad_(True)
    f_rest = scene.shs[:, 1:].to(dev).clone().requires_grad_(True)
    opt = torch.optim.Adam([{"params": [xyz], "lr": 0.00048}, {"params": [f_dc], "lr": 0.0025},
                            {"params": [f_rest], "lr": 0.0025 / 20.0}, {"params": [op_l], "lr": 0.05},
                            {"params": [log_s], "lr": 0.005}, {"params": [rot], "lr": 0.001}], eps=1e-15,
                           fused=True)

    def view_loss(v):
        scales = torch.exp(log_s)
        rots = torch.nn.functional.normalize(rot)
        opac = torch.sigmoid(op_l)
        shs = torch.cat((f_dc, f_rest), dim=1)
        m2 = torch.zeros_like(xyz, requires_grad=True)
        color, radii, allmap = mod.GaussianRasterizer(sets[v])(means3D=xyz, means2D=m2, shs=shs,
                                                               colors_precomp=None, opacities=opac,
                                                               scales=scales, rotations=rots)
        color, allmap, tgt = color[None], allmap[None], targets[v:v + 1]
        l1 = torch.abs(color - tgt).mean()
        loss = 0.8 * l1 + 0.2 * (1.0 - ssim(color, tgt, window))
        alpha = allmap[:, 1:2]
        rend_normal = torch.einsum("vchw,vcd->vdhw", allmap[:, 2:5], normals[v].view_to_world)
        median = torch.nan_to_num(allmap[:, 5:6], 0, 0)
        surf_normal = normals[v].normals(median) * alpha.detach()
        normal_loss = 0.05 * (1 - (rend_normal * surf_normal).sum(dim=1)).mean()
        return (loss + 1000.0 * allmap[:, 6:7].mean() + normal_loss) / V

    def step():
        for v in range(V):
            view_loss(v).backward()
        opt.step()
        opt.zero_grad(set_to_none=False)

    def timed(fn, n):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(n):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n

    for _ in range(warmup):
        step()
    step_ms = timed(step, steps)

    # rasteriser alone: forward + backward of every view, fixed inputs
    with torch.no_grad():
        a = (torch.exp(log_s), torch.nn.functional.normalize(rot), torch.sigmoid(op_l),
             torch.cat((f_dc, f_rest), dim=1))
    gr = torch.Generator(device=dev).manual_seed(3)
    up_c = torch.randn(3, cams[0].height, cams[0].width, device=dev, generator=gr)
    up_o = torch.randn(7, cams[0].height, cams[0].width, device=dev, generator=gr) * 0.1
    leaves = [t.detach().clone().requires_grad_(True) for t in (xyz,) + a]

    def raster_only():
        for v in range(V):
            m2 = torch.zeros_like(leaves[0], requires_grad=True)
            color, radii, allmap = mod.GaussianRasterizer(sets[v])(
                means3D=leaves[0], means2D=m2, shs=leaves[4], colors_precomp=None, opacities=leaves[3],
                scales=leaves[1], rotations=leaves[2])
            ((color * up_c).sum() + (allmap * up_o).sum()).backward()

    raster_only()
    raster_ms = timed(raster_only, steps)
    return {"step_ms": step_ms, "raster_ms": raster_ms, "steps": steps, "warmup": warmup,
            "what": "reference diff_surfel_rasterization (unmodified, nvcc -O3 sm_103a) through its own "
                    "GaussianRasterizer, one view at a time; loss and Adam in PyTorch"}


def time_part_variant(workload_name, cell_tiles, blend_shape, tile_schedule, semantics=8, steps=3, warmup=1,
                      with_reference=True, device=None):
    """The part variant, the rasteriser behind PartGS's ``render_part``
    (renderer/gaussian_renderer_2d/__init__.py:11-149): this library's and
    the reference's own (``diff_surfel_rasterization_part``, compiled
    unmodified by ``oracle/ref_build.py``), forward + backward of every view
    of the workload against fixed upstream gradients on the colour,
    auxiliary and semantic maps, with ``semantics`` channels of seeded
    softmax weights.  This library renders all views in one batched call at
    the given launch shape; the reference one view at a time, as
    ``render_part`` calls it.  Returns ms per pass over all views."""
    import torch
    from partgs_gb300 import _lib as L
    from partgs_gb300.batched import MultiViewRasterizer
    from partgs_gb300.scenes import workload
    dev = device or torch.device("cuda")
    scene, cams = workload(workload_name, 0)
    V, H, W, S = len(cams), cams[0].height, cams[0].width, semantics
    g = torch.Generator().manual_seed(1)
    sem = torch.softmax(torch.randn(scene.P, S, generator=g) * 3, -1)
    inputs = [t.to(dev) for t in (scene.means3D, scene.opacities, scene.shs, scene.scales, scene.rotations, sem)]
    gr = torch.Generator(device=dev).manual_seed(3)
    up_c = torch.randn(V, 3, H, W, device=dev, generator=gr)
    up_o = torch.randn(V, 8, H, W, device=dev, generator=gr) * 0.1
    up_s = torch.randn(V, S, H, W, device=dev, generator=gr)

    def timed(fn, n):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(n):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n

    r = MultiViewRasterizer(cams, [0.0, 0.0, 0.0], scene.sh_degree, variant=L.SGR_VARIANT_PART, num_surfels=scene.P,
                            device=dev, cell_tiles=cell_tiles, blend_shape=blend_shape, tile_schedule=tile_schedule)
    leaves = [t.clone().requires_grad_(True) for t in inputs]

    def ours():
        col, oth, smap, _ = r(leaves[0], leaves[1], leaves[2], leaves[3], leaves[4], semantics=leaves[5])
        ((col * up_c).sum() + (oth * up_o).sum() + (smap * up_s).sum()).backward()

    for _ in range(warmup):
        ours()
    out = {"semantics": S, "views": V, "ours_ms": timed(ours, steps)}
    if not with_reference:
        return out
    from oracle import ref_build, ref_cuda
    try:
        if not ref_cuda.available():
            ref_build.build()
        mod = ref_cuda.load("part")
    except Exception as ex:   # sources not staged
        out["reference_unavailable"] = str(ex)[:200]
        return out
    sets = [ref_cuda.settings(mod, c, [0.0, 0.0, 0.0], scene.sh_degree) for c in cams]
    rl = [t.clone().requires_grad_(True) for t in inputs]

    def reference():
        for v in range(V):
            m2 = torch.zeros_like(rl[0], requires_grad=True)
            color, semantic, _, allmap = mod.GaussianRasterizer(sets[v])(
                means3D=rl[0], means2D=m2, opacities=rl[1], semantics=rl[5], shs=rl[2], colors_precomp=None,
                scales=rl[3], rotations=rl[4])
            ((color * up_c[v]).sum() + (allmap * up_o[v]).sum() + (semantic * up_s[v]).sum()).backward()

    for _ in range(warmup):
        reference()
    out["reference_ms"] = timed(reference, steps)
    out["speedup"] = out["reference_ms"] / out["ours_ms"]
    out["what"] = ("part rasteriser alone, forward + backward of all views; reference "
                   "diff_surfel_rasterization_part (unmodified, nvcc -O3 sm_103a), one view at a time")
    return out


def run_gpu(args):
    import torch
    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", torch.cuda.current_device())
    from partgs_gb300 import _lib as L
    from partgs_gb300.scenes import workload
    from partgs_gb300.surfel_step import SurfelTrainer
    lib = L.load()
    scene, cams = workload(args.workload, 0)
    V, H, W = len(cams), cams[0].height, cams[0].width
    g = torch.Generator().manual_seed(7)
    targets_host = torch.rand(V, 3, H, W, generator=g).pin_memory()
    targets = targets_host.to(dev)

    tr = SurfelTrainer(scene, cams, device=dev)
    fixed = bool(args.cell_tiles)
    if fixed:                                      # a fixed launch shape (profiling runs: no tuning launches)
        tr.raster.cell_tiles = args.cell_tiles
        tr.raster.blend_shape = args.blend_shape
        tr.raster.tile_schedule = args.tile_schedule
        tr.raster.stage_entries = args.stage_entries
    # cell size, warp footprint, tile schedule and staged batch timed per workload unless
    # given; the warm-up steps size the lists
    tr.capture(targets, warmup=3, autotune=not fixed)
    tuning = {}
    if not fixed:
        from partgs_gb300 import autotune as AT
        tuning = {"cells_ms": {str(k): round(v, 3) for k, v in AT.tune_cells.last_timings.items()},
                  "blend_ms": {f"shape{k[0]}_sched{k[1]}_stage{k[2]}": round(v, 3)
                               for k, v in AT.tune_blend.last_timings.items()}}
    launches_per_step = tr.launches_per_step
    for _ in range(args.warmup):
        tr.replay()
    torch.cuda.synchronize()
    # both timed regions start from this state, so they run the same steps
    start = tr.snapshot()

    # ---- timed region: graph replays, inputs resident ----
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(dev.index or 0) if rank == 0 else None
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        tr.replay()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop() if clocks else None
    if ws > 1:
        ms = max_over_ranks(ms, dev)
        torch.distributed.barrier()
    keys, flags, nbins = tr.raster.counts()
    if flags & L.SGR_FLAG_BIN_OVERFLOW:
        raise RuntimeError(f"cell-list capacity {tr.raster.bin_capacity} exceeded ({nbins} entries)")
    ms_per_step = ms / args.steps
    value = ws * 1000.0 / ms_per_step

    # ---- end to end: targets uploaded from pinned host memory, loss read back ----
    # Each step's targets are uploaded on a copy stream while the previous
    # step runs, then moved into the graph's input buffer on the device; the
    # first upload is inside the timed region too.
    tr.restore(start)
    staging = torch.empty_like(tr.targets)
    copy_stream = torch.cuda.Stream()
    main = torch.cuda.current_stream()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    with torch.cuda.stream(copy_stream):
        staging.copy_(targets_host, non_blocking=True)
    consumed = torch.cuda.Event()
    for k in range(args.steps):
        main.wait_stream(copy_stream)
        tr.targets.copy_(staging)
        consumed.record(main)                      # staging may be overwritten after this copy
        loss = tr.replay()
        if k + 1 < args.steps:
            copy_stream.wait_event(consumed)
            with torch.cuda.stream(copy_stream):
                staging.copy_(targets_host, non_blocking=True)
        float(loss.item())
    e2e_s = (time.perf_counter() - t0) / args.steps
    e2e_s = max_over_ranks(e2e_s, dev)

    # ---- dominant kernel: per-phase CUDA events over eager steps of the same work ----
    import ctypes as C
    lib.sgr_profile_enable(1)
    n_prof = 3
    for _ in range(n_prof):
        tr.step(tr.targets)
    torch.cuda.synchronize()
    msv = (C.c_float * 6)()
    cnt = (C.c_int32 * 6)()
    lib.sgr_profile_read(msv, cnt)
    lib.sgr_profile_enable(0)
    phases = {L.PHASES[i]: (msv[i] / max(1, cnt[i])) for i in range(6)}
    dom = max(phases, key=phases.get)
    roofline = roofline_report(args.workload, phases, dom, tr, scene.P, V, H, W, keys, nbins, dev)
    frag_fwd, frag_bwd = roofline["fragments_fwd"], roofline["fragments_bwd"]

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene and targets)",
            "config": dict(_workload_config(args.workload), keys=keys, cell_list_entries=nbins,
                           fragments_fwd=frag_fwd, fragments_bwd=frag_bwd,
                           cell_list_capacity=tr.raster.bin_capacity, cell_tiles=tr.raster.cell_tiles,
                           blend_shape=["strip16", "patch8"][tr.raster.blend_shape],
                           tile_schedule=["grid", "queue"][tr.raster.tile_schedule],
                           stage_entries=tr.raster.stage_entries or "library default (256 for plain)",
                           autotune_ms=tuning or None, parallelism=f"replicas x{ws}"),
            "e2e": {"value": ws / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(targets_host.numel() * 4),
                    "d2h_bytes_per_step": 4},
            "roofline": roofline, "gpu_launches": int(launches_per_step) * args.steps, "clocks": clk}
    if rank == 0 and ws == 1 and not args.no_reference_cuda:
        rc = time_reference_cuda(args.workload, device=dev)
        if rc is None:
            line["reference_cuda"] = {"unavailable": "reference extension not built (sources not staged)"}
        else:
            raster_ms = sum(phases.values())
            rc.update(ours_step_ms=ms_per_step, ours_raster_ms=raster_ms,
                      step_speedup=rc["step_ms"] / ms_per_step, raster_speedup=rc["raster_ms"] / raster_ms)
            line["reference_cuda"] = {k: (round(v, 4) if isinstance(v, float) else v) for k, v in rc.items()}
    if rank == 0 and ws == 1 and not args.no_part:
        pv = time_part_variant(args.workload, tr.raster.cell_tiles, tr.raster.blend_shape, tr.raster.tile_schedule,
                               with_reference=not args.no_reference_cuda, device=dev)
        line["part_variant"] = {k: (round(v, 4) if isinstance(v, float) else v) for k, v in pv.items()}
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        from oracle import cpu_baseline as CB
        procs = os.cpu_count() or 1
        est, desc, cores, _ = CB.time_step(args.workload, 0, procs=procs)      # a tenth of the tiles
        line["cpu_baseline"] = {"value": 1.0 / est, "unit": UNIT, "cores": cores, "kind": "port", "sample": desc}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


MULTISCENE = "multiscene_32x8x400x300"


def run_multiscene(args):
    """The uneven multi-scene workload: 32 scenes of log-uniform surfel
    counts in [20k, 400k] (each a union of 16 superquadric surfaces), 8 orbit
    views each at 400x300.  One step = rasteriser forward + backward of all
    256 views in one batched call (loss: fixed seeded weights on every output
    map), at the cell edge, warp footprint and tile schedule the autotuner
    picks; against the same work as 32 per-scene calls of this library and
    as 256 per-view calls of the reference's CUDA rasteriser.  e2e uploads
    the step's weights from pinned host memory and reads the loss back."""
    import math

    import torch
    from partgs_gb300 import _lib as L
    from partgs_gb300.batched import MultiViewRasterizer
    from partgs_gb300.scenes import scene_cameras, superquadric_surfels
    ws, rank, _ = _dist()
    dev = torch.device("cuda")
    L.load()
    n_scenes, views, H, W = 32, 8, 300, 400
    g = torch.Generator().manual_seed(0)
    sizes = [int(math.exp(math.log(20_000) + (math.log(400_000) - math.log(20_000)) * float(torch.rand(1, generator=g))))
             for _ in range(n_scenes)]
    scenes = [superquadric_surfels(n, 16, s) for s, n in enumerate(sizes)]
    cams = [scene_cameras(views, H, W, 50.0, seed=s) for s in range(n_scenes)]
    all_cams = [c for cs in cams for c in cs]
    cat = lambda name: torch.cat([getattr(sc, name) for sc in scenes]).to(dev)  # noqa: E731
    inputs = [cat(k) for k in ("means3D", "opacities", "shs", "scales", "rotations")]
    offs = [0]
    for n in sizes:
        offs.append(offs[-1] + n)
    V = n_scenes * views
    wg = torch.Generator().manual_seed(1)
    w_host = torch.randn(V, 10, H, W, generator=wg).pin_memory()
    w_dev = w_host.to(dev)

    def make(cell, shape, sched, stage=0):
        return MultiViewRasterizer(all_cams, [0, 0, 0], 3, scene_sizes=sizes, scene_views=[views] * n_scenes,
                                   device=dev, cell_tiles=cell, blend_shape=shape, tile_schedule=sched,
                                   stage_entries=stage)

    def step(r, w):
        leaves = [t.detach().requires_grad_(True) for t in inputs]
        col, oth, _, _ = r(*leaves)
        loss = (col * w[:, :3]).sum() + (oth * w[:, 3:]).sum()
        loss.backward()
        return loss

    def timed(fn, n):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(n):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n

    # autotune: cell edge (default footprint, schedule and staged batch),
    # then footprint x schedule x staged batch
    tune = {}
    for cell in (2, 4, 8):
        r = make(cell, 0, 0, L.SGR_STAGE_DEFAULT)
        step(r, w_dev)
        tune[(cell, 0, 0, L.SGR_STAGE_DEFAULT)] = timed(lambda: step(r, w_dev), 2)
    cell = min(tune, key=tune.get)[0]
    for shape in (0, 1):
        for sched in (0, 1):
            for stage in (L.SGR_STAGE_DEFAULT, L.SGR_STAGE_SMALL, L.SGR_STAGE_TINY):
                if (cell, shape, sched, stage) not in tune:
                    r = make(cell, shape, sched, stage)
                    step(r, w_dev)
                    tune[(cell, shape, sched, stage)] = timed(lambda: step(r, w_dev), 2)
    best = min(tune, key=tune.get)
    r = make(*best)
    for _ in range(args.warmup):
        step(r, w_dev)
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    ms = timed(lambda: step(r, w_dev), args.steps)
    clk = clocks.stop()

    # end to end: the weights uploaded from pinned memory, the loss read back
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        w = w_host.to(dev, non_blocking=True)
        float(step(r, w).item())
    e2e_s = (time.perf_counter() - t0) / args.steps

    # the same work as 32 per-scene calls
    per = [MultiViewRasterizer(cams[s], [0, 0, 0], 3, num_surfels=sizes[s], device=dev, cell_tiles=best[0],
                               blend_shape=best[1], stage_entries=best[3]) for s in range(n_scenes)]

    def per_scene():
        for s in range(n_scenes):
            a, b = offs[s], offs[s + 1]
            leaves = [t[a:b].detach().requires_grad_(True) for t in inputs]
            col, oth, _, _ = per[s](*leaves)
            w = w_dev[s * views:(s + 1) * views]
            ((col * w[:, :3]).sum() + (oth * w[:, 3:]).sum()).backward()
    per_scene()
    per_ms = timed(per_scene, max(2, args.steps // 2))

    line = {"metric": "uneven multi-scene fwd+bwd steps/s (32 scenes x 8 views x 400x300)",
            "value": 1000.0 / ms, "unit": "steps/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded scenes and loss weights)",
            "config": {"workload": MULTISCENE, "scenes": n_scenes, "surfels": offs[-1], "views_per_scene": views,
                       "height": H, "width": W, "cell_tiles": best[0], "blend_shape": best[1],
                       "tile_schedule": best[2], "stage_entries": best[3],
                       "autotune_ms": {f"cell{c}_shape{sh}_sched{sc}_stage{st}": round(v, 3)
                                       for (c, sh, sc, st), v in tune.items()},
                       "l2": "per-step working set (3.7M surfels x 8 views of records, lists, images) far larger than "
                             "the 129 MB L2"},
            "e2e": {"value": 1.0 / e2e_s, "unit": "steps/s", "h2d_bytes_per_step": int(w_host.numel() * 4),
                    "d2h_bytes_per_step": 4},
            "per_scene_calls_ms": round(per_ms, 3), "batched_speedup_over_per_scene": round(per_ms / ms, 3),
            "clocks": clk}
    if not args.no_reference_cuda:
        from oracle import ref_build, ref_cuda
        try:
            if not ref_cuda.available():
                ref_build.build()
            mod = ref_cuda.load("plain")
        except Exception as ex:   # sources not staged
            line["reference_cuda"] = {"unavailable": str(ex)[:200]}
        else:
            sets = [ref_cuda.settings(mod, c, [0.0, 0.0, 0.0], 3) for c in all_cams]

            def ref_all():
                for s in range(n_scenes):
                    a, b = offs[s], offs[s + 1]
                    leaves = [t[a:b].detach().requires_grad_(True) for t in inputs]
                    m2 = torch.zeros_like(leaves[0], requires_grad=True)
                    for k in range(views):
                        v = s * views + k
                        col, _, oth = mod.GaussianRasterizer(sets[v])(
                            means3D=leaves[0], means2D=m2, shs=leaves[2], colors_precomp=None,
                            opacities=leaves[1], scales=leaves[3], rotations=leaves[4])
                        ((col * w_dev[v, :3]).sum() + (oth * w_dev[v, 3:]).sum()).backward()
            ref_all()
            ref_ms = timed(ref_all, 2)
            line["reference_cuda"] = {"ms": round(ref_ms, 3), "speedup": round(ref_ms / ms, 3),
                                      "what": "reference diff_surfel_rasterization, 256 per-view calls through its "
                                              "GaussianRasterizer (forward + backward)"}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference", "reference-cuda"])
    ap.add_argument("--workload", default="sq500k_16x800x600")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-reference-cuda", action="store_true",
                    help="skip timing the reference's CUDA rasteriser on the same workload")
    ap.add_argument("--no-part", action="store_true",
                    help="skip timing the part variant's rasteriser (and the reference's) on the same workload")
    ap.add_argument("--cell-tiles", type=int, default=0, choices=[0, 1, 2, 4, 8, 16],
                    help="cell edge in tiles (0: cell edge, warp footprint, tile schedule and staged batch autotuned)")
    ap.add_argument("--blend-shape", type=int, default=0, choices=[0, 1],
                    help="with --cell-tiles: the blends' warp footprint (0: 16x2 strips, 1: 8-wide patches)")
    ap.add_argument("--tile-schedule", type=int, default=0, choices=[0, 1],
                    help="with --cell-tiles: 0 a CTA per tile, 1 persistent CTAs on a tile queue")
    ap.add_argument("--stage-entries", type=int, default=0, choices=[0, 64, 128, 256],
                    help="with --cell-tiles: list entries per staged batch of the blends (0: 256)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.impl == "reference-cuda":
        print(json.dumps({"impl": "reference-cuda", "workload": args.workload,
                          **(time_reference_cuda(args.workload, steps=args.steps, warmup=args.warmup) or
                             {"unavailable": "reference extension not built"})}), flush=True)
    elif args.workload == MULTISCENE:
        run_multiscene(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
