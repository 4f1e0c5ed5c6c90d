"""Parity against the reference's own CUDA rasterisers, compiled unmodified
for sm_103a (``oracle/ref_build.py``) and run through their own Python API
on the same inputs as this library's drop-in API.

Per case:
* radii, tile ranges, per-tile surfel lists, last and median contributor
  counts: bit-exact;
* RGB within 1e-5 of the reference's, relative to max(1, channel
  magnitude); the auxiliary maps (depth, alpha, normal, median depth,
  distortion, the final T / M1 / M2 planes, semantics) within 3e-5;
* gradients of every input within 1e-4 relative, as the L2 norm of the
  difference over the L2 norm of the reference's gradient tensor, against
  the reference and against the FP64 oracle; and, element by element, the
  largest difference within 1e-4 of the tensor's largest magnitude, except
  for the position, screen-space and rotation gradients (2e-4 in L2, 3e-4
  element-wise).  Those run
  through the splat-to-pixel matrix adjoint, whose FP32 evaluation cancels
  terms weighted by pixel coordinates per fragment: the reference binary
  itself lands up to 1.1e-4 from the FP64 oracle there on these cases (an
  FP32 restatement of the oracle, summing in FP64, up to 4.6e-4), while its
  L2 error stays below 6e-5.  The reference's own distances are printed.

Left out, with their upstream gradients zeroed, are the pixels and surfels
where the FP64 oracle finds a discrete decision (the alpha cut-off, the stop
test, the median switch, a radius or rectangle rounding, counting the
cancellation in the extent) within FP32 rounding, and the pixels where
rounding every surfel's matrix and centre by one FP32 unit moves the FP64
result by more than half the tolerance (oracle.fp32_sensitivity: nearly
edge-on splats make those pixels ill-conditioned in FP32, so that two FP32
evaluations cannot agree to the tolerance there).  Contributor counts also
skip the pixels whose list position a rounding-ambiguous surfel may shift.
The masks come from the FP64 oracle alone, so they do not depend on the
machine.  The same runs also pin the oracle to the reference binary.

Skipped when the reference extension is not built (it needs the reference's
sources staged under oracle/_ref/src)."""
import numpy as np
import pytest
import torch

from oracle import surfel_oracle as O
from tests._util import (GEOMETRY_GRADS, GRAD_L2_TOL_GEOMETRY, GRAD_TOL, GRAD_TOL_GEOMETRY, grad_error,
                         ill_conditioned, image_error, l2_error, oracle_camera, oracle_surfels, ours_render)

pytestmark = pytest.mark.gpu

IMG_TOL = 1e-5           # RGB
AUX_TOL = 3e-5           # auxiliary maps, final T planes, semantics


def _ref():
    from oracle import ref_build, ref_cuda
    if not ref_cuda.available():
        try:
            ref_build.build()
        except Exception as ex:   # sources not staged, or no compiler
            pytest.skip(f"reference CUDA rasteriser not built: {ex}")
        if not ref_cuda.available():
            pytest.skip("reference CUDA rasteriser not built (sources not staged under oracle/_ref/src)")
    return ref_cuda


def _scene_case(name):
    from partgs_gb300.cameras import orbit_cameras
    from partgs_gb300.scenes import random_surfels, workload
    g = torch.Generator()
    if name == "plain_random4k_128":
        scene, cams = workload("random4k_128")
        return dict(variant="plain", scene=scene, cam=cams[0], bg=[0.0, 0.0, 0.0], inputs="sh")
    if name == "plain_bg_64x80":             # the smoke() case
        return dict(variant="plain", scene=random_surfels(1024, seed=3), cam=orbit_cameras(1, 3.0, 64, 80, 60.0, seed=3)[0],
                    bg=[0.1, 0.2, 0.3], inputs="sh")
    if name == "plain_ragged_77x45":
        return dict(variant="plain", scene=random_surfels(2000, seed=17),
                    cam=orbit_cameras(1, 3.0, 45, 77, 60.0, seed=9)[0], bg=[0.2, 0.2, 0.2], inputs="sh")
    if name == "plain_colors_precomp":
        scene = random_surfels(1500, seed=51)
        cols = torch.rand(scene.P, 3, generator=g.manual_seed(7))
        return dict(variant="plain", scene=scene, cam=orbit_cameras(1, 3.0, 64, 80, 55.0, seed=23)[0],
                    bg=[0.1, 0.5, 0.3], inputs="colors", colors=cols)
    if name == "part_S8":
        scene = random_surfels(3000, seed=11)
        sem = torch.rand(scene.P, 8, generator=g.manual_seed(2))
        return dict(variant="part", scene=scene, cam=orbit_cameras(1, 3.0, 96, 112, 55.0, seed=5)[0],
                    bg=[0.3, 0.1, 0.2], inputs="sh", semantics=sem)
    if name == "part_colors_precomp":        # precomputed colours with scales / rotations
        scene = random_surfels(1500, seed=51)
        sem = torch.rand(scene.P, 4, generator=g.manual_seed(6))
        cols = torch.rand(scene.P, 3, generator=g.manual_seed(7))
        return dict(variant="part", scene=scene, cam=orbit_cameras(1, 3.0, 64, 80, 55.0, seed=23)[0],
                    bg=[0.1, 0.5, 0.3], inputs="colors", colors=cols, semantics=sem)
    raise KeyError(name)


CASES = ["plain_random4k_128", "plain_bg_64x80", "plain_ragged_77x45", "plain_colors_precomp", "part_S8",
         "part_colors_precomp"]


def _run(case):
    ref_cuda = _ref()
    sc, cam = case["scene"], case["cam"]
    part = case["variant"] == "part"
    kw = dict(means3D=sc.means3D, opacities=sc.opacities, scales=sc.scales, rotations=sc.rotations,
              semantics=case.get("semantics"))
    if case["inputs"] == "sh":
        kw["shs"] = sc.shs
    else:
        kw["colors_precomp"] = case["colors"]
    ocam = oracle_camera(cam)
    osf = oracle_surfels(sc, colors_precomp=case.get("colors"), semantics=case.get("semantics"))
    variant = O.PART if part else O.PLAIN
    st = O.forward_view(osf, ocam, np.array(case["bg"]), variant, np.float64)
    ill = ill_conditioned(st, ocam, osf, case["bg"], variant, IMG_TOL, AUX_TOL)
    amb_px = st.amb_pixel | ill
    amb_s, amb_t = st.amb_surfel, st.extra["amb_tiles"]
    amb_count = st.extra["amb_count_pixel"]
    g = np.random.default_rng(12)
    dcol = g.standard_normal(st.color.shape).astype(np.float32)
    doth = (g.standard_normal(st.others.shape) * 0.1).astype(np.float32)
    dsem = g.standard_normal(st.semantic.shape).astype(np.float32) if part else None
    for a in (dcol, doth, dsem):
        if a is not None:
            a[:, amb_px] = 0
    ups = (dcol, doth, dsem)
    ref = ref_cuda.render(case["variant"], cam, case["bg"], upstream=ups, **kw)
    ref2 = ref_cuda.render(case["variant"], cam, case["bg"], upstream=ups, **kw)
    ours = ours_render(case["variant"], cam, case["bg"], upstream=ups, **kw)
    o64 = O.backward_view(st, ocam, osf, np.array(case["bg"]), dcol, doth, dsem, variant=variant, dtype=np.float64)
    return dict(ref=ref, ref2=ref2, ours=ours, st=st, o64=o64, amb_px=amb_px, amb_s=amb_s, amb_t=amb_t, part=part,
                amb_count=amb_count, ill=ill)


_CACHE = {}


@pytest.fixture(scope="module", params=CASES)
def run(sgr_lib, request):
    if request.param not in _CACHE:
        _CACHE[request.param] = _run(_scene_case(request.param))
    return _CACHE[request.param]


def _grad_names(r):
    return sorted(k for k in r["ref"] if k.startswith("dL_d"))


def test_radii_bit_exact(run):
    ok = ~run["amb_s"]
    assert run["amb_s"].sum() <= 8
    np.testing.assert_array_equal(run["ours"]["radii"][ok], run["ref"]["radii"][ok])
    vis = (run["ref"]["radii"] > 0) & ok
    np.testing.assert_array_equal(run["ours"]["tiles_touched"][vis], run["ref"]["geom_tiles_touched"][vis])


def test_tile_ranges_and_lists_bit_exact(run):
    ref, ours, amb_t = run["ref"], run["ours"], run["amb_t"]
    rr, ro = ref["ranges"], ours["ranges"]
    checked = 0
    for t in range(rr.shape[0]):
        if amb_t[t]:
            continue
        a = ref["point_list"][rr[t, 0]:rr[t, 1]]
        b = ours["point_list"][ro[t, 0]:ro[t, 1]]
        np.testing.assert_array_equal(b, a, err_msg=f"tile {t}")
        checked += 1
    assert checked >= 0.75 * rr.shape[0]
    if not amb_t.any():
        assert ours["num_rendered"] == ref["num_rendered"]
        np.testing.assert_array_equal(ro, rr)


def test_contributors_bit_exact(run):
    amb = run["amb_count"]     # a rounding-ambiguous surfel's band tiles: two of twenty on the smallest image
    assert amb.mean() < 0.1
    for k in range(2):
        np.testing.assert_array_equal(run["ours"]["n_contrib"][k][~amb], run["ref"]["n_contrib"][k][~amb])


def test_images(run):
    amb = run["amb_px"]
    assert amb.mean() < 0.02, (run["ill"].mean(), amb.mean())
    ours, ref = run["ours"], run["ref"]
    errs = {"color": max(image_error(ours["color"], ref["color"], amb)),
            "allmap": max(image_error(ours["allmap"], ref["allmap"], amb)),
            "final_T": max(image_error(ours["final_T"], ref["final_T"], amb))}
    if run["part"]:
        errs["semantic"] = max(image_error(ours["semantic"], ref["semantic"], amb))
    print("image errors vs reference CUDA:", errs)
    assert errs["color"] <= IMG_TOL, errs
    assert max(v for k, v in errs.items() if k != "color") <= AUX_TOL, errs


def test_gradients(run):
    ours, ref, ref2, o64 = run["ours"], run["ref"], run["ref2"], run["o64"]
    report, bad = {}, {}
    for k in _grad_names(run):
        a, b = ours[k].reshape(-1), ref[k].reshape(-1)
        c = np.asarray(o64[k]).reshape(-1)
        e_max = grad_error(a, b)
        e_l2 = l2_error(a, b)
        e_l2_64 = l2_error(a, c)
        report[k] = dict(max=f"{e_max:.2e}", l2=f"{e_l2:.2e}", l2_fp64=f"{e_l2_64:.2e}",
                         ref_max_fp64=f"{grad_error(b, c):.2e}", ref_l2_fp64=f"{l2_error(b, c):.2e}",
                         ref_run_to_run=f"{grad_error(ref2[k].reshape(-1), b):.1e}")
        tol = GRAD_TOL_GEOMETRY if k in GEOMETRY_GRADS else GRAD_TOL
        tol_l2 = GRAD_L2_TOL_GEOMETRY if k in GEOMETRY_GRADS else GRAD_TOL
        if e_max > tol or e_l2 > tol_l2 or e_l2_64 > tol_l2:
            bad[k] = report[k]
    print("gradients vs reference CUDA:", report)
    assert not bad, bad


def test_oracle_pinned_to_reference(run):
    """The FP64 oracle against the reference binary: radii and contributor
    counts exact; images within 2e-5 (RGB) and 5e-5 (auxiliary maps): the
    reference's FP32 evaluation sits up to 1.8e-5 / 4.4e-5 from FP64 on the
    background case, and ours within 3.2e-6 / 7.9e-6 of the reference."""
    st, ref, amb = run["st"], run["ref"], run["amb_px"]
    cnt = run["amb_count"]
    for k in range(2):
        np.testing.assert_array_equal(st.n_contrib[k][~cnt], ref["n_contrib"][k][~cnt])
    ok = ~run["amb_s"]
    np.testing.assert_array_equal(st.radii[ok], ref["radii"][ok])
    e = max(image_error(ref["color"], st.color, amb))
    e_aux = max(image_error(ref["allmap"], st.others, amb))
    print("reference CUDA vs FP64 oracle:", e, e_aux)
    assert e <= 2e-5 and e_aux <= 5e-5, (e, e_aux)
