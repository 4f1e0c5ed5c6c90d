"""The oracle pinned to golden vectors of the reference's own CUDA
rasterisers (compiled unmodified for sm_103a and run on a GB300 by
tests/golden/make_ref_cuda_golden.py): plain and part variants, SH colours
and precomputed colours, with semantics.

CPU only.  Integer state bit-exact (radii, per-pixel last and median
contributors, tile ranges and lists), away from the decisions the FP64
oracle finds within FP32 rounding (masks stored with the vectors); images
within 1e-5 (RGB) and 3e-5 (auxiliary maps, semantics) relative to
max(1, channel magnitude); gradients within 1e-4 relative in the L2 norm
of each tensor, and element by element within 1e-4 of each tensor's largest
magnitude, except the screen-space and 3D position and rotation gradients.
Those run through the transMat adjoint, whose FP32 evaluation cancels terms
weighted by pixel coordinates: the reference binary itself lands 1e-4 to
3.3e-4 from the FP64 oracle there (an FP32 restatement of the oracle lands
as far), so their element-wise bar is 5e-4."""
import glob
import os

import numpy as np
import pytest

from oracle import surfel_oracle as O
from tests._util import GEOMETRY_GRADS, GRAD_L2_TOL_GEOMETRY, grad_error, image_error, l2_error

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FILES = sorted(glob.glob(os.path.join(HERE, "ref_cuda_*.npz")))
IMG_TOL, AUX_TOL = 1e-5, 3e-5
GRAD_TOL = 1e-4
GRAD_TOL_GEOMETRY = 5e-4     # the reference binary's own FP32 error reaches 3.3e-4 here


@pytest.fixture(scope="module", params=FILES, ids=lambda p: os.path.basename(p)[9:-4])
def golden(request):
    z = dict(np.load(request.param))
    variant = O.PART if str(z["variant"]) == "part" else O.PLAIN
    H, W = (int(x) for x in z["hw"])
    cam = O.Camera(z["viewmatrix"].reshape(-1), z["projmatrix"].reshape(-1), z["campos"], float(z["tanfov"][0]),
                   float(z["tanfov"][1]), H, W)
    s = O.Surfels(z["means3D"], z["opacities"], z["scales"], z["rotations"], shs=z.get("shs"),
                  colors_precomp=z.get("colors_precomp"), semantics=z.get("semantics"), sh_degree=3)
    bg = z["bg"].astype(np.float64)
    st = O.forward_view(s, cam, bg, variant, np.float64)
    grads = O.backward_view(st, cam, s, bg, z["dL_dcolor_in"], z["dL_dothers_in"], z.get("dL_dsemantic_in"),
                            variant=variant, dtype=np.float64)
    return z, st, grads


def test_golden_files_present():
    assert len(FILES) >= 3


def test_radii_and_tiles_touched(golden):
    z, st, _ = golden
    ok = ~z["amb_surfel"]
    np.testing.assert_array_equal(st.radii[ok], z["ref_radii"][ok])
    if "ref_geom_tiles_touched" in z:
        np.testing.assert_array_equal(st.tiles_touched[ok], z["ref_geom_tiles_touched"][ok])


def test_tile_lists(golden):
    z, st, _ = golden
    amb_t = z["amb_tiles"]
    rr = z["ref_ranges"]
    for t in range(rr.shape[0]):
        if amb_t[t]:
            continue
        np.testing.assert_array_equal(st.point_list[st.ranges[t, 0]:st.ranges[t, 1]],
                                      z["ref_point_list"][rr[t, 0]:rr[t, 1]], err_msg=f"tile {t}")
    if not amb_t.any():
        assert len(st.point_list) == int(z["ref_num_rendered"])


def test_contributors(golden):
    z, st, _ = golden
    amb = z["amb_count_pixel"] if "amb_count_pixel" in z else z["amb_pixel"]
    assert amb.mean() < 0.1
    for k in range(2):
        np.testing.assert_array_equal(st.n_contrib[k][~amb], z["ref_n_contrib"][k][~amb])


def test_images(golden):
    z, st, _ = golden
    amb = z["amb_pixel"]
    assert max(image_error(z["ref_color"], st.color, amb)) <= IMG_TOL
    assert max(image_error(z["ref_allmap"], st.others, amb)) <= AUX_TOL
    assert max(image_error(z["ref_final_T"], st.final_T, amb)) <= AUX_TOL
    if "ref_semantic" in z:
        assert max(image_error(z["ref_semantic"], st.semantic, amb)) <= AUX_TOL


def test_preprocess_geometry(golden):
    """The splat-to-pixel matrices and screen centres of the visible surfels."""
    z, st, _ = golden
    if "ref_geom_transmat" not in z:
        pytest.skip("vectors written without the geometry buffer")
    vis = (z["ref_radii"] > 0) & ~z["amb_surfel"]
    T = z["ref_geom_transmat"][vis].astype(np.float64)
    To = st.transmat[vis]
    assert np.abs(T - To).max() / np.abs(To).max() < 1e-6
    m2 = z["ref_geom_means2D"][vis].astype(np.float64)
    assert np.abs(m2 - st.means2D[vis]).max() < 1e-3      # pixels


def test_gradients(golden):
    z, _, grads = golden
    names = [k[4:] for k in z if k.startswith("ref_dL_d")]
    got = {k: np.asarray(grads[k], np.float64).reshape(z["ref_" + k].shape) for k in names}
    want = {k: z["ref_" + k] for k in names}
    errs, bad = {}, {}
    for k in names:   # the oracle against the reference binary: L2 1e-4, largest element 1e-4 / 5e-4
        e = (grad_error(got[k], want[k]), l2_error(got[k], want[k]))
        errs[k] = e
        geo = k in GEOMETRY_GRADS
        if e[0] > (GRAD_TOL_GEOMETRY if geo else GRAD_TOL) or e[1] > (GRAD_L2_TOL_GEOMETRY if geo else GRAD_TOL):
            bad[k] = e
    assert not bad, errs
