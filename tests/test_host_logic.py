"""Host-side logic that needs no GPU: the drop-in API's argument checks,
the scene / view tables, the synthetic workloads."""
import numpy as np
import pytest
import torch

import partgs_gb300.diff_surfel_rasterization as dsr
import partgs_gb300.diff_surfel_rasterization_part as dsrp
from partgs_gb300 import _lib as L
from partgs_gb300 import raster


def _settings(mod):
    return mod.GaussianRasterizationSettings(
        image_height=8, image_width=8, tanfovx=0.5, tanfovy=0.5, bg=torch.zeros(3), scale_modifier=1.0,
        viewmatrix=torch.eye(4), projmatrix=torch.eye(4), sh_degree=0, campos=torch.zeros(3), prefiltered=False,
        debug=False)


def test_settings_fields_match_the_reference():
    assert dsr.GaussianRasterizationSettings._fields == (
        "image_height", "image_width", "tanfovx", "tanfovy", "bg", "scale_modifier", "viewmatrix", "projmatrix",
        "sh_degree", "campos", "prefiltered", "debug")
    assert dsrp.GaussianRasterizationSettings is dsr.GaussianRasterizationSettings


@pytest.mark.parametrize("mod", [dsr, dsrp])
def test_exactly_one_colour_source(mod):
    r = mod.GaussianRasterizer(_settings(mod))
    x = torch.zeros(4, 3)
    extra = {"semantics": torch.zeros(4, 2)} if mod is dsrp else {}
    with pytest.raises(Exception, match="excatly one of either SHs or precomputed colors"):
        r(means3D=x, means2D=x, opacities=torch.ones(4, 1), scales=torch.ones(4, 2), rotations=torch.ones(4, 4),
          **extra)
    with pytest.raises(Exception, match="exactly one of either scale/rotation pair"):
        r(means3D=x, means2D=x, opacities=torch.ones(4, 1), colors_precomp=x, **extra)


def test_semantic_channel_limit():
    with pytest.raises(ValueError, match="at most 16 semantic channels"):
        raster.make_batch(L.SGR_VARIANT_PART, torch.zeros(4, 3), torch.ones(4), None, torch.zeros(4, 3),
                          torch.ones(4, 2), torch.ones(4, 4), None, torch.zeros(4, 17),
                          raster.ViewSet(torch.eye(4).reshape(1, 16), torch.eye(4).reshape(1, 16), torch.zeros(1, 3),
                                         [(0.5, 0.5)], 8, 8), torch.zeros(3), 0, 1.0, False)


def test_tables_for_uneven_scenes():
    vs = raster.ViewSet(torch.zeros(5, 16), torch.zeros(5, 16), torch.zeros(5, 3), [(0.5, 0.6)] * 5, 8, 8,
                        scene_sizes=[3, 7], scene_views=[2, 3])
    sct, vwt, n, R = raster._tables(L.SGR_VARIANT_PLAIN, 10, vs, torch.device("cpu"))
    scenes = np.frombuffer(sct.numpy().tobytes(), dtype=np.int32).reshape(-1, 4)
    views = np.frombuffer(vwt.numpy().tobytes(), dtype=np.int32).reshape(-1, 4)
    np.testing.assert_array_equal(scenes, [[0, 3, 0, 2], [3, 7, 2, 3]])
    np.testing.assert_array_equal(views[:, :2], [[0, 0], [0, 3], [1, 6], [1, 13], [1, 20]])
    assert n == 2 and R == 27
    assert np.allclose(views[:, 2:].view(np.float32), [[0.5, 0.6]] * 5)
    with pytest.raises(ValueError):
        raster._tables(L.SGR_VARIANT_PLAIN, 11, vs, torch.device("cpu"))


def test_workloads_are_seeded_and_shaped():
    from partgs_gb300.scenes import random_surfels, superquadric_surfels
    a, b = random_surfels(256, seed=4), random_surfels(256, seed=4)
    assert torch.equal(a.means3D, b.means3D) and torch.equal(a.shs, b.shs)
    assert a.shs.shape == (256, 16, 3) and a.scales.shape == (256, 2) and a.rotations.shape == (256, 4)
    np.testing.assert_allclose(a.rotations.norm(dim=1).numpy(), 1.0, rtol=1e-6)
    s = superquadric_surfels(1000, 4, seed=1)
    assert s.P == 1000 and torch.isfinite(s.means3D).all()


@pytest.mark.parametrize("mod", [dsr, dsrp])
def test_host_tensors_are_rejected_before_any_device_work(sgr_lib, mod):
    """Inputs in host memory raise ValueError in the host layer, before any
    pointer reaches the library (a kernel given a host address would fault)."""
    r = mod.GaussianRasterizer(_settings(mod))
    x = torch.zeros(4, 3)
    extra = {"semantics": torch.zeros(4, 2)} if mod is dsrp else {}
    launches = sgr_lib.sgr_kernel_launches()
    with pytest.raises(ValueError, match="must be CUDA tensors"):
        r(means3D=x, means2D=x, opacities=torch.ones(4, 1), colors_precomp=x, scales=torch.ones(4, 2),
          rotations=torch.ones(4, 4), **extra)
    assert sgr_lib.sgr_kernel_launches() == launches
