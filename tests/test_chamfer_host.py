"""The Chamfer evaluation's host side on the CPU: mesh sampling and the
removal of unreferenced vertices agree with the numpy restatement of the
reference (utils/blender_eval.py:15-69) bit for bit, including a degenerate
triangle (skipped, as the reference's zero-area filter does) and vertices
no triangle uses."""
import numpy as np
import torch

from oracle import chamfer_oracle as O


def _mesh():
    g = np.random.default_rng(5)
    v = g.standard_normal((60, 3)) * 0.3
    f = g.integers(0, 50, size=(80, 3))            # vertices 50..59 are unreferenced
    f[3] = [7, 7, 9]                                 # a zero-area triangle
    return v, f


def test_unreferenced_vertices_are_dropped_like_open3d():
    from partgs_gb300 import chamfer_eval as E
    v, f = _mesh()
    v1, f1 = E.drop_unreferenced(v, f)
    v2, f2 = O.drop_unreferenced(v, f)
    np.testing.assert_array_equal(v1, v2)
    np.testing.assert_array_equal(f1, f2)
    assert v1.shape[0] <= 50 and np.array_equal(v1[f1], v[f])


def test_mesh_samples_are_the_references_bit_for_bit():
    from partgs_gb300 import chamfer_eval as E
    v, f = E.drop_unreferenced(*_mesh())
    for density in (0.02, 0.005):
        mine = E.sample_mesh(v, f, density, device="cpu").numpy()
        ref = O.sample_mesh(v, f, density)
        assert mine.shape == ref.shape
        np.testing.assert_array_equal(mine, ref)
    assert torch.get_default_dtype() == torch.float32
