"""Known-answer cases derived by hand, and finite-difference checks of the
oracle's backward (the restatement of the reference's hand-written
adjoints), all in float64 on the CPU."""
import math

import numpy as np
import pytest

from oracle import surfel_oracle as O


def _camera(W=33, H=33, tan=0.5, dist=3.0):
    """Camera at (0, 0, -dist) looking along +z, P00 = 1/tan exactly."""
    wv = np.eye(4)
    wv[3, 2] = dist                       # row-vector form: p_view = p + (0, 0, dist)
    znear, zfar = 0.01, 100.0
    P = np.zeros((4, 4))
    P[0, 0] = 1.0 / tan
    P[1, 1] = 1.0 / tan
    P[3, 2] = 1.0
    P[2, 2] = zfar / (zfar - znear)
    P[2, 3] = -(zfar * znear) / (zfar - znear)
    full = wv @ P.T
    return O.Camera(wv.reshape(-1), full.reshape(-1), np.array([0.0, 0.0, -dist]), tan, tan, H, W)


def _one_surfel(sigma=0.1, opacity=0.7, rgb=(0.2, 0.5, 0.8)):
    return O.Surfels(means3D=np.zeros((1, 3)), opacities=np.array([opacity]), scales=np.array([[sigma, sigma]]),
                     rotations=np.array([[1.0, 0.0, 0.0, 0.0]]), colors_precomp=np.array([rgb]))


@pytest.mark.parametrize("variant", [O.PLAIN, O.PART])
def test_single_fronto_parallel_surfel(variant):
    """A surfel facing the camera: alpha = o exp(-rho/2) with
    rho = min((k d / (f sigma))^2, 2 k^2) at k pixels from the centre, depth
    d, normal toward the camera, colour rgb * alpha."""
    cam = _camera()
    s = _one_surfel()
    st = O.forward_view(s, cam, np.zeros(3), variant, np.float64)
    f = 33 / (2 * 0.5)
    d, sigma, o = 3.0, 0.1, 0.7
    # plain: ndc2pix maps the centre to (W-1)/2 = 16 with integer pixel
    # centres; part: to W/2 = 16.5 with half-pixel centres, i.e. pixel 16 too
    cy = 16
    for k in [0, 1, 2, 4]:
        x = 16 + k
        rho3d = (k * d / (f * sigma)) ** 2
        rho2d = 2.0 * k * k
        alpha = o * math.exp(-0.5 * min(rho3d, rho2d))
        if alpha < 1 / 255:
            assert st.others[1, cy, x] == 0
            continue
        np.testing.assert_allclose(st.others[1, cy, x], alpha, rtol=1e-9)
        np.testing.assert_allclose(st.color[:, cy, x], np.array([0.2, 0.5, 0.8]) * alpha, rtol=1e-9)
        np.testing.assert_allclose(st.others[0, cy, x], d * alpha, rtol=1e-9)              # expected depth
        np.testing.assert_allclose(st.others[2:5, cy, x], np.array([0, 0, -1.0]) * alpha, atol=1e-12)
        np.testing.assert_allclose(st.others[5, cy, x], d, rtol=1e-9)                      # median depth
        assert st.others[6, cy, x] == 0                                                    # one fragment
    assert st.radii[0] == math.ceil(3 * sigma * f / d) or variant == O.PART


def test_two_surfels_front_to_back():
    """Two coincident-footprint surfels at depths 2 and 3: the nearer one
    blends first; T, distortion and the median follow the 2DGS formulas."""
    cam = _camera(dist=3.0)
    s = O.Surfels(means3D=np.array([[0, 0, 0.0], [0, 0, -1.0]]), opacities=np.array([0.6, 0.5]),
                  scales=np.array([[0.1, 0.1], [0.1, 0.1]]), rotations=np.array([[1.0, 0, 0, 0]] * 2),
                  colors_precomp=np.array([[1.0, 0, 0], [0, 1.0, 0]]))
    st = O.forward_view(s, cam, np.zeros(3), O.PLAIN, np.float64)
    a_near, a_far = 0.5, 0.6          # depth 2 (index 1) then depth 3 (index 0), at the centre pixel
    T1 = 1 - a_near
    w_near, w_far = a_near, a_far * T1
    np.testing.assert_allclose(st.color[:, 16, 16], [w_far, w_near, 0], rtol=1e-12)
    np.testing.assert_allclose(st.others[1, 16, 16], 1 - T1 * (1 - a_far), rtol=1e-12)
    near, far = 0.2, 100.0
    m = lambda z: far / (far - near) * (1 - near / z)  # noqa: E731
    dist = (m(3) ** 2 * (1 - T1) + m(2) ** 2 * w_near - 2 * m(3) * m(2) * w_near) * w_far
    np.testing.assert_allclose(st.others[6, 16, 16], dist, rtol=1e-10)
    # the median moves only while T > 0.5; T is exactly 0.5 before the far
    # surfel, so the near surfel (first contributor) stays the median
    np.testing.assert_allclose(st.others[5, 16, 16], 2.0, rtol=1e-12)
    assert st.n_contrib[0, 16, 16] == 2 and st.n_contrib[1, 16, 16] == 1


def _scene(seed=0, P=6):
    g = np.random.default_rng(seed)
    q = g.standard_normal((P, 4))
    q[:, 0] = np.abs(q[:, 0]) + 1.0
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    return O.Surfels(means3D=g.uniform(-0.4, 0.4, (P, 3)), opacities=g.uniform(0.3, 0.9, P),
                     scales=np.exp(g.normal(-2.2, 0.3, (P, 2))), rotations=q,
                     shs=g.normal(0, 0.3, (P, 16, 3)), sh_degree=3)


def _loss_and_grads(s, cam, wc, wo):
    st = O.forward_view(s, cam, np.array([0.1, 0.2, 0.3]), O.PLAIN, np.float64)
    L = float((st.color * wc).sum() + (st.others * wo).sum())
    return L, st


@pytest.mark.parametrize("name,shape_idx", [("means3D", None), ("scales", None), ("rotations", None),
                                            ("opacities", None), ("shs", None)])
def test_backward_matches_finite_differences(name, shape_idx):
    """The restated backward is the gradient of the restated forward
    (central differences in float64, away from discrete decisions)."""
    cam = _camera(W=24, H=24, tan=0.5, dist=2.5)
    s = _scene()
    g = np.random.default_rng(3)
    wc = g.standard_normal((3, 24, 24))
    wo = g.standard_normal((7, 24, 24)) * 0.1
    wo[5] = 0.0          # the median depth jumps between surfels: not differentiable
    L0, st = _loss_and_grads(s, cam, wc, wo)
    grads = O.backward_view(st, cam, s, np.array([0.1, 0.2, 0.3]), wc, wo, variant=O.PLAIN, dtype=np.float64)
    key = {"means3D": "dL_dmeans3D", "scales": "dL_dscales", "rotations": "dL_drotations",
           "opacities": "dL_dopacity", "shs": "dL_dsh"}[name]
    an = np.asarray(grads[key]).reshape(getattr(s, name).shape)
    base = getattr(s, name)
    eps = 1e-6
    fd = np.zeros_like(base)
    it = np.nditer(base, flags=["multi_index"])
    for _ in it:
        idx = it.multi_index
        if name == "shs" and idx[1] > 8:
            continue   # keep the loop short: degree <= 2 coefficients
        for sgn in (1, -1):
            pert = base.copy()
            pert[idx] += sgn * eps
            s2 = O.Surfels(**{**s.__dict__, name: pert})
            Lp, _ = _loss_and_grads(s2, cam, wc, wo)
            fd[idx] += sgn * Lp / (2 * eps)
    if name == "rotations":
        # the reference returns dL/d(normalised q); project both onto the
        # tangent space of the unit quaternion
        q = base / np.linalg.norm(base, axis=1, keepdims=True)
        an = an - q * np.sum(an * q, 1, keepdims=True)
        fd = fd - q * np.sum(fd * q, 1, keepdims=True)
    if name == "shs":
        an = an[:, :9]
        fd = fd[:, :9]
    err = np.abs(an - fd).max() / max(1e-9, np.abs(fd).max())
    assert err < 2e-4, (name, err)


def test_scale_modifier_applies_to_the_plain_variant_only():
    """The plain variant scales the tangent axes by scale_modifier
    (P0/cr/forward.cu:75-115, scale_to_mat(scale, mod)); the part variant's
    computeTransMat builds its scale matrix with 1.0 whatever the modifier
    (P1/cr/forward.cu:95).  The oracle keeps both."""
    cam = _camera()

    def render(variant, mod):
        s = _one_surfel()
        s.scale_modifier = mod
        return O.forward_view(s, cam, np.zeros(3), variant, np.float64)

    part_a, part_b = render(O.PART, 0.5), render(O.PART, 1.0)
    np.testing.assert_array_equal(part_a.color, part_b.color)
    np.testing.assert_array_equal(part_a.others, part_b.others)
    plain_a, plain_b = render(O.PLAIN, 0.5), render(O.PLAIN, 1.0)
    assert (plain_a.others[1] > 0).sum() < (plain_b.others[1] > 0).sum()      # a smaller footprint
