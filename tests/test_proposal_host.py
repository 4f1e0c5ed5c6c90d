"""Host-side pieces of the proposal network, on the CPU: the oracle's bf16
rounding against PyTorch's, the scene sampler's slot order and ranges, the
output decoding, the cell topology against the binding oracle's, and the
reference-style plain initialisation."""
import math

import numpy as np
import torch

from oracle import binding_oracle as BO
from oracle import proposal_oracle as O


def test_bf16_rounding_matches_torch():
    x = (np.random.default_rng(0).standard_normal(100_000) * 10 ** np.random.default_rng(1).uniform(-8, 8, 100_000))
    x = x.astype(np.float32)
    ref = torch.from_numpy(x).to(torch.bfloat16).float().numpy()
    np.testing.assert_array_equal(O.bf16(x), ref)


def test_scene_sampler_slots():
    from partgs_gb300 import sq_data as D
    b = D.sample_sq_batch(500, torch.Generator().manual_seed(0))
    k = b.counts
    assert int(k.min()) >= 1 and int(k.max()) <= 8
    assert bool((b.exist[:, :-1] >= b.exist[:, 1:]).all())              # existing slots first
    for s in range(500):
        x = b.trans[s, :int(k[s]), 0]
        assert bool((x[1:] >= x[:-1]).all())                            # sorted by centre x
    e = b.exist > 0
    assert float(b.semi[e].min()) >= 0.1 and float(b.semi[e].max()) <= 0.5
    assert float(b.eps[e].min()) >= 0.2 and float(b.eps[e].max()) <= 1.8
    assert bool((b.quat[..., 0] >= 0).all()) and torch.allclose(b.quat.norm(dim=-1), torch.ones(500, 8))
    assert float(b.trans.norm(dim=-1).max()) <= 1.0 + 1e-6


def test_binding_parameters_round_trip():
    from partgs_gb300 import sq_data as D
    b = D.sample_sq_batch(50, torch.Generator().manual_seed(1))
    sq_s, sq_eps, _, _ = D.to_binding_params(b.semi, b.eps, b.quat, b.trans)
    assert torch.allclose(D.RATIO * (torch.exp(sq_s) + D.SMIN), b.semi, atol=1e-6)
    assert torch.allclose(torch.sigmoid(sq_eps) * 1.8 + 0.1, b.eps, atol=1e-5)


def test_grid_topology_matches_binding_oracle():
    from partgs_gb300 import sq_data as D
    e, o, f = D.grid_topology(7, 9)
    e2, o2, f2 = BO.grid_topology(7, 9)
    np.testing.assert_allclose(e, e2)
    np.testing.assert_allclose(o, o2)
    np.testing.assert_array_equal(f, f2)


def test_decode_ranges():
    from partgs_gb300.proposal import decode
    out = torch.randn(4, 104) * 10
    semi, eps, quat, trans, logit = decode(out)
    assert float(semi.min()) >= 0.1 - 1e-6 and float(semi.max()) <= 0.5 + 1e-6
    assert float(eps.min()) >= 0.2 - 1e-6 and float(eps.max()) <= 1.8 + 1e-6
    assert torch.allclose(quat.norm(dim=-1), torch.ones(4, 8), atol=1e-6)


def test_plain_init_is_the_reference_block_init():
    from partgs_gb300.proposal import plain_init
    g = torch.Generator().manual_seed(0)
    pts = torch.cat([torch.randn(300, 3, generator=g) * 0.05 + c for c in (torch.tensor([0.5, 0, 0]),
                                                                            torch.tensor([-0.5, 0, 0]))])
    semi, eps, quat, c = plain_init(pts, 2, g)
    assert torch.allclose(semi, torch.full((2, 3), 0.25 * (0.25 + 0.2)))
    assert torch.allclose(eps, torch.ones(2, 2)) and torch.allclose(quat[:, 0], torch.ones(2))
    xs = sorted(float(v) for v in c[:, 0])
    assert abs(xs[0] + 0.5) < 0.05 and abs(xs[1] - 0.5) < 0.05
    assert math.isclose(0.25 * (math.exp(math.log(0.25)) + 0.2), 0.1125)


def test_kmeans_batch_finds_separated_clusters():
    """The batched k-means of the labelling fits: on scenes of well-separated
    blobs it puts one centre in each blob, per scene and with each scene's
    own block count; slots past the count stay zero."""
    from partgs_gb300.proposal import kmeans_batch
    g = torch.Generator().manual_seed(0)
    S, n = 5, 2048
    counts = [1, 3, 8, 5, 2]
    pts = torch.empty(S, n, 3)
    truth = []
    for s, k in enumerate(counts):
        c = torch.randn(k, 3, generator=g) * 4.0
        c = c + torch.arange(k)[:, None] * torch.tensor([10.0, 0.0, 0.0])     # blobs far apart
        lab = torch.arange(n) % k
        pts[s] = c[lab] + 0.05 * torch.randn(n, 3, generator=g)
        truth.append(c)
    got = kmeans_batch(pts, counts, seed=3)
    assert got.shape == (S, 8, 3)
    for s, k in enumerate(counts):
        d = torch.cdist(truth[s], got[s, :k])
        assert float(d.min(dim=1).values.max()) < 0.05, (s, d)       # every blob has a centre
        assert bool((got[s, k:] == 0).all())
