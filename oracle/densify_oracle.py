"""CPU restatement of the densification statistics.

TEST INFRASTRUCTURE ONLY: the checker of ``sgr_densify_stats``.  Follows
train.py:293-297 and scene/gaussian_model.py:515-517, one iteration per
view: where radii > 0, max_radii2D = max(max_radii2D, radii), accum +=
|grad[:2]|, denom += 1.
"""
from __future__ import annotations

import numpy as np


def stats(scenes, views, radii, grads, max_radii, accum, denom, grad_scale=1.0):
    """scenes: [(surfel_offset, count, view_begin, view_count)], views:
    [(scene, record_offset)], radii [R] int, grads [R,3]; updates the three
    per-surfel arrays (copies returned)."""
    max_radii, accum, denom = max_radii.copy(), accum.copy(), denom.copy()
    for so, n, vb, vn in scenes:
        for v in range(vb, vb + vn):
            ro = views[v][1]
            r = radii[ro:ro + n]
            vis = r > 0
            idx = np.arange(so, so + n)[vis]
            max_radii[idx] = np.maximum(max_radii[idx], r[vis].astype(np.float32))
            g = grads[ro:ro + n][vis]
            accum[idx] += (np.sqrt(g[:, 0].astype(np.float32) ** 2 + g[:, 1].astype(np.float32) ** 2)
                           * np.float32(grad_scale))
            denom[idx] += 1
    return max_radii, accum, denom
