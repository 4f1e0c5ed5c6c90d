"""CPU restatement of the reference's Chamfer evaluation.

TEST INFRASTRUCTURE ONLY: the checker of ``partgs_gb300.chamfer_eval``.
Follows utils/blender_eval.py:15-111 (evaluate_mesh, sample_single_tri) with
numpy and scipy's cKDTree standing in for scikit-learn's kd-tree
NearestNeighbors (both exact; scikit-learn is absent on the GPU host), and
the shuffle given as a permutation so both sides see the same order.
"""
from __future__ import annotations

import numpy as np
from scipy.spatial import cKDTree

MAX_DIST = 1.0
DOWNSAMPLE_DENSITY = 0.005


def sample_single_tri(n1, n2, v1, v2, tri_vert):
    """utils/blender_eval.py:15-23."""
    c = np.mgrid[:n1 + 1, :n2 + 1].astype(np.float64)
    c += 0.5
    c[0] /= max(n1, 1e-7)
    c[1] /= max(n2, 1e-7)
    c = np.transpose(c, (1, 2, 0))
    k = c[c.sum(axis=-1) < 1]
    return v1 * k[:, :1] + v2 * k[:, 1:] + tri_vert


def sample_mesh(vertices, triangles, density=DOWNSAMPLE_DENSITY):
    """utils/blender_eval.py:39-69 (vertices first, triangles in order)."""
    vertices = np.asarray(vertices, np.float64)
    tri_vert = vertices[np.asarray(triangles)]
    v1 = tri_vert[:, 1] - tri_vert[:, 0]
    v2 = tri_vert[:, 2] - tri_vert[:, 0]
    l1 = np.linalg.norm(v1, axis=-1, keepdims=True)
    l2 = np.linalg.norm(v2, axis=-1, keepdims=True)
    area2 = np.linalg.norm(np.cross(v1, v2), axis=-1, keepdims=True)
    nz = (area2 > 0)[:, 0]
    l1, l2, area2, v1, v2, tri_vert = [a[nz] for a in (l1, l2, area2, v1, v2, tri_vert)]
    thr = density * np.sqrt(l1 * l2 / area2)
    n1 = np.floor(l1 / thr)
    n2 = np.floor(l2 / thr)
    pts = [sample_single_tri(int(n1[i, 0]), int(n2[i, 0]), v1[i:i + 1], v2[i:i + 1], tri_vert[i:i + 1, 0])
           for i in range(len(n1))]
    return np.concatenate([vertices] + pts, axis=0)


def downsample_mask(pcd, density=DOWNSAMPLE_DENSITY):
    """utils/blender_eval.py:76-83: in order, a kept point removes its radius neighbours."""
    tree = cKDTree(pcd)
    nbrs = tree.query_ball_point(pcd, r=density)
    mask = np.ones(pcd.shape[0], dtype=bool)
    for curr, idxs in enumerate(nbrs):
        if mask[curr]:
            mask[idxs] = False
            mask[curr] = True
    return mask


def drop_unreferenced(vertices, triangles):
    """Open3D's remove_unreferenced_vertices (utils/blender_eval.py:34)."""
    vertices = np.asarray(vertices)
    triangles = np.asarray(triangles)
    keep = np.unique(triangles.reshape(-1))
    remap = -np.ones(vertices.shape[0], dtype=np.int64)
    remap[keep] = np.arange(keep.shape[0])
    return vertices[keep], remap[triangles]


def evaluate(vertices, triangles, stl, perm, max_dist=MAX_DIST, density=DOWNSAMPLE_DENSITY):
    """utils/blender_eval.py:34-111 with the shuffle ``perm``: (acc, comp, avg, pcd, mask)."""
    vertices, triangles = drop_unreferenced(vertices, triangles)
    pcd = sample_mesh(vertices, triangles, density)[perm]
    mask = downsample_mask(pcd, density)
    down = pcd[mask]
    d2s, _ = cKDTree(stl).query(pcd, k=1)
    s2d, _ = cKDTree(down).query(stl, k=1)
    acc = d2s[d2s < max_dist].mean()
    comp = s2d[s2d < max_dist].mean()
    return acc, comp, (acc + comp) / 2, pcd, mask
