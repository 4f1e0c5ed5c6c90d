"""Surfel PLY files in the reference's layout, for interchange with its
checkpoints (scene/gaussian_model.py:280-363 and
games/block_mesh_splatting/scene/two_gaussian_model.py:257-336).

One ``vertex`` element of float32 properties, in this order:
x y z, nx ny nz (zeros), f_dc_0..2, f_rest_0..3(M-1)-1 (each channel's
coefficients together: the [P, M-1, 3] tensor transposed to [P, 3, M-1]),
opacity (the logit), semantic_0.. (the part model only), scale_0.. (log
scales), rot_0..3.  Written as binary little-endian PLY 1.0; read from
binary (either byte order) or ASCII PLY with the properties in any order,
names sorted by their index as the reference's loader does.
"""
from __future__ import annotations

import os

import numpy as np
import torch

_PLY_TYPES = {"char": "i1", "int8": "i1", "uchar": "u1", "uint8": "u1", "short": "i2", "int16": "i2",
              "ushort": "u2", "uint16": "u2", "int": "i4", "int32": "i4", "uint": "u4", "uint32": "u4",
              "float": "f4", "float32": "f4", "double": "f8", "float64": "f8"}


def attribute_names(n_rest: int, n_scale: int = 2, n_rot: int = 4, n_semantic: int = 0, n_dc: int = 3):
    """construct_list_of_attributes: n_rest = 3 (M - 1) f_rest values."""
    names = ["x", "y", "z", "nx", "ny", "nz"]
    names += [f"f_dc_{i}" for i in range(n_dc)]
    names += [f"f_rest_{i}" for i in range(n_rest)]
    names.append("opacity")
    names += [f"semantic_{i}" for i in range(n_semantic)]
    names += [f"scale_{i}" for i in range(n_scale)]
    names += [f"rot_{i}" for i in range(n_rot)]
    return names


def _np(t):
    return t.detach().float().cpu().numpy() if torch.is_tensor(t) else np.asarray(t, dtype=np.float32)


def save_ply(path, xyz, f_dc, f_rest, opacity, scaling, rotation, semantic=None):
    """Writes the surfels; f_dc [P,1,3], f_rest [P,M-1,3], opacity [P,1]
    logits, scaling [P,S] log scales, rotation [P,4], semantic [P,K] or None."""
    xyz = _np(xyz)
    P = xyz.shape[0]
    cols = [xyz, np.zeros_like(xyz), _np(f_dc).transpose(0, 2, 1).reshape(P, -1),
            _np(f_rest).transpose(0, 2, 1).reshape(P, -1), _np(opacity).reshape(P, 1)]
    n_sem = 0
    if semantic is not None:
        sem = _np(semantic).reshape(P, -1)
        n_sem = sem.shape[1]
        cols.append(sem)
    scale, rot = _np(scaling).reshape(P, -1), _np(rotation).reshape(P, -1)
    cols += [scale, rot]
    names = attribute_names(cols[3].shape[1], scale.shape[1], rot.shape[1], n_sem, cols[2].shape[1])
    data = np.ascontiguousarray(np.concatenate(cols, axis=1), dtype="<f4")
    assert data.shape[1] == len(names)
    header = ["ply", "format binary_little_endian 1.0", f"element vertex {P}"]
    header += [f"property float {n}" for n in names]
    header.append("end_header")
    d = os.path.dirname(os.path.abspath(path))
    os.makedirs(d, exist_ok=True)
    with open(path, "wb") as fh:
        fh.write(("\n".join(header) + "\n").encode("ascii"))
        fh.write(data.tobytes())


def _read_header(fh):
    lines = []
    while True:
        line = fh.readline()
        if not line:
            raise ValueError("PLY header has no end_header")
        line = line.decode("ascii").strip()
        lines.append(line)
        if line == "end_header":
            return lines


def read_vertices(path) -> dict:
    """The vertex element's properties as {name: float array}."""
    with open(path, "rb") as fh:
        lines = _read_header(fh)
        if lines[0] != "ply":
            raise ValueError("not a PLY file")
        fmt = lines[1].split()[1]
        elements = []
        for ln in lines[2:]:
            tok = ln.split()
            if not tok or tok[0] in ("comment", "obj_info"):
                continue
            if tok[0] == "element":
                elements.append((tok[1], int(tok[2]), []))
            elif tok[0] == "property":
                if tok[1] == "list":
                    elements[-1][2].append((tok[4], None))
                else:
                    elements[-1][2].append((tok[2], _PLY_TYPES[tok[1]]))
        body = fh.read()
    if fmt == "ascii":   # one line per element entry
        rows = [r for r in body.decode("ascii").splitlines() if r.strip()]
        start = 0
        for name, count, props in elements:
            if name == "vertex":
                arr = np.array([[float(x) for x in r.split()] for r in rows[start:start + count]],
                               dtype=np.float64).reshape(count, len(props))
                return {p: arr[:, i] for i, (p, _) in enumerate(props)}
            start += count
        raise ValueError("PLY file has no vertex element")
    if fmt not in ("binary_little_endian", "binary_big_endian"):
        raise ValueError(f"unknown PLY format {fmt}")
    order = "<" if fmt == "binary_little_endian" else ">"
    off = 0
    for name, count, props in elements:
        if any(t is None for _, t in props):
            raise ValueError(f"list properties in binary element {name} are not supported")
        dt = np.dtype([(p, order + t) for p, t in props])
        if name == "vertex":
            arr = np.frombuffer(body, dtype=dt, count=count, offset=off)
            return {p: arr[p].astype(np.float64) for p, _ in props}
        off += dt.itemsize * count
    raise ValueError("PLY file has no vertex element")


def _sorted(props, prefix):
    names = [n for n in props if n.startswith(prefix)]
    return sorted(names, key=lambda x: int(x.split("_")[-1]))


def load_ply(path, sh_degree: int | None = None, device="cpu") -> dict:
    """{xyz [P,3], f_dc [P,1,3], f_rest [P,M-1,3], opacity [P,1], scaling
    [P,S], rotation [P,4], semantic [P,K] or None} as float32 tensors."""
    v = read_vertices(path)
    P = len(v["x"])
    xyz = np.stack([v["x"], v["y"], v["z"]], 1)
    f_dc = np.stack([v[f"f_dc_{i}"] for i in range(3)], 1)[:, :, None]            # [P,3,1]
    rest = _sorted(v, "f_rest_")
    if sh_degree is not None and len(rest) != 3 * (sh_degree + 1) ** 2 - 3:
        raise ValueError(f"{len(rest)} f_rest properties for SH degree {sh_degree}")
    f_rest = np.stack([v[n] for n in rest], 1).reshape(P, 3, -1) if rest else np.zeros((P, 3, 0))
    sem = _sorted(v, "semantic_")
    # the reference's loader takes every property starting with "rot" as a rotation
    rot_names = sorted([n for n in v if n.startswith("rot")], key=lambda x: int(x.split("_")[-1]))

    def t(a):
        return torch.tensor(np.ascontiguousarray(a), dtype=torch.float32, device=device)

    return {"xyz": t(xyz), "f_dc": t(f_dc.transpose(0, 2, 1)), "f_rest": t(f_rest.transpose(0, 2, 1)),
            "opacity": t(np.asarray(v["opacity"])[:, None]),
            "scaling": t(np.stack([v[n] for n in _sorted(v, "scale_")], 1)),
            "rotation": t(np.stack([v[n] for n in rot_names], 1)),
            "semantic": t(np.stack([v[n] for n in sem], 1)) if sem else None}
