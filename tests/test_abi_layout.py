"""The Python side's ctypes images of the C ABI agree with include/sgr.h as a
C compiler reads it.  For every struct: its size, and each field's name,
order, offset and size (gcc prints them with sizeof/offsetof from the
header itself).  For every entry point the Python side binds: the number of
parameters and the return type the header declares.  No GPU is used."""
import ctypes as C
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "sgr.h")


def _source():
    src = re.sub(r"/\*.*?\*/", " ", open(HEADER).read(), flags=re.S)
    return "\n".join(line for line in src.splitlines() if not line.lstrip().startswith("#"))


def _structs():
    """{typedef name: [field names in declaration order]}."""
    out = {}
    for m in re.finditer(r"typedef\s+struct\s+\w+\s*\{(.*?)\}\s*(\w+)\s*;", _source(), flags=re.S):
        names = []
        for decl in m.group(1).split(";"):
            for part in filter(None, (p.strip() for p in decl.split(","))):
                names.append(re.search(r"([A-Za-z_]\w*)\s*(\[[^\]]*\])?$", part).group(1))
        out[m.group(2)] = names
    return out


def _prototypes():
    """{entry point: (return type, parameter count)}."""
    src = _source().replace('extern "C" {', " ")
    out = {}
    for stmt in src.split(";"):
        if "struct" in stmt or "{" in stmt or "}" in stmt:
            continue
        m = re.match(r"\s*(.*?)\b(sgr_\w+)\s*\((.*)\)\s*$", stmt, flags=re.S)
        if not m:
            continue
        args = " ".join(m.group(3).split())
        out[m.group(2)] = (" ".join(m.group(1).split()), 0 if args in ("", "void") else args.count(",") + 1)
    return out


def _mirrors():
    from partgs_gb300 import _lib as L
    from partgs_gb300 import activations, losses, optim, proposal_gemm, sq_losses
    return {"sgr_scene_desc": L.SceneDesc, "sgr_view_desc": L.ViewDesc, "sgr_batch": L.Batch,
            "sgr_sizes": L.Sizes, "sgr_fwd_outputs": L.FwdOutputs, "sgr_bwd_inputs": L.BwdInputs,
            "sgr_bwd_outputs": L.BwdOutputs, "sgr_bind_args": L.BindArgs, "sgr_loss_args": losses.LossArgs,
            "sgr_adam_tensor": optim.AdamTensor, "sgr_adam_args": optim.AdamArgs,
            "sgr_activate_args": activations.ActivateArgs, "sgr_sq_loss_args": sq_losses.SQLossArgs,
            "sgr_gemm_args": proposal_gemm.GemmArgs}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    """{struct: (sizeof, {field: (offset, size)})} as gcc lays out the header."""
    gcc = shutil.which("gcc") or shutil.which("cc")
    if gcc is None:
        pytest.skip("no C compiler on this host")
    structs = _structs()
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "sgr.h"', "int main(void) {"]
    for s, fields in structs.items():
        lines.append(f'  printf("S {s} %zu\\n", sizeof({s}));')
        for f in fields:
            lines.append(f'  printf("F {s} {f} %zu %zu\\n", offsetof({s}, {f}), sizeof((({s}*)0)->{f}));')
    lines += ["  return 0;", "}"]
    d = tmp_path_factory.mktemp("abi_layout")
    (d / "layout.c").write_text("\n".join(lines) + "\n")
    subprocess.run([gcc, "-std=c11", "-I", os.path.dirname(HEADER), str(d / "layout.c"), "-o", str(d / "layout")],
                   check=True, capture_output=True)
    out = {}
    for line in subprocess.run([str(d / "layout")], check=True, capture_output=True, text=True).stdout.splitlines():
        kind, s, *rest = line.split()
        if kind == "S":
            out.setdefault(s, [0, {}])[0] = int(rest[0])
        else:
            out.setdefault(s, [0, {}])[1][rest[0]] = (int(rest[1]), int(rest[2]))
    return out


def test_every_header_struct_has_a_mirror():
    assert set(_structs()) == set(_mirrors())


def test_struct_layouts_match_the_header(c_layout):
    bad = []
    for s, cls in _mirrors().items():
        size, fields = c_layout[s]
        names = [f[0] for f in cls._fields_]
        if names != _structs()[s]:
            bad.append((s, "fields", names, _structs()[s]))
            continue
        if C.sizeof(cls) != size:
            bad.append((s, "sizeof", C.sizeof(cls), size))
        for n in names:
            d = getattr(cls, n)
            if (d.offset, d.size) != fields[n]:
                bad.append((s, n, (d.offset, d.size), fields[n]))
    assert not bad, bad


_RESTYPES = {"int": C.c_int, "size_t": C.c_size_t, "const char*": C.c_char_p, "uint64_t": C.c_uint64}


def test_bound_entry_points_match_their_prototypes(sgr_lib):
    """Every entry point a Python module binds has the header's parameter
    count and return type."""
    from partgs_gb300 import activations, chamfer_eval, densify, losses, optim, proposal, proposal_gemm, sq_losses
    lib = sgr_lib
    for bind in (activations._lib, chamfer_eval._lib, densify._lib, losses._lib, optim._lib, proposal._pool_lib,
                 proposal_gemm._lib, sq_losses._lib):
        assert bind() is lib
    protos = _prototypes()
    checked, bad = 0, []
    for name, (ret, nargs) in protos.items():
        fn = getattr(lib, name)
        if fn.argtypes is None:
            continue
        checked += 1
        if len(fn.argtypes) != nargs:
            bad.append((name, "arity", len(fn.argtypes), nargs))
        want = _RESTYPES.get(ret)
        if want is None or fn.restype is not want:
            bad.append((name, "restype", fn.restype, ret))
    assert not bad, bad
    assert checked >= 30, checked
