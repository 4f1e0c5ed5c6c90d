"""The C ABI library loads and exports every entry point include/sgr.h
declares; argument checks that need no GPU return the documented codes."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if not fn.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(sgr_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


def test_header_declares_the_entry_points():
    names = declared_functions()
    for n in ["sgr_forward_geometry", "sgr_forward_raster", "sgr_backward", "sgr_mark_visible",
              "sgr_bind_forward", "sgr_bind_backward", "sgr_query_sizes"]:
        assert n in names


def test_library_exports_every_declared_symbol(sgr_lib):
    missing = [n for n in declared_functions() if not hasattr(sgr_lib, n)]
    assert not missing, missing


def test_status_strings_and_version(sgr_lib):
    from partgs_gb300 import _lib as L
    assert sgr_lib.sgr_abi_version() == L.ABI_VERSION
    assert sgr_lib.sgr_status_string(0) == b"ok"
    assert b"16" in sgr_lib.sgr_status_string(3)


def test_invalid_arguments_rejected_without_touching_the_gpu(sgr_lib):
    from partgs_gb300 import _lib as L
    sizes = L.Sizes()
    assert sgr_lib.sgr_query_sizes(None, 0, C.byref(sizes)) == 1
    b = L.Batch()
    b.variant = 1
    b.num_scenes = b.num_views = b.height = b.width = 1
    b.semantic_channels = 17
    assert sgr_lib.sgr_query_sizes(C.byref(b), 0, C.byref(sizes)) == 3      # S > 16
    b.semantic_channels = 0
    b.variant = 7
    assert sgr_lib.sgr_query_sizes(C.byref(b), 0, C.byref(sizes)) == 1      # unknown variant
    b.variant = 0
    b.scenes = b.views = b.viewmatrix = b.projmatrix = b.campos = b.background = 16
    assert sgr_lib.sgr_query_sizes(C.byref(b), -1, C.byref(sizes)) == 5     # negative capacity
    b.num_surfels = 10
    b.means3D = b.opacities = 16
    assert sgr_lib.sgr_query_sizes(C.byref(b), 0, C.byref(sizes)) == 1      # neither SH nor colours
    b.shs = 16
    b.sh_coeffs = 25
    b.scales = b.rotations = 16
    assert sgr_lib.sgr_query_sizes(C.byref(b), 0, C.byref(sizes)) == 2      # more than 16 SH coefficients
    b.sh_coeffs = 16
    for stage, rc in ((32, 1), (512, 1), (L.SGR_STAGE_TINY, 0), (L.SGR_STAGE_SMALL, 0), (L.SGR_STAGE_DEFAULT, 0),
                      (0, 0)):
        b.stage_entries = stage                                             # staged batch: 0, 256, 128 or 64
        assert sgr_lib.sgr_query_sizes(C.byref(b), 0, C.byref(sizes)) == rc, stage
    assert sgr_lib.sgr_mark_visible(-1, None, None, None, None, None) == 1
    assert sgr_lib.sgr_mark_visible(0, None, None, None, None, None) == 0


def test_loader_fails_loudly_without_the_library(tmp_path):
    from partgs_gb300 import _lib as L
    saved = L._lib
    try:
        L._lib = None
        with pytest.raises(ImportError):
            L.load(tmp_path / "libsgr.so")
    finally:
        L._lib = saved
