"""ctypes mirror of include/sgr.h and the loader of libsgr.so.

The library is the only compute path: if it has not been built, importing a
rasteriser module raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "_lib" / "libsgr.so"

SGR_OK = 0
SGR_ERR_CUDA = 6
ABI_VERSION = 4
SGR_FLAG_KEY_OVERFLOW = 1
SGR_FLAG_PREFILTERED = 2
SGR_FLAG_BIN_OVERFLOW = 4
SGR_FLAG_LIST_INCONSISTENT = 8
STATUS_BYTES = 32
SGR_BLEND_STRIP16 = 0
SGR_BLEND_PATCH8 = 1
SGR_SCHEDULE_GRID = 0
SGR_SCHEDULE_QUEUE = 1
SGR_STAGE_DEFAULT = 256
SGR_STAGE_SMALL = 128
SGR_STAGE_TINY = 64
SGR_VARIANT_PLAIN = 0
SGR_VARIANT_PART = 1
SGR_MAX_SEMANTICS = 16
SGR_TILE = 16
PHASES = ("preprocess", "depth_order", "binning", "blend_fwd", "blend_bwd", "preprocess_bwd")

_p = C.c_void_p
_f = C.c_float
_i = C.c_int32


class SceneDesc(C.Structure):
    _fields_ = [("surfel_offset", _i), ("surfel_count", _i), ("view_begin", _i), ("view_count", _i)]


class ViewDesc(C.Structure):
    _fields_ = [("scene", _i), ("record_offset", _i), ("tanfovx", _f), ("tanfovy", _f)]


class Batch(C.Structure):
    _fields_ = [
        ("variant", _i), ("num_scenes", _i), ("num_views", _i), ("height", _i), ("width", _i),
        ("num_surfels", _i), ("num_records", _i), ("sh_degree", _i), ("sh_coeffs", _i),
        ("semantic_channels", _i), ("prefiltered", _i), ("scale_modifier", _f),
        ("scenes", _p), ("views", _p), ("viewmatrix", _p), ("projmatrix", _p), ("campos", _p),
        ("background", _p), ("means3D", _p), ("scales", _p), ("rotations", _p), ("opacities", _p),
        ("shs", _p), ("colors_precomp", _p), ("transmat_precomp", _p), ("semantics", _p), ("cell_tiles", _i),
        ("blend_shape", _i), ("tile_schedule", _i), ("stage_entries", _i),
    ]


class Sizes(C.Structure):
    _fields_ = [
        ("geom_bytes", C.c_size_t), ("list_bytes", C.c_size_t), ("fwd_scratch_bytes", C.c_size_t),
        ("bwd_scratch_bytes", C.c_size_t), ("tile_list_scratch_bytes", C.c_size_t), ("off_records", C.c_size_t),
        ("off_radii", C.c_size_t), ("off_tiles_touched", C.c_size_t), ("off_depth_order", C.c_size_t),
        ("off_offsets", C.c_size_t), ("off_ranges", C.c_size_t), ("off_final_T", C.c_size_t),
        ("off_n_contrib", C.c_size_t), ("off_status", C.c_size_t), ("off_rects", C.c_size_t),
        ("off_bin_start", C.c_size_t), ("off_bin_count", C.c_size_t), ("off_tile_resume", C.c_size_t),
        ("off_tile_queue", C.c_size_t),
        ("tiles_x", _i), ("tiles_y", _i), ("tile_key_bits", _i), ("cell_tiles", _i),
    ]


class FwdOutputs(C.Structure):
    _fields_ = [("color", _p), ("others", _p), ("semantic", _p), ("radii", _p)]


class BwdInputs(C.Structure):
    _fields_ = [("dL_dcolor", _p), ("dL_dothers", _p), ("dL_dsemantic", _p)]


class BwdOutputs(C.Structure):
    _fields_ = [("dL_dmeans2D", _p), ("dL_dcolors", _p), ("dL_dopacity", _p), ("dL_dmeans3D", _p),
                ("dL_dtransmat", _p), ("dL_dsh", _p), ("dL_dscales", _p), ("dL_drotations", _p),
                ("dL_dsemantics", _p)]


class BindArgs(C.Structure):
    _fields_ = [("B", _i), ("V", _i), ("F", _i), ("N", _i), ("ratio_block_scene", _f), ("scale_block_min", _f),
                ("sq_s", _p), ("sq_r", _p), ("sq_t", _p), ("sq_eps", _p), ("eta", _p), ("omega", _p),
                ("faces", _p), ("sq_occ", _p), ("alpha", _p), ("scale", _p)]


# (name, restype, argtypes) of every exported entry point
SIGNATURES = {
    "sgr_abi_version": (C.c_int, []),
    "sgr_kernel_launches": (C.c_uint64, []),
    "sgr_status_string": (C.c_char_p, [C.c_int]),
    "sgr_last_error_message": (C.c_char_p, []),
    "sgr_query_sizes": (C.c_int, [C.POINTER(Batch), C.c_int64, C.POINTER(Sizes)]),
    "sgr_forward_geometry": (C.c_int, [C.POINTER(Batch), _p, _p, C.c_size_t, _p, _p]),
    "sgr_forward_raster": (C.c_int, [C.POINTER(Batch), _p, _p, C.c_int64, _p, C.c_size_t, C.POINTER(FwdOutputs), _p]),
    "sgr_backward": (C.c_int, [C.POINTER(Batch), _p, _p, C.c_int64, _p, C.c_size_t, C.POINTER(BwdInputs),
                               C.POINTER(BwdOutputs), _p]),
    "sgr_tile_lists": (C.c_int, [C.POINTER(Batch), _p, _p, C.c_int64, _p, C.c_size_t, _p]),
    "sgr_mark_visible": (C.c_int, [_i, _p, _p, _p, _p, _p]),
    "sgr_status_accumulate": (C.c_int, [_p, _p, _p]),
    "sgr_radix_sort_temp_bytes": (C.c_size_t, [C.c_int64, C.c_int]),
    "sgr_radix_sort_pairs": (C.c_int, [_p, _p, _p, _p, C.c_int64, C.c_int, C.c_int, _p, C.c_size_t, _p]),
    "sgr_prefix_sum_temp_bytes": (C.c_size_t, [C.c_int64, C.c_int]),
    "sgr_inclusive_sum_u64": (C.c_int, [_p, _p, C.c_int64, _p, C.c_size_t, _p]),
    "sgr_exclusive_sum_u32": (C.c_int, [_p, _p, C.c_int64, _p, C.c_size_t, _p]),
    "sgr_profile_enable": (C.c_int, [C.c_int]),
    "sgr_profile_read": (C.c_int, [C.POINTER(C.c_float), C.POINTER(C.c_int32)]),
    "sgr_bind_forward": (C.c_int, [C.POINTER(BindArgs), _p, _p, _p, _p, _p]),
    "sgr_bind_scratch_bytes": (C.c_size_t, [C.POINTER(BindArgs)]),
    "sgr_bind_backward": (C.c_int, [C.POINTER(BindArgs), _p, _p, _p, _p, _p, _p, _p, _p, _p, _p, _p]),
}

_lib = None


class SgrError(RuntimeError):
    pass


def load(path: str | os.PathLike | None = None):
    """Loads libsgr.so once; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(f"{p} is missing: build the CUDA library first "
                          "(python -c 'import __graft_entry__ as g; g.build()' or python partgs_gb300/build.py)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.sgr_abi_version() != ABI_VERSION:
        raise ImportError("libsgr.so ABI version mismatch")
    _lib = lib
    return lib


def check(rc: int, what: str):
    if rc != SGR_OK:
        lib = load()
        msg = lib.sgr_status_string(rc).decode()
        if rc == SGR_ERR_CUDA:
            msg += ": " + lib.sgr_last_error_message().decode()
        raise SgrError(f"{what} failed: {msg}")
