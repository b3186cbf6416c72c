"""ctypes binding of libnsg.so (the C ABI declared in include/nsg.h).

The library is built in-tree by nscale_gb300/build.py.  Loading fails loudly
when it is missing: there is no CPU fallback anywhere in this package.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnsg.so")

STATUS = {0: "SUCCESS", 1: "BACKGROUND", 2: "BACKGROUND_LIKELY", 3: "NO_CANDIDATES_LEFT", 4: "CONTINUE",
          -1: "INVALID_IMAGE", -2: "RUNTIME_FAILED", -10: "ERR_ARG", -11: "ERR_OOM", -12: "ERR_TIMEOUT",
          -13: "ERR_QUEUE_FULL", -14: "ERR_CUDA", -15: "ERR_UNSUPPORTED"}

SUCCESS, BACKGROUND, BACKGROUND_LIKELY, NO_CANDIDATES_LEFT = 0, 1, 2, 3
INVALID_IMAGE, RUNTIME_FAILED = -1, -2
ERR_ARG, ERR_OOM, ERR_TIMEOUT, ERR_QUEUE_FULL, ERR_CUDA = -10, -11, -12, -13, -14


class NsgError(RuntimeError):
    def __init__(self, code: int, msg: str = ""):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class SegParams(C.Structure):
    """nsg_seg_params: field order and defaults of
    HistologicalEntities::segmentNuclei (HistologicalEntities.h:52-54)."""

    _fields_ = [("blue", C.c_int), ("green", C.c_int), ("red", C.c_int),
                ("T1", C.c_double), ("T2", C.c_double), ("G1", C.c_int),
                ("minSize", C.c_int), ("maxSize", C.c_int), ("G2", C.c_int),
                ("minSizePl", C.c_int), ("minSizeSeg", C.c_int), ("maxSizeSeg", C.c_int),
                ("fillHolesConnectivity", C.c_int), ("reconConnectivity", C.c_int),
                ("watershedConnectivity", C.c_int)]

    def __init__(self, **kw):
        super().__init__(220, 220, 220, 5.0, 4.0, 80, 11, 1000, 45, 30, 21, 1000, 4, 8, 8)
        for k, v in kw.items():
            setattr(self, k, v)


class Tuning(C.Structure):
    """nsg_tuning: launch shapes (results do not depend on them)."""

    _fields_ = [("recon_max_ctas", C.c_int), ("bfs_max_cluster", C.c_int), ("recon_wl_phases", C.c_int)]


class Tile(C.Structure):
    """nsg_tile: one tile of a batch or server submission (include/nsg.h)."""

    _fields_ = [("bgr", C.c_void_p), ("rows", C.c_int), ("cols", C.c_int), ("row_stride_bytes", C.c_size_t),
                ("labels", C.c_void_p), ("mask", C.c_void_p), ("want_bbox", C.c_int), ("want_features", C.c_int),
                ("status", C.c_int), ("compcount", C.c_int), ("bbox", C.POINTER(C.c_int32)),
                ("features", C.POINTER(C.c_float))]


class Result(C.Structure):
    """nsg_result: one finished server tile."""

    _fields_ = [("ticket", C.c_longlong), ("status", C.c_int), ("compcount", C.c_int),
                ("bbox", C.POINTER(C.c_int32)), ("features", C.POINTER(C.c_float)), ("latency_ms", C.c_double)]


TILE_HOST = 1

_P = C.c_void_p
_I = C.c_int
_SIGS = {
    "nsg_version": (_I, []),
    "nsg_default_params": (None, [C.POINTER(SegParams)]),
    "nsg_status_string": (C.c_char_p, [_I]),
    "nsg_context_create": (_I, [C.POINTER(_P), _I, _I, _I]),
    "nsg_context_destroy": (_I, [_P]),
    "nsg_context_last_error": (C.c_char_p, [_P]),
    "nsg_context_bytes": (C.c_size_t, [_P]),
    "nsg_context_set_spin_budget": (_I, [_P, C.c_longlong]),
    "nsg_get_background": (_I, [_P, _P, _I, _I, _I, _I, _I, _P, C.POINTER(C.c_int64), _P]),
    "nsg_get_rbc": (_I, [_P, _P, _I, _I, C.c_double, C.c_double, _P, _P]),
    "nsg_invert_u8": (_I, [_P, _P, _P, C.c_int64, _P]),
    "nsg_invert_i32": (_I, [_P, _P, _P, C.c_int64, _P]),
    "nsg_invert_f32": (_I, [_P, _P, _P, C.c_int64, _P]),
    "nsg_morph_erode_u8": (_I, [_P, _P, _P, _I, _I, _P, _I, _P]),
    "nsg_morph_dilate_u8": (_I, [_P, _P, _P, _I, _I, _P, _I, _P]),
    "nsg_morph_open_u8": (_I, [_P, _P, _P, _I, _I, _P, _I, _P]),
    "nsg_imreconstruct_u8": (_I, [_P, _P, _P, _P, _I, _I, _I, _P]),
    "nsg_imreconstruct_f32": (_I, [_P, _P, _P, _P, _I, _I, _I, _P]),
    "nsg_imreconstruct_binary_u8": (_I, [_P, _P, _P, _P, _I, _I, _I, _P]),
    "nsg_imfill_holes_u8": (_I, [_P, _P, _P, _I, _I, _I, _P]),
    "nsg_imfill_holes_u8_noalloc": (_I, [_P, _P, _I, _I, _I, _P]),
    "nsg_stain_matrix": (_I, [_P, _P, C.POINTER(C.c_float)]),
    "nsg_color_deconv": (_I, [_P, _P, _I, _I, C.c_size_t, C.POINTER(C.c_float), _P, _P, _P]),
    "nsg_gradient_u8": (_I, [_P, _P, _P, _I, _I, _P]),
    "nsg_color_target_parameters": (_I, [_P, _P, _I, _I, C.c_size_t, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                         _P]),
    "nsg_color_normalization": (_I, [_P, _P, _I, _I, C.c_size_t, C.POINTER(C.c_float), C.POINTER(C.c_float), _P,
                                     _P]),
    "nsg_nucleus_features": (_I, [_P, _P, _P, _I, _I, _P, _I, C.POINTER(_I), _P]),
    "nsg_pool_create": (_I, [C.POINTER(_P), _I, _I, _I, _I]),
    "nsg_pool_destroy": (_I, [_P]),
    "nsg_pool_workers": (_I, [_P]),
    "nsg_pool_set_tuning": (_I, [_P, C.POINTER(Tuning)]),
    "nsg_context_set_tuning": (_I, [_P, C.POINTER(Tuning)]),
    "nsg_pool_context_bytes": (C.c_size_t, [_I, _I]),
    "nsg_segment_nuclei_batch": (_I, [_P, C.POINTER(Tile), _I, C.POINTER(SegParams), _I]),
    "nsg_server_create": (_I, [C.POINTER(_P), _I, _I, C.c_size_t, _I, _I]),
    "nsg_server_workers": (_I, [_P]),
    "nsg_server_create_classes": (_I, [C.POINTER(_P), C.POINTER(_I), C.POINTER(_I), C.POINTER(C.c_double), _I,
                                       C.c_size_t, _I, _I]),
    "nsg_server_class_workers": (_I, [_P, _I, _I]),
    "nsg_server_submit": (_I, [_P, C.POINTER(Tile), C.POINTER(SegParams), C.POINTER(C.c_longlong)]),
    "nsg_server_poll": (_I, [_P, C.POINTER(Result), _I, _I]),
    "nsg_server_destroy": (_I, [_P]),
    "nsg_bwselect_u8": (_I, [_P, _P, _P, _P, _I, _I, _I, _P]),
    "nsg_bwlabel": (_I, [_P, _P, _P, _I, _I, _I, _P]),
    "nsg_bwareaopen": (_I, [_P, _P, _P, _I, _I, _I, _I, _I, C.POINTER(_I), _P]),
    "nsg_dist_transform": (_I, [_P, _P, _P, _I, _I, _P]),
    "nsg_imhmin_f32": (_I, [_P, _P, _P, _I, _I, C.c_float, _I, _P]),
    "nsg_local_maxima_f32": (_I, [_P, _P, _P, _I, _I, _I, _P]),
    "nsg_local_minima_f32": (_I, [_P, _P, _P, _I, _I, _I, _P]),
    "nsg_watershed": (_I, [_P, _P, _P, _P, _I, _I, _I, _P]),
    "nsg_watershed_serial": (_I, [_P, _P, _P, _P, _I, _I, _I, _P]),
    "nsg_watershed_diagnostics": (_I, [_P, _P, _P]),
    "nsg_bounding_box": (_I, [_P, _P, _I, _I, _P, _I, C.POINTER(_I), _P]),
    "nsg_segment_nuclei": (_I, [_P, _P, _I, _I, C.c_size_t, C.POINTER(SegParams), _P, _P, C.POINTER(_I),
                                C.POINTER(C.POINTER(C.c_int32)), _P]),
    "nsg_segment_nuclei_host": (_I, [_P, _P, _I, _I, C.POINTER(SegParams), _P, _P, C.POINTER(_I),
                                     C.POINTER(C.POINTER(C.c_int32)), _P]),
    "nsg_context_set_timing": (_I, [_P, _I]),
    "nsg_context_stage_times": (_I, [_P, C.POINTER(C.c_double), _I, C.POINTER(C.c_longlong)]),
    "nsg_pool_set_timing": (_I, [_P, _I]),
    "nsg_pool_stage_times": (_I, [_P, C.POINTER(C.c_double), _I, C.POINTER(C.c_longlong)]),
    "nsg_stage_name": (C.c_char_p, [_I]),
    "nsg_kernel_launches": (C.c_longlong, []),
    "nsg_alloc": (_P, [C.c_size_t]),
    "nsg_free": (None, [_P]),
}

_lib = None


def exported_symbols() -> list[str]:
    return list(_SIGS)


def load(path: str = LIB_PATH):
    """Load libnsg.so and bind every ABI function (raises if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError(
            f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(nscale_gb300 has no CPU fallback)")
    L = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L
