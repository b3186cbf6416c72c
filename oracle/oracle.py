"""ctypes wrapper over the CPU oracle (oracle/_build/libnsg_oracle.so) and the
two reference libraries built from nscale's own code: ConnComponents
(oracle/_ref/libnsg_refcc.so) and the nscale morphology / pixel functions of
the segmentNuclei path compiled against an OpenCV stand-in
(oracle/_ref/libnsg_refnscale.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU legs of bench.py, to check results.  The product path never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(HERE, "_build", "libnsg_oracle.so")
_REF = os.path.join(HERE, "_ref", "libnsg_refcc.so")
_REFN = os.path.join(HERE, "_ref", "libnsg_refnscale.so")

_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")


class Params(C.Structure):
    """Field order and defaults of HistologicalEntities::segmentNuclei
    (src/segment/HistologicalEntities.h:52-54)."""

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


class Dump(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in (
        "rbc", "rc_open", "rc_recon", "diffIm", "bw1", "bw1_t", "seg_norbc", "seg_nohole",
        "seg_open", "seg_big", "dist", "distance2", "minima", "minima_labels", "watermask",
        "seg_nonoverlap", "seg", "final_mask")] + [
        ("stage_seconds", C.c_double * 24), ("bg_count", C.c_int),
        ("compcount_first", C.c_int), ("compcount_seg", C.c_int)]


DUMP_TYPES = {"dist": np.float32, "distance2": np.float32, "minima_labels": np.int32,
              "watermask": np.int32}


def nscale_src() -> str:
    """The nscale source tree: NSCALE_SRC from the environment, else the
    build recipe's default (oracle/Makefile)."""
    v = os.environ.get("NSCALE_SRC")
    if v:
        return v
    r = subprocess.run(["make", "-s", "-C", HERE, "nscale-src"], capture_output=True, text=True)
    return r.stdout.strip()


def build(ref: bool | None = None) -> None:
    """Compile the oracle (and, when the nscale sources are present, the two
    reference libraries made from nscale's own code into oracle/_ref)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    src = nscale_src()
    if ref is None:
        ref = bool(src) and os.path.isdir(os.path.join(src, "src", "segment"))
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"NSCALE_SRC={src}"], check=True)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB):
            build(ref=False)
        L = C.CDLL(_LIB)
        L.orc_get_background.restype = C.c_int64
        L.orc_get_background.argtypes = [_u8p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
        L.orc_get_rbc.argtypes = [_u8p, C.c_int, C.c_int, C.c_double, C.c_double, _u8p]
        L.orc_get_rbc_f64.argtypes = [_u8p, C.c_int, C.c_int, C.c_double, C.c_double, _u8p]
        _f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        L.orc_stain_matrix.argtypes = [_f64p, _u8p, _f64p]
        L.orc_stain_matrix.restype = C.c_int
        L.orc_color_lut.argtypes = [_f32p]
        L.orc_color_deconv.argtypes = [_u8p, C.c_int, C.c_int, _f32p, _f32p, _u8p, _u8p]
        L.orc_color_deconv_f64.argtypes = [_u8p, C.c_int, C.c_int, _f64p, _u8p, _u8p]
        L.orc_gradient_u8.argtypes = [_u8p, C.c_int, C.c_int, _u8p]
        L.orc_target_parameters.argtypes = [_u8p, C.c_int, C.c_int, _f32p, _f32p]
        L.orc_normalization.argtypes = [_u8p, C.c_int, C.c_int, _f32p, _f32p, _u8p]
        L.orc_nucleus_features.argtypes = [_i32p, _u8p, C.c_int, C.c_int, _f32p]
        L.orc_nucleus_features.restype = C.c_int
        L.orc_erode_u8.argtypes = [_u8p, C.c_int, C.c_int, _u8p, C.c_int, _u8p]
        L.orc_dilate_u8.argtypes = [_u8p, C.c_int, C.c_int, _u8p, C.c_int, _u8p]
        L.orc_morph_open_u8.argtypes = [_u8p, C.c_int, C.c_int, _u8p, C.c_int, _u8p]
        L.orc_disk19.restype = C.POINTER(C.c_uint8)
        L.orc_cross3.restype = C.POINTER(C.c_uint8)
        L.orc_imreconstruct_u8.argtypes = [_u8p, _u8p, C.c_int, C.c_int, C.c_int, _u8p]
        L.orc_imreconstruct_f32.argtypes = [_f32p, _f32p, C.c_int, C.c_int, C.c_int, _f32p]
        L.orc_imreconstruct_binary_u8.argtypes = [_u8p, _u8p, C.c_int, C.c_int, C.c_int, _u8p]
        L.orc_imfill_holes_u8.argtypes = [_u8p, C.c_int, C.c_int, C.c_int, _u8p]
        L.orc_bwselect_u8.argtypes = [_u8p, _u8p, C.c_int, C.c_int, C.c_int, _u8p]
        L.orc_cc_label.argtypes = [_u8p, C.c_int, C.c_int, _i32p, C.c_int, C.c_int]
        L.orc_cc_area_threshold_labeled.restype = C.c_int
        L.orc_cc_area_threshold_labeled.argtypes = [_i32p, C.c_int, C.c_int, _i32p, C.c_int, C.c_int, C.c_int]
        L.orc_bwlabel2.argtypes = [_u8p, C.c_int, C.c_int, C.c_int, _i32p]
        L.orc_bwareaopen2.restype = C.c_int
        L.orc_bwareaopen2.argtypes = [_u8p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _u8p]
        L.orc_dist_transform.argtypes = [_u8p, C.c_int, C.c_int, _f32p]
        L.orc_imhmin_f32.argtypes = [_f32p, C.c_int, C.c_int, C.c_float, C.c_int, _f32p]
        L.orc_local_maxima_f32.argtypes = [_f32p, C.c_int, C.c_int, C.c_int, _u8p]
        L.orc_local_minima_f32.argtypes = [_f32p, C.c_int, C.c_int, C.c_int, _u8p]
        L.orc_cv_watershed.argtypes = [_u8p, _i32p, C.c_int, C.c_int]
        L.orc_border_fix_i32.argtypes = [_i32p, C.c_int, C.c_int, C.c_int32, _i32p]
        L.orc_watershed2.argtypes = [_u8p, _f32p, C.c_int, C.c_int, C.c_int, _i32p, C.c_void_p]
        L.orc_bounding_box.restype = C.c_int
        L.orc_bounding_box.argtypes = [_i32p, C.c_int, C.c_int, C.c_void_p]
        L.orc_bounding_box_refbug.restype = C.c_int
        L.orc_bounding_box_refbug.argtypes = [_i32p, C.c_int, C.c_int, C.c_int, C.c_void_p]
        L.orc_segment_nuclei.restype = C.c_int
        L.orc_segment_nuclei.argtypes = [_u8p, C.c_int, C.c_int, C.POINTER(Params), C.c_void_p, C.c_void_p,
                                         C.POINTER(C.c_int), C.c_void_p, C.POINTER(Dump)]
        _lib = L
    return _lib


def ref_lib():
    """The reference's own ConnComponents (None when it was not built)."""
    global _ref
    if _ref is None and os.path.exists(_REF):
        R = C.CDLL(_REF)
        R.ref_cc_label.argtypes = [_u8p, C.c_int, C.c_int, _i32p, C.c_int, C.c_int]
        R.ref_cc_area_threshold_labeled.restype = C.c_int
        R.ref_cc_area_threshold_labeled.argtypes = [_i32p, C.c_int, C.c_int, _i32p, C.c_int, C.c_int, C.c_int]
        R.ref_cc_bounding_box.restype = C.c_int
        R.ref_cc_bounding_box.argtypes = [_i32p, C.c_int, C.c_int, C.c_int, C.c_void_p]
        R.ref_cc_area_threshold.restype = C.c_int
        R.ref_cc_area_threshold.argtypes = [_u8p, C.c_int, C.c_int, _i32p, C.c_int, C.c_int, C.c_int, C.c_int]
        _ref = R
    return _ref


_refn = None


def refn_lib():
    """nscale's own morphology / pixel functions (None when not built)."""
    global _refn
    if _refn is None and os.path.exists(_REFN):
        R = C.CDLL(_REFN)
        for name, args in [
            ("ref_imreconstruct_u8", [_u8p, _u8p, C.c_int, C.c_int, C.c_int, _u8p]),
            ("ref_imreconstruct_f32", [_f32p, _f32p, C.c_int, C.c_int, C.c_int, _f32p]),
            ("ref_imreconstruct_binary_u8", [_u8p, _u8p, C.c_int, C.c_int, C.c_int, _u8p]),
            ("ref_imfill_holes_u8", [_u8p, C.c_int, C.c_int, C.c_int, _u8p]),
            ("ref_bwselect_u8", [_u8p, _u8p, C.c_int, C.c_int, C.c_int, _u8p]),
            ("ref_bwlabel2", [_u8p, C.c_int, C.c_int, C.c_int, _i32p]),
            ("ref_bwareaopen2", [_u8p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _u8p, C.POINTER(C.c_int)]),
            ("ref_imhmin_f32", [_f32p, C.c_int, C.c_int, C.c_float, C.c_int, _f32p]),
            ("ref_border_i32", [_i32p, C.c_int, C.c_int, C.c_int32, _i32p]),
            ("ref_get_rbc", [_u8p, C.c_int, C.c_int, C.c_double, C.c_double, _u8p]),
            ("ref_get_background", [_u8p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _u8p]),
            ("ref_invert_u8", [_u8p, C.c_int, C.c_int, _u8p]),
            ("ref_invert_i32", [_i32p, C.c_int, C.c_int, _i32p]),
            ("ref_invert_f32", [_f32p, C.c_int, C.c_int, _f32p]),
            ("ref_local_minima_f32", [_f32p, C.c_int, C.c_int, C.c_int, _u8p]),
            ("ref_morph_open_u8", [_u8p, C.c_int, C.c_int, _u8p, C.c_int, _u8p]),
            ("ref_watershed2", [_u8p, _f32p, C.c_int, C.c_int, C.c_int, _i32p]),
            ("ref_segment_nuclei", [_u8p, C.c_int, C.c_int] + [C.c_int] * 3 + [C.c_double] * 2 + [C.c_int] * 10
             + [_i32p, _u8p, _i32p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        ]:
            f = getattr(R, name)
            f.argtypes = args
            f.restype = C.c_int
        _refn = R
    return _refn


def ref_segment_nuclei(bgr, params: "Params | None" = None):
    """nscale's own segmentNuclei (both overloads) from oracle/_ref: returns
    (status, labels, mask, bbox as 5 x n in the reference's own output, i.e.
    its boundingBox(bgval 0) call, mask-overload status)."""
    R = refn_lib()
    p = params or Params()
    bgr = _c(bgr, np.uint8)
    rows, cols = bgr.shape[:2]
    lab = np.full((rows, cols), -1, np.int32)
    mask = np.zeros((rows, cols), np.uint8)
    cap = rows * cols // 4 + 16
    box = np.zeros(5 * cap, np.int32)
    cc, mst = C.c_int(0), C.c_int(0)
    st = R.ref_segment_nuclei(bgr, rows, cols, p.blue, p.green, p.red, p.T1, p.T2, p.G1, p.minSize, p.maxSize, p.G2,
                              p.minSizePl, p.minSizeSeg, p.maxSizeSeg, p.fillHolesConnectivity, p.reconConnectivity,
                              p.watershedConnectivity, lab, mask, box, cap, C.byref(cc), C.byref(mst))
    n = cc.value if st == 0 else 0
    return st, lab, mask, box[:5 * n].reshape(n, 5).T.copy() if n else np.zeros((5, 0), np.int32), mst.value


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def se_disk19() -> np.ndarray:
    p = lib().orc_disk19()
    return np.ctypeslib.as_array(p, shape=(361,)).copy().reshape(19, 19)


def se_cross3() -> np.ndarray:
    p = lib().orc_cross3()
    return np.ctypeslib.as_array(p, shape=(9,)).copy().reshape(3, 3)


def get_background(bgr, blue=220, green=220, red=220):
    bgr = _c(bgr, np.uint8)
    out = np.empty(bgr.shape[:2], np.uint8)
    n = lib().orc_get_background(bgr, bgr.shape[0], bgr.shape[1], blue, green, red, out.ctypes.data)
    return out, int(n)


def get_rbc(bgr, T1=5.0, T2=4.0, f64=False):
    bgr = _c(bgr, np.uint8)
    out = np.empty(bgr.shape[:2], np.uint8)
    (lib().orc_get_rbc_f64 if f64 else lib().orc_get_rbc)(bgr, bgr.shape[0], bgr.shape[1], T1, T2, out)
    return out


# the feature pipeline's stains and selector (nu-features.cpp:691-692)
STAINS_M = np.array([[0.650, 0.072, 0], [0.704, 0.990, 0], [0.286, 0.105, 0]], np.float64)
STAINS_B = np.array([1, 1, 0], np.uint8)


def stain_matrix(M=STAINS_M, b=STAINS_B):
    """PixelOperations::ComputeInverseStainMatrix (PixelOperations.cpp:94-156), in double (2 x 3)."""
    q = np.empty(6, np.float64)
    kept = lib().orc_stain_matrix(_c(M, np.float64).ravel(), _c(b, np.uint8), q)
    assert kept == 2
    return q.reshape(2, 3)


def color_lut():
    lut = np.empty(256, np.float32)
    lib().orc_color_lut(lut)
    return lut


def color_deconv(bgr, Q=None, f64=False):
    """PixelOperations::ColorDeconv(BGR2RGB = true) -> (H, E) uint8; f64 = all in double."""
    bgr = _c(bgr, np.uint8)
    Qd = stain_matrix() if Q is None else np.asarray(Q, np.float64)
    H = np.empty(bgr.shape[:2], np.uint8)
    E = np.empty_like(H)
    if f64:
        lib().orc_color_deconv_f64(bgr, bgr.shape[0], bgr.shape[1], _c(Qd, np.float64).ravel(), H, E)
    else:
        lib().orc_color_deconv(bgr, bgr.shape[0], bgr.shape[1], _c(Qd.astype(np.float32), np.float32).ravel(),
                               color_lut(), H, E)
    return H, E


def target_parameters(bgr):
    """Normalization::targetParameters: (mean[3], std[3]) float32."""
    bgr = _c(bgr, np.uint8)
    m, sd = np.empty(3, np.float32), np.empty(3, np.float32)
    lib().orc_target_parameters(bgr, bgr.shape[0], bgr.shape[1], m, sd)
    return m, sd


def normalization(bgr, mean_t, std_t):
    """Normalization::normalization: the BGR tile moved to the target's lab
    statistics."""
    bgr = _c(bgr, np.uint8)
    out = np.empty_like(bgr)
    lib().orc_normalization(bgr, bgr.shape[0], bgr.shape[1], _c(mean_t, np.float32), _c(std_t, np.float32), out)
    return out


def gradient(img):
    """Operators::gradient (Operators.cpp:568-640) -> uint8."""
    img = _c(img, np.uint8)
    out = np.empty_like(img)
    lib().orc_gradient_u8(img, img.shape[0], img.shape[1], out)
    return out


def nucleus_features(labels, gray):
    """(n, 5) float32: area, perimeter, mean gray, std gray, mean gradient, per
    component in bounding-box order."""
    labels, gray = _c(labels, np.int32), _c(gray, np.uint8)
    out = np.empty((labels.size, 5), np.float32) if labels.size else np.empty((1, 5), np.float32)
    n = lib().orc_nucleus_features(labels, gray, labels.shape[0], labels.shape[1], out.reshape(-1))
    return out[:n].copy()


def erode(img, se):
    img, se = _c(img, np.uint8), _c(se, np.uint8)
    out = np.empty_like(img)
    lib().orc_erode_u8(img, img.shape[0], img.shape[1], se.ravel(), se.shape[0], out)
    return out


def dilate(img, se):
    img, se = _c(img, np.uint8), _c(se, np.uint8)
    out = np.empty_like(img)
    lib().orc_dilate_u8(img, img.shape[0], img.shape[1], se.ravel(), se.shape[0], out)
    return out


def morph_open(img, se):
    img, se = _c(img, np.uint8), _c(se, np.uint8)
    out = np.empty_like(img)
    lib().orc_morph_open_u8(img, img.shape[0], img.shape[1], se.ravel(), se.shape[0], out)
    return out


def imreconstruct(marker, mask, conn=8):
    if mask.dtype == np.float32:
        marker, mask = _c(marker, np.float32), _c(mask, np.float32)
        out = np.empty_like(mask)
        lib().orc_imreconstruct_f32(marker, mask, mask.shape[0], mask.shape[1], conn, out)
    else:
        marker, mask = _c(marker, np.uint8), _c(mask, np.uint8)
        out = np.empty_like(mask)
        lib().orc_imreconstruct_u8(marker, mask, mask.shape[0], mask.shape[1], conn, out)
    return out


def imreconstruct_binary(marker, mask, conn=8):
    marker, mask = _c(marker, np.uint8), _c(mask, np.uint8)
    out = np.empty_like(mask)
    lib().orc_imreconstruct_binary_u8(marker, mask, mask.shape[0], mask.shape[1], conn, out)
    return out


def imfill_holes(img, conn=4):
    img = _c(img, np.uint8)
    out = np.empty_like(img)
    lib().orc_imfill_holes_u8(img, img.shape[0], img.shape[1], conn, out)
    return out


def bwselect(bw, seeds, conn=8):
    bw, seeds = _c(bw, np.uint8), _c(seeds, np.uint8)
    out = np.empty_like(bw)
    lib().orc_bwselect_u8(bw, seeds, bw.shape[0], bw.shape[1], conn, out)
    return out


def bwlabel2(img, conn=8):
    img = _c(img, np.uint8)
    out = np.empty(img.shape, np.int32)
    lib().orc_bwlabel2(img, img.shape[0], img.shape[1], conn, out)
    return out


def cc_label(img, conn=8, bgval=-1):
    img = _c(img, np.uint8)
    out = np.empty(img.shape, np.int32)
    lib().orc_cc_label(img, img.shape[1], img.shape[0], out, bgval, conn)
    return out


def area_threshold_labeled(label, lower, upper, bgval=-1):
    label = _c(label, np.int32)
    out = np.empty_like(label)
    n = lib().orc_cc_area_threshold_labeled(label, label.shape[1], label.shape[0], out, bgval, lower, upper)
    return out, n


def bwareaopen2(img, min_size, max_size, conn=8):
    img = _c(img, np.uint8)
    out = np.empty_like(img)
    n = lib().orc_bwareaopen2(img, img.shape[0], img.shape[1], min_size, max_size, conn, out)
    return out, n


def dist_transform(mask):
    mask = _c(mask, np.uint8)
    out = np.empty(mask.shape, np.float32)
    lib().orc_dist_transform(mask, mask.shape[0], mask.shape[1], out)
    return out


def imhmin(img, h=1.0, conn=8):
    img = _c(img, np.float32)
    out = np.empty_like(img)
    lib().orc_imhmin_f32(img, img.shape[0], img.shape[1], h, conn, out)
    return out


def local_maxima(img, conn=8):
    img = _c(img, np.float32)
    out = np.empty(img.shape, np.uint8)
    lib().orc_local_maxima_f32(img, img.shape[0], img.shape[1], conn, out)
    return out


def local_minima(img, conn=8):
    img = _c(img, np.float32)
    out = np.empty(img.shape, np.uint8)
    lib().orc_local_minima_f32(img, img.shape[0], img.shape[1], conn, out)
    return out


def cv_watershed(bgr, markers):
    """OpenCV-style watershed on full-size arrays (the caller pads)."""
    bgr = _c(bgr, np.uint8)
    m = _c(markers, np.int32).copy()
    lib().orc_cv_watershed(bgr, m, m.shape[0], m.shape[1])
    return m


def border_fix(img, bg=-1):
    img = _c(img, np.int32)
    out = np.empty_like(img)
    lib().orc_border_fix_i32(img, img.shape[0], img.shape[1], bg, out)
    return out


def watershed2(bgr, img, conn=8, return_labels=False):
    bgr, img = _c(bgr, np.uint8), _c(img, np.float32)
    out = np.empty(img.shape, np.int32)
    labels = np.empty(img.shape, np.int32) if return_labels else None
    lib().orc_watershed2(bgr, img, img.shape[0], img.shape[1], conn, out,
                         labels.ctypes.data if return_labels else None)
    return (out, labels) if return_labels else out


def bounding_box(labels):
    labels = _c(labels, np.int32)
    buf = np.empty(5 * labels.size + 5, np.int32)
    n = lib().orc_bounding_box(labels, labels.shape[1], labels.shape[0], buf.ctypes.data)
    return buf[:5 * n].reshape(5, n)


def bounding_box_refbug(labels, bgval=0):
    labels = _c(labels, np.int32)
    buf = np.empty(5 * labels.size + 5, np.int32)
    n = lib().orc_bounding_box_refbug(labels, labels.shape[1], labels.shape[0], bgval, buf.ctypes.data)
    return buf[:5 * n].reshape(5, n)


def segment_nuclei(bgr, params: Params | None = None, dump_stages=()):
    """Full pipeline.  Returns (status, labels int32, mask u8, bbox (5, n), dump dict)."""
    bgr = _c(bgr, np.uint8)
    rows, cols = bgr.shape[:2]
    labels = np.full((rows, cols), -1, np.int32)
    mask = np.zeros((rows, cols), np.uint8)
    bbox = np.empty(5 * rows * cols + 5, np.int32)
    cc = C.c_int(0)
    d = Dump()
    keep = {}
    for name in dump_stages:
        if name in ("stage_seconds",):
            continue
        a = np.zeros((rows, cols), DUMP_TYPES.get(name, np.uint8))
        keep[name] = a
        setattr(d, name, a.ctypes.data)
    p = params if params is not None else Params()
    st = lib().orc_segment_nuclei(bgr, rows, cols, C.byref(p), labels.ctypes.data, mask.ctypes.data,
                                  C.byref(cc), bbox.ctypes.data, C.byref(d))
    n = cc.value
    keep["stage_seconds"] = list(d.stage_seconds)
    keep["bg_count"] = d.bg_count
    keep["compcount_first"] = d.compcount_first
    keep["compcount_seg"] = d.compcount_seg
    return st, labels, mask, bbox[:5 * n].reshape(5, n), keep
