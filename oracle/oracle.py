"""ctypes wrapper of the CPU oracle (oracle/hough_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg as the checker.  Nothing in opencuda_gb300/
imports it.
"""
from __future__ import annotations

import ctypes as C
import math
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libhough_oracle.so"
REF_RUNNER = HERE / "_build" / "libref_runner.so"
REF_FATBIN = HERE / "_ref" / "houghline_ref.fatbin"
REF_CIRCLE_FATBIN = HERE / "_ref" / "houghcircle_ref.fatbin"

RANK_CANONICAL = 0
RANK_REF_SHELL = 1


class ho_line(C.Structure):
    _fields_ = [("angle", C.c_float), ("distance", C.c_int), ("votes", C.c_int)]


class ho_geom(C.Structure):
    _fields_ = [("T", C.c_int), ("rho_min", C.c_int), ("R", C.c_int),
                ("ref_numrho", C.c_int), ("detheta", C.c_double),
                ("thresdis", C.c_int), ("thresang", C.c_float)]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            from opencuda_gb300 import build
            build.build_oracle()
        L = C.CDLL(str(LIB))
        P = C.c_void_p
        L.ho_numtheta.argtypes = [C.c_double]
        L.ho_numtheta.restype = C.c_int
        L.ho_ref_numrho.argtypes = [C.c_int, C.c_int, C.c_double]
        L.ho_ref_numrho.restype = C.c_int
        L.ho_layout.argtypes = [C.c_int, C.c_int, C.c_double, P, P]
        L.ho_trig_libm.argtypes = [C.c_int, C.c_double, P, P]
        L.ho_vote_image.argtypes = [P, C.c_long, C.c_int, C.c_int, P, P, C.c_int,
                                    C.c_double, C.c_int, C.c_int, P, C.c_int]
        L.ho_vote_image.restype = C.c_longlong
        L.ho_vote_points.argtypes = [P, C.c_long, P, P, C.c_int, C.c_double,
                                     C.c_int, C.c_int, P, C.c_int]
        L.ho_vote_points.restype = C.c_longlong
        L.ho_peaks.argtypes = [P, C.c_int, C.c_int, C.c_int, P, C.c_long]
        L.ho_peaks.restype = C.c_long
        L.ho_rank_merge.argtypes = [P, C.POINTER(ho_geom), P, C.c_long, C.c_int,
                                    C.POINTER(C.c_int), P]
        L.ho_rank_merge.restype = C.c_int
        L.ho_decode_ref.argtypes = [C.POINTER(ho_geom), C.c_int, P, P, P, P]
        L.ho_to_ref_layout.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int, P]
        L.ho_draw_lines.argtypes = [P, C.c_long, C.c_int, C.c_int, P, P, P, C.c_int]
        L.ho_fnv1a.argtypes = [P, C.c_size_t]
        L.ho_fnv1a.restype = C.c_uint64
        L.ho_max_threads.restype = C.c_int
        L.ho_real_line.argtypes = [P, C.c_long, C.c_int, C.c_int, C.c_int, C.c_int,
                                   C.c_int, C.c_int, C.c_float, C.c_float, P]
        L.ho_real_line.restype = C.c_int
        L.hc_vote.argtypes = [P, C.c_long, C.c_int, C.c_int, C.c_int, C.c_int, P]
        L.hc_vote.restype = C.c_longlong
        L.hc_peaks.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int, P, C.c_long]
        L.hc_peaks.restype = C.c_long
        L.hc_circles.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                 C.c_float, C.c_int, C.POINTER(C.c_int), P]
        L.hc_circles.restype = C.c_long
        _lib = L
    return _lib


def _p(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def numtheta(detheta: float) -> int:
    return lib().ho_numtheta(detheta)


def ref_numrho(w: int, h: int, derho: float = 1.0) -> int:
    return lib().ho_ref_numrho(w, h, derho)


def layout(w: int, h: int, derho: float = 1.0) -> tuple[int, int]:
    a, b = C.c_int(), C.c_int()
    lib().ho_layout(w, h, derho, C.byref(a), C.byref(b))
    return a.value, b.value


def trig_libm(T: int, detheta: float) -> tuple[np.ndarray, np.ndarray]:
    c = np.zeros(T, np.float32)
    s = np.zeros(T, np.float32)
    lib().ho_trig_libm(T, detheta, _p(c), _p(s))
    return c, s


def vote_image(roi: np.ndarray, cosv, sinv, derho: float = 1.0,
               layout_wh: tuple[int, int] | None = None, nthreads: int = 0):
    """roi: 2-D uint8 array (the ROI itself).  Returns (acc[R, T], rho_min,
    dropped)."""
    roi = np.ascontiguousarray(roi, dtype=np.uint8)
    h, w = roi.shape
    T = len(cosv)
    lw, lh = layout_wh if layout_wh else (w, h)
    rho_min, R = layout(lw, lh, derho)
    acc = np.zeros((R, T), np.int32)
    cosv = np.ascontiguousarray(cosv, np.float32)
    sinv = np.ascontiguousarray(sinv, np.float32)
    d = lib().ho_vote_image(_p(roi), w, w, h, _p(cosv), _p(sinv), T, derho,
                            rho_min, R, _p(acc), nthreads)
    return acc, rho_min, d


def vote_points(xy: np.ndarray, cosv, sinv, rho_min: int, R: int,
                derho: float = 1.0, nthreads: int = 0):
    xy = np.ascontiguousarray(xy, np.int32).reshape(-1, 2)
    T = len(cosv)
    acc = np.zeros((R, T), np.int32)
    cosv = np.ascontiguousarray(cosv, np.float32)
    sinv = np.ascontiguousarray(sinv, np.float32)
    d = lib().ho_vote_points(_p(xy), len(xy), _p(cosv), _p(sinv), T, derho,
                             rho_min, R, _p(acc), nthreads)
    return acc, d


def peaks(acc: np.ndarray, threshold: int) -> np.ndarray:
    acc = np.ascontiguousarray(acc, np.int32)
    R, T = acc.shape
    cap = R * ((T + 1) // 2) + 2
    out = np.zeros(cap, np.int32)
    n = lib().ho_peaks(_p(acc), R, T, threshold, _p(out), cap)
    return out[:min(n, cap)].copy()


def geom(T: int, rho_min: int, R: int, ref_nrho: int, detheta: float,
         thresdis: int, thresang: float) -> ho_geom:
    return ho_geom(T, rho_min, R, ref_nrho, detheta, thresdis, thresang)


def rank_merge(acc: np.ndarray, g: ho_geom, idx: np.ndarray, linesmax: int,
               mode: int = RANK_CANONICAL):
    """Returns (lines as list of (angle, distance, votes), linenum)."""
    acc = np.ascontiguousarray(acc, np.int32)
    idx = np.ascontiguousarray(idx, np.int32)
    lm = C.c_int(linesmax)
    out = (ho_line * max(linesmax, 1))()
    linenum = lib().ho_rank_merge(_p(acc), C.byref(g), _p(idx), len(idx), mode,
                                  C.byref(lm), out)
    return [(out[i].angle, out[i].distance, out[i].votes)
            for i in range(max(lm.value, 0))], linenum, lm.value


def decode_ref(g: ho_geom, ref_idx: int):
    row, k, a, d = C.c_int(), C.c_int(), C.c_float(), C.c_int()
    lib().ho_decode_ref(C.byref(g), ref_idx, C.byref(row), C.byref(k),
                        C.byref(a), C.byref(d))
    return row.value, k.value, a.value, d.value


def to_ref_layout(acc: np.ndarray, rho_min: int, ref_nrho: int) -> np.ndarray:
    acc = np.ascontiguousarray(acc, np.int32)
    R, T = acc.shape
    ref = np.zeros((ref_nrho + 2, T + 2), np.int32)
    lib().ho_to_ref_layout(_p(acc), R, T, rho_min, ref_nrho, _p(ref))
    return ref


def fnv1a(a: np.ndarray) -> int:
    a = np.ascontiguousarray(a)
    return int(lib().ho_fnv1a(_p(a), a.nbytes))


def draw_lines(w: int, h: int, cosl, sinl, dist) -> np.ndarray:
    out = np.zeros((h, w), np.uint8)
    cosl = np.ascontiguousarray(cosl, np.float32)
    sinl = np.ascontiguousarray(sinl, np.float32)
    dist = np.ascontiguousarray(dist, np.int32)
    lib().ho_draw_lines(_p(out), w, w, h, _p(cosl), _p(sinl), _p(dist), len(dist))
    return out


def houghline(roi: np.ndarray, cosv, sinv, detheta: float, derho: float,
              threshold: int, thresang: float, thresdis: int, linesmax: int,
              mode: int = RANK_CANONICAL, nthreads: int = 0):
    """Whole plain path on an ROI; returns (lines, linenum, nlines)."""
    roi = np.ascontiguousarray(roi, np.uint8)
    h, w = roi.shape
    acc, rho_min, _ = vote_image(roi, cosv, sinv, derho, nthreads=nthreads)
    R, T = acc.shape
    pk = peaks(acc, threshold)
    g = geom(T, rho_min, R, ref_numrho(w, h, derho), detheta, thresdis,
             np.float32(thresang))
    return rank_merge(acc, g, pk, linesmax, mode)


def real_line(roi: np.ndarray, x1, y1, x2, y2, threshold: float, thresperc: float):
    """(count, is_real) of realLine's rule on an ROI."""
    roi = np.ascontiguousarray(roi, np.uint8)
    h, w = roi.shape
    flag = C.c_int()
    n = lib().ho_real_line(_p(roi), w, w, h, x1, y1, x2, y2, threshold, thresperc,
                           C.byref(flag))
    return n, bool(flag.value)


def max_threads() -> int:
    return lib().ho_max_threads()


def default_thresang() -> float:
    """okano_3_0/HoughLine.h:123  thresang = M_PI/180*5.0f (float member)."""
    return float(np.float32(math.pi / 180 * 5.0))


# ---- HoughCircle (oracle/circle_oracle.c) -------------------------------

def circle_vote(roi: np.ndarray, rmin: int, rmax: int) -> np.ndarray:
    """acc[z, y, x] of okano_3_0/HoughCircle.cu:187-245 for radii rmin..rmax
    over the ROI array roi (uint8, 255 = edge)."""
    roi = np.ascontiguousarray(roi, dtype=np.uint8)
    h, w = roi.shape
    acc = np.zeros((rmax - rmin + 1, h, w), np.int32)
    lib().hc_vote(_p(roi), w, w, h, rmin, rmax, _p(acc))
    return acc


def circle_peaks(acc: np.ndarray, threshold: int) -> np.ndarray:
    nr, h, w = acc.shape
    acc = np.ascontiguousarray(acc, dtype=np.int32)
    n = lib().hc_peaks(_p(acc), nr, w, h, threshold, None, 0)
    idx = np.zeros(max(n, 1), np.int64)
    lib().hc_peaks(_p(acc), nr, w, h, threshold, _p(idx), n)
    return idx[:n]


def houghcircle(roi: np.ndarray, rmin: int, rmax: int, threshold: int, dist_thres: float,
                r_thres: int, circlemax: int):
    """The image path of HoughCircle::houghcircle (okano_3_0/HoughCircle.cu:
    1165-1214) on an ROI array: [(a, b, radius, votes)] in ROI-local
    coordinates, and the candidate count."""
    acc = circle_vote(roi, rmin, rmax)
    nr, h, w = acc.shape
    out = np.zeros((max(circlemax, 1), 4), np.int32)
    cm = C.c_int(circlemax)
    n = lib().hc_circles(_p(acc), nr, w, h, rmin, threshold, C.c_float(dist_thres),
                         r_thres, C.byref(cm), _p(out))
    return [tuple(int(v) for v in out[i]) for i in range(max(cm.value, 0))], int(n)
