"""ctypes binding of libhoughline_gb300.so (the C ABI in include/houghline_gb300.h).

The shared library is the product; this module only declares its symbols.
Loading fails loudly when the library has not been built -- there is no
Python or CPU fallback for any kernel.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_build" / "libhoughline_gb300.so"

NO_ERROR = 0
INVALID_DATA = -1
NULL_POINTER = -2
OP_OVERFLOW = -3
NO_FILE = -4
WRONG_FILE = -5
OUT_OF_MEM = -6
CUDA_ERROR = -7
UNMATCH_IMG = -8
UNIMPLEMENT = -998
UNKNOW_ERROR = -999


class hl_params(C.Structure):
    _fields_ = [("detheta", C.c_double), ("derho", C.c_double),
                ("threshold", C.c_int), ("thresang", C.c_float),
                ("thresdis", C.c_int)]


class hl_line(C.Structure):
    _fields_ = [("angle", C.c_float), ("distance", C.c_int), ("votes", C.c_int)]

    def as_tuple(self):
        return (self.angle, self.distance, self.votes)


class hl_circle(C.Structure):
    """CircleParam, okano_3_0/HoughCircle.h:37-44"""
    _fields_ = [("a", C.c_int), ("b", C.c_int), ("radius", C.c_int), ("votes", C.c_int)]

    def as_tuple(self):
        return (self.a, self.b, self.radius, self.votes)


class hl_circle_params(C.Structure):
    _fields_ = [("radius_min", C.c_int), ("radius_max", C.c_int),
                ("dist_thres", C.c_float), ("r_thres", C.c_int), ("threshold", C.c_int)]


class hl_image_desc(C.Structure):
    _fields_ = [("data", C.c_void_p), ("pitch", C.c_size_t),
                ("width", C.c_int), ("height", C.c_int),
                ("roi_x1", C.c_int), ("roi_y1", C.c_int),
                ("roi_x2", C.c_int), ("roi_y2", C.c_int)]


class hl_geom(C.Structure):
    _fields_ = [("numtheta", C.c_int), ("theta_pad", C.c_int),
                ("rho_min", C.c_int), ("numrho", C.c_int),
                ("ref_numrho", C.c_int), ("tiles_x", C.c_int),
                ("tiles_y", C.c_int)]


class hl_scene_params(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("nseg", C.c_int),
                ("len_min", C.c_int), ("len_max", C.c_int),
                ("salt_ppm", C.c_int), ("nbezier", C.c_int),
                ("seed", C.c_uint64)]


class hl_coarse_geom(C.Structure):
    _fields_ = [("cell", C.c_float), ("rho_min", C.c_float), ("inv_rw", C.c_float),
                ("qh", C.c_int), ("qw", C.c_int), ("pad", C.c_int)]


class hl_proposal_opts(C.Structure):
    _fields_ = [("p_cut", C.c_float), ("max_props", C.c_int), ("dilate_theta", C.c_int),
                ("dilate_rho", C.c_int), ("judge_every", C.c_int), ("top_m", C.c_int),
                ("nms", C.c_int), ("p_conf", C.c_float)]


class hl_proposal_stats(C.Structure):
    _fields_ = [("fallback", C.c_int), ("windows", C.c_int), ("judged", C.c_int),
                ("judged_lines", C.c_int), ("judged_found", C.c_int),
                ("fallback_conf", C.c_int), ("votes", C.c_longlong), ("cells", C.c_int),
                ("pad", C.c_int)]


class hl_tune_entry(C.Structure):
    _fields_ = [("window_rows", C.c_int), ("threads", C.c_int), ("ms", C.c_float)]


H = C.c_void_p
P = C.c_void_p
I = C.c_int
PI = C.POINTER(C.c_int)

# name -> (restype, argtypes); every symbol include/houghline_gb300.h declares
SIGNATURES = {
    "hl_create": (I, [C.POINTER(H), C.POINTER(hl_params)]),
    "hl_destroy": (I, [H]),
    "hl_set_params": (I, [H, C.POINTER(hl_params)]),
    "hl_get_params": (I, [H, C.POINTER(hl_params)]),
    "hl_geometry": (I, [H, I, I, C.POINTER(hl_geom)]),
    "hl_trig_table": (I, [H, P, P]),
    "hl_plain": (I, [H, C.POINTER(hl_image_desc), PI, P, P]),
    "hl_plain_async": (I, [H, C.POINTER(hl_image_desc), I, P, P, P]),
    "hl_last_status": (I, [H, PI, P]),
    "hl_batch": (I, [H, C.POINTER(hl_image_desc), I, PI, I, P, PI, P]),
    "hl_batch_async": (I, [H, C.POINTER(hl_image_desc), I, PI, I, P, P, P]),
    "hl_set_batch_graph": (I, [H, I]),
    "hl_tiles": (I, [H, C.POINTER(hl_image_desc), I, I, P, PI, P]),
    "hl_circles": (I, [H, C.POINTER(hl_image_desc), C.POINTER(hl_circle_params), PI, P, P]),
    "hl_circles_batch": (I, [H, P, I, C.POINTER(hl_circle_params), I, P, PI, P]),
    "hl_circle_accumulator": (I, [H, C.POINTER(hl_image_desc), C.POINTER(hl_circle_params),
                                  P, P]),
    "hl_autotune": (I, [H, C.POINTER(hl_image_desc), I, PI, I, C.POINTER(hl_tune_entry),
                        C.POINTER(hl_tune_entry), I, PI, P]),
    "hl_plain_points": (I, [H, P, I, PI, P, P]),
    "hl_compact": (I, [H, C.POINTER(hl_image_desc), P, P, P, P]),
    "hl_compact_noalloc": (I, [C.POINTER(hl_image_desc), P, P, P, P]),
    "hl_compact_noalloc_status": (I, [PI, P]),
    "hl_accumulator": (I, [H, C.POINTER(hl_image_desc), P, P]),
    "hl_accumulator_ref_layout": (I, [H, C.POINTER(hl_image_desc), P, P]),
    "hl_lines_from_accumulator": (I, [H, P, I, I, PI, P, P]),
    "hl_set_vote_shape": (I, [H, I, I]),
    "hl_measure_smem_atomic_peak": (I, [I, C.POINTER(C.c_double), P]),
    "hl_last_launch_count": (I, [H]),
    "hl_profile": (I, [H, I]),
    "hl_profile_read": (I, [H, C.POINTER(C.c_double), PI]),
    "hl_plain_draw": (I, [H, C.POINTER(hl_image_desc), C.POINTER(hl_image_desc), PI, P, P]),
    "hl_draw_lines": (I, [H, C.POINTER(hl_image_desc), P, I, P]),
    "hl_real_line": (I, [H, C.POINTER(hl_image_desc), I, I, I, I, C.c_float, C.c_float,
                         PI, PI, P]),
    "hl_synth_scene": (I, [C.POINTER(hl_scene_params), P, C.c_long]),
    "hl_cnn_conv3x3": (I, [P, P, P, P, P, I, I, I, I, I, I, I, I, P, P]),
    "hl_net_create": (I, [C.POINTER(P), C.c_ulonglong]),
    "hl_net_destroy": (I, [P]),
    "hl_net_num_params": (I, []),
    "hl_net_get_params": (I, [P, P]),
    "hl_net_set_params": (I, [P, P]),
    "hl_net_get_grads": (I, [P, P]),
    "hl_net_forward": (I, [P, P, C.POINTER(hl_coarse_geom), I, P, P]),
    "hl_net_train_step": (I, [P, P, C.POINTER(hl_coarse_geom), P, I, C.c_float, C.c_float,
                              C.POINTER(C.c_float), P]),
    "hl_occupancy": (I, [H, C.POINTER(hl_image_desc), I, P, C.POINTER(hl_coarse_geom), P]),
    "hl_synth_scenes_device": (I, [C.POINTER(hl_scene_params), I, C.POINTER(hl_image_desc), P]),
    "hl_proposal_batch": (I, [H, P, C.POINTER(hl_image_desc), I, PI, I,
                              C.POINTER(hl_proposal_opts), P, P, C.POINTER(hl_proposal_stats),
                              P]),
    "hl_synth_spec": (I, [I, C.c_uint64, I, C.POINTER(hl_scene_params)]),
}

_lib = None


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load (once) and return the native library; raises if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build the CUDA library first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(rc: int, what: str = "call") -> None:
    if rc != NO_ERROR:
        raise RuntimeError(f"{what} failed with ErrorCode {rc}")
