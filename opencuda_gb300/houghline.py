"""Python mirror of OpenCUDA's HoughLine class (okano_3_0/HoughLine.h:82-330)
over the C ABI of libhoughline_gb300.so.

Same member names, defaults, argument meaning and ErrorCode returns as the
reference; each entry point returns ``(errcode, lines)`` where the reference
writes through ``int *linesmax`` / ``LineParam *``.  Device memory comes from
PyTorch tensors (plumbing only: every kernel is in the shared library).
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import _lib

M_PI = math.pi


@dataclass
class LineParam:
    """okano_3_0/HoughLine.h:70-74"""
    angle: float
    distance: int
    votes: int

    def astuple(self):
        return (self.angle, self.distance, self.votes)


class Image:
    """8-bit image with ROI (Image / ImageCuda, okano_3_0/Image.h:44-78).

    ``data`` is a 2-D uint8 tensor; on a CUDA device it is stored pitched
    (row pitch a multiple of 512 bytes, as cudaMallocPitch would give).
    """

    def __init__(self, data, roi=None):
        self.data = data
        self.height, self.width = int(data.shape[0]), int(data.shape[1])
        x1, y1, x2, y2 = roi if roi else (0, 0, self.width, self.height)
        self.roiX1, self.roiY1, self.roiX2, self.roiY2 = x1, y1, x2, y2

    @classmethod
    def from_host(cls, arr: np.ndarray, roi=None, device="cuda", pitch_align=512):
        """copyToCurrentDevice (okano_3_0/Image.cu:435-534): upload a host
        image into pitched device memory."""
        import torch
        arr = np.ascontiguousarray(arr, dtype=np.uint8)
        h, w = arr.shape
        pitch = (w + pitch_align - 1) // pitch_align * pitch_align
        buf = torch.zeros((h, pitch), dtype=torch.uint8, device=device)
        buf[:, :w].copy_(torch.from_numpy(arr))
        img = cls(buf[:, :w], roi)
        img._buf = buf
        return img

    @property
    def pitchBytes(self) -> int:
        return int(self.data.stride(0))

    def desc(self) -> _lib.hl_image_desc:
        return _lib.hl_image_desc(self.data.data_ptr(), self.pitchBytes,
                                  self.width, self.height, self.roiX1,
                                  self.roiY1, self.roiX2, self.roiY2)


class HoughLine:
    """okano_3_0/HoughLine.h:82-330 over the C ABI."""

    def __init__(self, detheta: float = M_PI / 180, derho: float = 1.0,
                 threshold: int = 90, thresang: float | None = None,
                 thresdis: int = 50):
        self._L = _lib.load()
        if thresang is None:
            thresang = float(np.float32(M_PI / 180 * 5.0))
        self._p = _lib.hl_params(detheta, derho, threshold, thresang, thresdis)
        self._h = C.c_void_p()
        _lib.check(self._L.hl_create(C.byref(self._h), C.byref(self._p)), "hl_create")

    def close(self):
        if self._h:
            self._L.hl_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- parameters (okano_3_0/HoughLine.h:158-262) ------------------------
    def _set(self, **kw) -> int:
        p = _lib.hl_params(self._p.detheta, self._p.derho, self._p.threshold,
                           self._p.thresang, self._p.thresdis)
        for k, v in kw.items():
            setattr(p, k, v)
        rc = self._L.hl_set_params(self._h, C.byref(p))
        if rc == _lib.NO_ERROR:
            self._p = p
        return rc

    def getDeTheta(self): return self._p.detheta
    def setDeTheta(self, v): return self._set(detheta=v)
    def getDeRho(self): return self._p.derho
    def setDeRho(self, v): return self._set(derho=v)
    def getThreshold(self): return self._p.threshold
    def setThreshold(self, v): return self._set(threshold=v)
    def getThresAng(self): return self._p.thresang
    def setThresAng(self, v): return self._set(thresang=v)
    def getThresDis(self): return self._p.thresdis
    def setThresDis(self, v): return self._set(thresdis=v)

    @property
    def handle(self):
        return self._h

    def geometry(self, w: int, h: int) -> _lib.hl_geom:
        g = _lib.hl_geom()
        _lib.check(self._L.hl_geometry(self._h, w, h, C.byref(g)), "hl_geometry")
        return g

    def trig_table(self):
        T = int(M_PI / self._p.detheta)
        c = np.zeros(T, np.float32)
        s = np.zeros(T, np.float32)
        _lib.check(self._L.hl_trig_table(self._h, C.c_void_p(c.ctypes.data),
                                         C.c_void_p(s.ctypes.data)))
        return c, s

    # -- entry points -------------------------------------------------------
    def houghLine(self, inimg: Image | None, guidingset=None, linesmax: int = 16,
                  stream=None):
        """okano_3_0/HoughLine.cu:635-955; a non-empty guidingset wins
        (okano_3_0/HoughLine.h:5-8)."""
        if inimg is None and guidingset is None:
            return _lib.NULL_POINTER, []
        if guidingset is not None:
            return self.houghLineCor(guidingset, linesmax, stream)
        lm = C.c_int(linesmax)
        out = (_lib.hl_line * max(linesmax, 1))()
        d = inimg.desc()
        rc = self._L.hl_plain(self._h, C.byref(d), C.byref(lm), out,
                              self._stream(stream))
        if rc != _lib.NO_ERROR:
            return rc, []
        return rc, [LineParam(*out[i].as_tuple()) for i in range(max(lm.value, 0))]

    def houghLineCor(self, guidingset, linesmax: int = 16, stream=None):
        """okano_3_0/HoughLine.cu:352-632; guidingset: (n, 2) int32 CUDA
        tensor of (x, y)."""
        lm = C.c_int(linesmax)
        out = (_lib.hl_line * max(linesmax, 1))()
        n = int(guidingset.shape[0])
        rc = self._L.hl_plain_points(self._h, C.c_void_p(guidingset.data_ptr()), n,
                                     C.byref(lm), out, self._stream(stream))
        if rc != _lib.NO_ERROR:
            return rc, []
        return rc, [LineParam(*out[i].as_tuple()) for i in range(max(lm.value, 0))]

    def accumulator(self, inimg: Image, stream=None):
        """Tight-layout int32 accumulator [R, T] (CUDA tensor) and rho_min."""
        import torch
        g = self.geometry(inimg.roiX2 - inimg.roiX1, inimg.roiY2 - inimg.roiY1)
        acc = torch.empty((g.numrho, g.numtheta), dtype=torch.int32,
                          device=inimg.data.device)
        d = inimg.desc()
        _lib.check(self._L.hl_accumulator(self._h, C.byref(d),
                                          C.c_void_p(acc.data_ptr()),
                                          self._stream(stream)), "hl_accumulator")
        return acc, g.rho_min

    def accumulator_ref_layout(self, inimg: Image, stream=None):
        import torch
        g = self.geometry(inimg.roiX2 - inimg.roiX1, inimg.roiY2 - inimg.roiY1)
        ref = torch.empty((g.ref_numrho + 2, g.numtheta + 2), dtype=torch.int32,
                          device=inimg.data.device)
        d = inimg.desc()
        _lib.check(self._L.hl_accumulator_ref_layout(
            self._h, C.byref(d), C.c_void_p(ref.data_ptr()), self._stream(stream)),
            "hl_accumulator_ref_layout")
        return ref

    def lines_from_accumulator(self, acc, w: int, h: int, linesmax: int, stream=None):
        lm = C.c_int(linesmax)
        out = (_lib.hl_line * max(linesmax, 1))()
        rc = self._L.hl_lines_from_accumulator(self._h, C.c_void_p(acc.data_ptr()), w, h,
                                               C.byref(lm), out, self._stream(stream))
        if rc != _lib.NO_ERROR:
            return rc, []
        return rc, [LineParam(*out[i].as_tuple()) for i in range(max(lm.value, 0))]

    def compact(self, inimg: Image, stream=None):
        """Stage (a): (points uint32 packed x | y << 16, tile offsets, count)."""
        import torch
        g = self.geometry(inimg.roiX2 - inimg.roiX1, inimg.roiY2 - inimg.roiY1)
        w, h = inimg.roiX2 - inimg.roiX1, inimg.roiY2 - inimg.roiY1
        dev = inimg.data.device
        pts = torch.empty(w * h, dtype=torch.int32, device=dev)
        offs = torch.empty(g.tiles_x * g.tiles_y + 1, dtype=torch.int32, device=dev)
        cnt = torch.zeros(1, dtype=torch.int32, device=dev)
        d = inimg.desc()
        _lib.check(self._L.hl_compact(self._h, C.byref(d), C.c_void_p(pts.data_ptr()),
                                      C.c_void_p(offs.data_ptr()), C.c_void_p(cnt.data_ptr()),
                                      self._stream(stream)), "hl_compact")
        return pts, offs, cnt

    def houghLineBatch(self, images, linesmax: int = 16, thresholds=None,
                       stream=None):
        """Batched plain HoughLine over a list of device Images (hl_batch):
        returns (rc, [[LineParam, ...] per image])."""
        n = len(images)
        descs = (_lib.hl_image_desc * max(n, 1))(*[im.desc() for im in images])
        K = max(linesmax, 0)
        out = (_lib.hl_line * max(K * n, 1))()
        counts = (C.c_int * max(n, 1))()
        thr = None
        if thresholds is not None:
            thr = (C.c_int * n)(*[int(t) for t in thresholds])
        rc = self._L.hl_batch(self._h, descs, n, thr, linesmax, out, counts,
                              self._stream(stream))
        if rc != _lib.NO_ERROR:
            return rc, []
        res = []
        for i in range(n):
            res.append([LineParam(*out[i * K + j].as_tuple())
                        for j in range(max(counts[i], 0))])
        return rc, res

    def houghLineTiles(self, inimg: Image, piecenum: int, linesmax: int = 16,
                       stream=None):
        """The tiled caller of okano_3_0/HoughRec.cu:716-760 as one batched
        launch (hl_tiles): piecenum x piecenum cells of (w / piecenum,
        h / piecenum) pixels, cell (x, y) with ROI x1 = x * cell_x,
        x2 = x1 + cell_x - 1 (the reference's exclusive end drops the cell's
        last column and row).  Returns (rc, lines) with lines[y * piecenum + x]
        in the cell's local coordinates, as the reference's per-cell
        houghLine calls give them."""
        n = max(piecenum, 0) ** 2
        K = max(linesmax, 0)
        out = (_lib.hl_line * max(K * n, 1))()
        counts = (C.c_int * max(n, 1))()
        d = inimg.desc()
        rc = self._L.hl_tiles(self._h, C.byref(d), piecenum, linesmax, out, counts,
                              self._stream(stream))
        if rc != _lib.NO_ERROR:
            return rc, []
        return rc, [[LineParam(*out[i * K + j].as_tuple()) for j in range(max(counts[i], 0))]
                    for i in range(n)]

    def set_batch_graph(self, enable: bool) -> int:
        return self._L.hl_set_batch_graph(self._h, 1 if enable else 0)

    def autotune(self, images, linesmax: int = 16, thresholds=None, stream=None):
        """hl_autotune over a list of device Images: (best, [tried...]) as
        (window_rows, threads, ms) tuples; the best shape stays selected."""
        n = len(images)
        descs = (_lib.hl_image_desc * max(n, 1))(*[im.desc() for im in images])
        thr = None
        if thresholds is not None:
            thr = (C.c_int * n)(*[int(t) for t in thresholds])
        best = _lib.hl_tune_entry()
        tried = (_lib.hl_tune_entry * 16)()
        nt = C.c_int()
        _lib.check(self._L.hl_autotune(self._h, descs, n, thr, linesmax, C.byref(best),
                                       tried, 16, C.byref(nt), self._stream(stream)),
                   "hl_autotune")
        return ((best.window_rows, best.threads, best.ms),
                [(tried[i].window_rows, tried[i].threads, tried[i].ms)
                 for i in range(min(nt.value, 16))])

    def set_vote_shape(self, window_rows: int = 0, threads: int = 0) -> int:
        return self._L.hl_set_vote_shape(self._h, window_rows, threads)

    def last_launch_count(self) -> int:
        return self._L.hl_last_launch_count(self._h)

    @staticmethod
    def _stream(stream):
        if stream is None:
            return None
        if isinstance(stream, C.c_void_p):
            return stream
        return C.c_void_p(getattr(stream, "cuda_stream", stream))
