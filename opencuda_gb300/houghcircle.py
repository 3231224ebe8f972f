"""Python mirror of OpenCUDA's HoughCircle class (okano_3_0/HoughCircle.h:
46-254) over the C ABI of libhoughline_gb300.so (include/hl_circle.h).

Same members, defaults, setters' validation and ErrorCode returns as the
reference; houghcircle returns ``(errcode, circles)`` where the reference
writes through ``int *circleMax`` / ``CircleParam *``.  The reference's
debugging side effect of writing result.bmp is not reproduced.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

from . import _lib
from .houghline import Image


@dataclass
class CircleParam:
    """okano_3_0/HoughCircle.h:37-44"""
    a: int
    b: int
    radius: int
    votes: int

    def astuple(self):
        return (self.a, self.b, self.radius, self.votes)


class HoughCircle:
    """okano_3_0/HoughCircle.h:46-254 over the C ABI."""

    def __init__(self, radiusMin: int = 5, radiusMax: int = 50, distThres: float = 50.0,
                 rThres: int = 20, cirThreshold: int = 100):
        self._L = _lib.load()
        self.radiusMin, self.radiusMax = 5, 50
        self.distThres, self.rThres, self.cirThreshold = 50.0, 20, 100
        # the reference's parameter constructor: defaults first, then the
        # setters (an invalid value keeps the default)
        self.setRadiusMin(radiusMin)
        self.setRadiusMax(radiusMax)
        self.setDistThres(distThres)
        self.setRThres(rThres)
        self.setCirThreshold(cirThreshold)
        p = _lib.hl_params(3.141592653589793 / 180, 1.0, 90, 0.0872664626, 50)
        self._h = C.c_void_p()
        _lib.check(self._L.hl_create(C.byref(self._h), C.byref(p)), "hl_create")

    def close(self):
        if self._h:
            self._L.hl_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- members (okano_3_0/HoughCircle.h:129-236) --------------------------
    def getRadiusMin(self): return self.radiusMin
    def getRadiusMax(self): return self.radiusMax
    def getDistThres(self): return self.distThres
    def getRThres(self): return self.rThres
    def getCirThreshold(self): return self.cirThreshold

    def setRadiusMin(self, v: int) -> int:
        if v < 0:
            return _lib.INVALID_DATA
        self.radiusMin = int(v)
        return _lib.NO_ERROR

    def setRadiusMax(self, v: int) -> int:
        if v < 0:
            return _lib.INVALID_DATA
        self.radiusMax = int(v)
        return _lib.NO_ERROR

    def setDistThres(self, v: float) -> int:
        self.distThres = float(v)
        return _lib.NO_ERROR

    def setRThres(self, v: int) -> int:
        self.rThres = int(v)
        return _lib.NO_ERROR

    def setCirThreshold(self, v: int) -> int:
        if v < 0:
            return _lib.INVALID_DATA
        self.cirThreshold = int(v)
        return _lib.NO_ERROR

    def _params(self) -> _lib.hl_circle_params:
        return _lib.hl_circle_params(self.radiusMin, self.radiusMax, self.distThres,
                                     self.rThres, self.cirThreshold)

    # -- entry points --------------------------------------------------------
    def houghcircle(self, inimg: Image | None, guidingset=None, circleMax: int = 16,
                    stream=None):
        """okano_3_0/HoughCircle.cu:1165-1214, the image path: circles of the
        ROI, centres in image coordinates (the ROI offset added)."""
        if inimg is None and guidingset is None:
            return _lib.NULL_POINTER, []
        if guidingset is not None:
            inimg = points_image(guidingset)
        cm = C.c_int(circleMax)
        out = (_lib.hl_circle * max(circleMax, 1))()
        d = inimg.desc()
        p = self._params()
        rc = self._L.hl_circles(self._h, C.byref(d), C.byref(p), C.byref(cm), out,
                                _stream(stream))
        if rc != _lib.NO_ERROR:
            return rc, []
        return rc, [CircleParam(*out[i].as_tuple()) for i in range(max(cm.value, 0))]

    def houghcircleBatch(self, images, circleMax: int, stream=None):
        """Circles of every image's ROI through one hl_circles_batch call:
        (errcode, [circles of image 0, circles of image 1, ...])."""
        n = len(images)
        if n == 0:
            return _lib.NO_ERROR, []
        descs = (_lib.hl_image_desc * n)(*[im.desc() for im in images])
        out = (_lib.hl_circle * max(n * circleMax, 1))()
        counts = (C.c_int * n)()
        p = self._params()
        rc = self._L.hl_circles_batch(self._h, descs, n, C.byref(p), circleMax, out, counts,
                                      _stream(stream))
        res = [[CircleParam(*out[i * circleMax + k].as_tuple()) for k in range(counts[i])]
               for i in range(n)]
        return rc, res

    def pieceCircle(self, inimg: Image, piecenum: int, circleMax: int, stream=None):
        """okano_3_0/HoughCircle.cu:1323-1400: piecenum x piecenum pieces of
        (width // piecenum) x (height // piecenum), ROI [x*c, x*c + c - 1),
        up to 10 circles each in image coordinates, concatenated in row-major
        piece order up to circleMax; the last piece's ROI stays on inimg.  The
        pieces run as one hl_circles_batch call."""
        if inimg is None:
            return _lib.NULL_POINTER, []
        if piecenum <= 0:
            return _lib.INVALID_DATA, []
        cx, cy = inimg.width // piecenum, inimg.height // piecenum
        pieces = []
        for y in range(piecenum):
            for x in range(piecenum):
                pieces.append(Image(inimg.data, (x * cx, y * cy, x * cx + cx - 1,
                                                 y * cy + cy - 1)))
        rc, per = self.houghcircleBatch(pieces, 10, stream)
        inimg.roiX1, inimg.roiY1 = (piecenum - 1) * cx, (piecenum - 1) * cy
        inimg.roiX2, inimg.roiY2 = piecenum * cx - 1, piecenum * cy - 1
        # the reference keeps the other pieces when one fails (:1366-1375):
        # a piece that overflowed its candidate buffer has no circles here
        if rc not in (_lib.NO_ERROR, _lib.OP_OVERFLOW):
            return rc, []
        out = [c for p in per for c in p]
        return _lib.NO_ERROR, out[:max(circleMax, 0)]

    def accumulator(self, inimg: Image, stream=None):
        """The vote accumulator [radius][row][col] of the ROI (CUDA tensor)."""
        import torch
        nr = self.radiusMax - self.radiusMin + 1
        h = inimg.roiY2 - inimg.roiY1
        w = inimg.roiX2 - inimg.roiX1
        acc = torch.empty((nr, h, w), dtype=torch.int32, device=inimg.data.device)
        d = inimg.desc()
        p = self._params()
        _lib.check(self._L.hl_circle_accumulator(self._h, C.byref(d), C.byref(p),
                                                 C.c_void_p(acc.data_ptr()), _stream(stream)),
                   "hl_circle_accumulator")
        return acc


def points_image(xy) -> Image:
    """The guidingset path of okano_3_0/HoughCircle.cu:1175-1193: a point set
    (an (n, 2) int array of x, y) drawn as 255-pixels into a zero image of
    (max x + 2) x (max y + 2)."""
    import numpy as np
    xy = np.asarray(xy, dtype=np.int64).reshape(-1, 2)
    w = int(xy[:, 0].max()) + 2
    h = int(xy[:, 1].max()) + 2
    img = np.zeros((h, w), np.uint8)
    img[xy[:, 1], xy[:, 0]] = 255
    return Image.from_host(img)


def _stream(stream):
    if stream is None:
        return None
    if isinstance(stream, C.c_void_p):
        return stream
    return C.c_void_p(getattr(stream, "cuda_stream", stream))
