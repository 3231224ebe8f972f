"""Learned proposal stage over the C ABI (include/hl_proposal.h).

HoughNet wraps the network object: occupancy maps of device images, forward
logits, one training step.  Weights are FP32 on the device (BF16 copies feed
the tensor cores); get/set move them as numpy arrays so a trained network
can be saved beside the package and loaded by the proposal pipeline.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import _lib

HEAD_T, HEAD_R, NET_IN = 90, 128, 256
WEIGHTS = Path(__file__).resolve().parent / "weights" / "proposal_net.npy"


class HoughNet:
    def __init__(self, seed: int = 1):
        self._L = _lib.load()
        self._n = C.c_void_p()
        _lib.check(self._L.hl_net_create(C.byref(self._n), seed), "hl_net_create")

    def close(self):
        if self._n:
            self._L.hl_net_destroy(self._n)
            self._n = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._n

    def num_params(self) -> int:
        return int(self._L.hl_net_num_params())

    def get_params(self) -> np.ndarray:
        a = np.zeros(self.num_params(), np.float32)
        _lib.check(self._L.hl_net_get_params(self._n, C.c_void_p(a.ctypes.data)))
        return a

    def set_params(self, a: np.ndarray) -> None:
        a = np.ascontiguousarray(a, np.float32)
        assert a.size == self.num_params()
        _lib.check(self._L.hl_net_set_params(self._n, C.c_void_p(a.ctypes.data)))

    def get_grads(self) -> np.ndarray:
        a = np.zeros(self.num_params(), np.float32)
        _lib.check(self._L.hl_net_get_grads(self._n, C.c_void_p(a.ctypes.data)))
        return a

    @staticmethod
    def geos(geo_list):
        arr = (_lib.hl_coarse_geom * len(geo_list))()
        for i, g in enumerate(geo_list):
            arr[i] = _lib.hl_coarse_geom(*g) if not isinstance(g, _lib.hl_coarse_geom) else g
        return arr

    def occupancy(self, hl, images, stream=None):
        """(occ bf16 tensor [n, 256, 256] as int16 bits, geometry array)"""
        import torch
        n = len(images)
        occ = torch.empty((n, NET_IN, NET_IN), dtype=torch.int16, device="cuda")
        descs = (_lib.hl_image_desc * n)(*[im.desc() for im in images])
        geo = (_lib.hl_coarse_geom * n)()
        _lib.check(self._L.hl_occupancy(hl.handle, descs, n, C.c_void_p(occ.data_ptr()),
                                        geo, hl._stream(stream)), "hl_occupancy")
        return occ, geo

    def forward(self, occ, geo, stream=None):
        """Logits [B, 90, 128] on `stream` (a torch stream, a raw handle, or
        None for the current torch stream)."""
        import torch
        B = int(occ.shape[0])
        out = torch.empty((B, HEAD_T, HEAD_R), dtype=torch.float32, device=occ.device)
        if stream is None:
            stream = torch.cuda.current_stream(occ.device)
        sp = C.c_void_p(getattr(stream, "cuda_stream", stream))
        _lib.check(self._L.hl_net_forward(self._n, C.c_void_p(occ.data_ptr()), geo, B,
                                          C.c_void_p(out.data_ptr()), sp), "hl_net_forward")
        return out

    def train_step(self, occ, geo, target, lr: float, pos_weight: float) -> float:
        B = int(occ.shape[0])
        loss = C.c_float()
        _lib.check(self._L.hl_net_train_step(self._n, C.c_void_p(occ.data_ptr()), geo,
                                             C.c_void_p(target.data_ptr()), B, lr,
                                             pos_weight, C.byref(loss), None),
                   "hl_net_train_step")
        return float(loss.value)

    def save(self, path: Path = WEIGHTS) -> None:
        path.parent.mkdir(parents=True, exist_ok=True)
        np.save(path, self.get_params())

    def load(self, path: Path = WEIGHTS) -> None:
        self.set_params(np.load(path))


def line_targets(lines_per_image, geo) -> np.ndarray:
    """[n, 90, 128] float32: 1 in the coarse cell of every line (angle in
    radians, distance in rho units) of each image."""
    n = len(lines_per_image)
    t = np.zeros((n, HEAD_T, HEAD_R), np.float32)
    for i, lines in enumerate(lines_per_image):
        g = geo[i]
        for ln in lines:
            a, d = (ln.angle, ln.distance) if hasattr(ln, "angle") else (ln[0], ln[1])
            ti = min(max(int(a / (np.pi / HEAD_T)), 0), HEAD_T - 1)
            ri = min(max(int(np.floor((d - g.rho_min) * g.inv_rw)), 0), HEAD_R - 1)
            t[i, ti, ri] = 1.0
    return t


def proposal_batch(hl, net: HoughNet, images, linesmax: int, thresholds=None,
                   p_cut: float = 0.5, max_props: int = 96, dilate_theta: int = 0,
                   dilate_rho: int = 1, judge_every: int = 0, top_m: int = 0,
                   nms: bool = False, p_conf: float = 0.0, stream=None):
    """hl_proposal_batch over a list of device Images: (rc, [[LineParam]],
    stats dict)."""
    import torch
    from .houghline import LineParam
    n = len(images)
    descs = (_lib.hl_image_desc * n)(*[im.desc() for im in images])
    K = max(linesmax, 0)
    lines = torch.zeros(max(n * K * 3, 1), dtype=torch.int32, device="cuda")
    counts = torch.zeros(n, dtype=torch.int32, device="cuda")
    thr = None
    if thresholds is not None:
        thr = (C.c_int * n)(*[int(t) for t in thresholds])
    opts = _lib.hl_proposal_opts(p_cut, max_props, dilate_theta, dilate_rho, judge_every,
                                 top_m, 1 if nms else 0, p_conf)
    st = _lib.hl_proposal_stats()
    L = _lib.load()
    rc = L.hl_proposal_batch(hl.handle, net.handle, descs, n, thr, linesmax, C.byref(opts),
                             C.c_void_p(lines.data_ptr()), C.c_void_p(counts.data_ptr()),
                             C.byref(st), hl._stream(stream))
    if rc != 0:
        return rc, [], {}
    raw = lines.cpu().numpy()[: n * K * 3].reshape(n, K, 3) if K else None
    cnt = counts.cpu().numpy()
    res = []
    for i in range(n):
        out = []
        for j in range(int(cnt[i])):
            a = float(np.array([raw[i, j, 0]], np.int32).view(np.float32)[0])
            out.append(LineParam(a, int(raw[i, j, 1]), int(raw[i, j, 2])))
        res.append(out)
    stats = {k: getattr(st, k) for k in ("fallback", "windows", "judged", "judged_lines",
                                         "judged_found", "fallback_conf", "votes", "cells")}
    return rc, res, stats
