"""hl_compact_noalloc: the compaction entry point for callers that may not
allocate device memory (their memory belongs to another manager or a fixed
budget).  Through the C ABI it must give exactly what the handle-based
hl_compact gives, on two calls in a row (the second call reuses the shared
static scratch the first one left behind).  Collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


def _desc(t, roi):
    from opencuda_gb300 import _lib
    h, w = t.shape
    x1, y1, x2, y2 = roi
    return _lib.hl_image_desc(t.data_ptr(), t.stride(0), w, h, x1, y1, x2, y2)


def _compact_handle(L, hnd, t, roi, torch):
    w, h = roi[2] - roi[0], roi[3] - roi[1]
    ntiles = ((w + 127) // 128) * ((h + 31) // 32)
    pts = torch.full((w * h + 16,), -1, dtype=torch.int32, device=t.device)
    off = torch.full((ntiles + 1,), -1, dtype=torch.int32, device=t.device)
    cnt = torch.full((1,), -1, dtype=torch.int32, device=t.device)
    d = _desc(t, roi)
    assert L.hl_compact(hnd, C.byref(d), C.c_void_p(pts.data_ptr()),
                        C.c_void_p(off.data_ptr()), C.c_void_p(cnt.data_ptr()),
                        None) == 0
    torch.cuda.synchronize()
    return pts, off, cnt


def _compact_noalloc(L, t, roi, torch):
    w, h = roi[2] - roi[0], roi[3] - roi[1]
    ntiles = ((w + 127) // 128) * ((h + 31) // 32)
    pts = torch.full((w * h + 16,), -1, dtype=torch.int32, device=t.device)
    off = torch.full((ntiles + 1,), -1, dtype=torch.int32, device=t.device)
    cnt = torch.full((1,), -1, dtype=torch.int32, device=t.device)
    d = _desc(t, roi)
    assert L.hl_compact_noalloc(C.byref(d), C.c_void_p(pts.data_ptr()),
                                C.c_void_p(off.data_ptr()),
                                C.c_void_p(cnt.data_ptr()), None) == 0
    st = C.c_int(-1)
    assert L.hl_compact_noalloc_status(C.byref(st), None) == 0
    assert st.value == 0, "a look-back wait gave up"
    torch.cuda.synchronize()
    return pts, off, cnt


def test_noalloc_matches_handle_twice(cuda):
    import torch
    from opencuda_gb300 import _lib
    L = _lib.load()
    hnd = C.c_void_p()
    assert L.hl_create(C.byref(hnd), None) == 0
    try:
        # two different inputs back to back: a full 1024 x 768 scene, then an
        # unaligned ROI of another scene with fewer tiles than the first
        runs = [(cases.synth_custom(1024, 768, 12, 60, 700, 25000, 41), (0, 0, 1024, 768)),
                (cases.synth_custom(900, 700, 9, 40, 500, 15000, 42), (3, 5, 611, 433))]
        for img, roi in runs:
            t = torch.from_numpy(img).to(cuda)
            p0, o0, c0 = _compact_handle(L, hnd, t, roi, torch)
            p1, o1, c1 = _compact_noalloc(L, t, roi, torch)
            n = int(c0.item())
            x1, y1, x2, y2 = roi
            assert n == int((img[y1:y2, x1:x2] == 255).sum())
            assert int(c1.item()) == n
            assert torch.equal(o1, o0)
            assert torch.equal(p1[:n], p0[:n])
    finally:
        L.hl_destroy(hnd)


def test_noalloc_rejects_oversized_roi(cuda):
    import torch
    from opencuda_gb300 import _lib
    L = _lib.load()
    # 65536 tiles of 128 x 32 (16384 groups of four) is the limit;
    # 16512 x 16384 needs 129 x 512 tiles = 16512 groups.
    # Inputs and outputs are sized for the ROI all the same, so nothing could
    # be touched out of bounds even if the size check were missing.
    w, h = 16512, 16384
    t = torch.zeros((h, w), dtype=torch.uint8, device=cuda)
    pts = torch.zeros(w * h + 16, dtype=torch.int32, device=cuda)
    off = torch.zeros(129 * 512 + 1, dtype=torch.int32, device=cuda)
    cnt = torch.zeros(1, dtype=torch.int32, device=cuda)
    d = _desc(t, (0, 0, w, h))
    assert L.hl_compact_noalloc(C.byref(d), C.c_void_p(pts.data_ptr()),
                                C.c_void_p(off.data_ptr()),
                                C.c_void_p(cnt.data_ptr()), None) == _lib.OP_OVERFLOW
    del t, pts, off, cnt
    torch.cuda.empty_cache()
