"""Parity cases: known-answer images and seeded synthetic scenes.

Shared by make_golden.py (which runs the reference's own vote kernel on each
case on a GPU and records the result) and by the tests (which recompute the
same case with the CPU oracle and with the CUDA path).  Images are built
from integer recipes only, so every host produces identical bytes.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

PI = math.pi
DEG1 = PI / 180      # okano_3_0/HoughLine.h:120 default detheta
DEG025 = PI / 720
DEG05 = PI / 360


def _line(img: np.ndarray, x0: int, y0: int, x1: int, y1: int) -> None:
    """Integer Bresenham (same recipe as the product's scene generator)."""
    h, w = img.shape
    dx = abs(x1 - x0)
    dy = -abs(y1 - y0)
    sx = 1 if x0 < x1 else -1
    sy = 1 if y0 < y1 else -1
    err = dx + dy
    while True:
        if 0 <= x0 < w and 0 <= y0 < h:
            img[y0, x0] = 255
        if x0 == x1 and y0 == y1:
            break
        e2 = 2 * err
        if e2 >= dy:
            err += dy
            x0 += sx
        if e2 <= dx:
            err += dx
            y0 += sy


def _splitmix(state: int):
    """Integer stream (the same on every host and numpy version)."""
    while True:
        state = (state + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
        z = state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
        yield z ^ (z >> 31)


def synth(kind: int, seed: int, index: int = 0) -> np.ndarray:
    """Image `index` of workload `kind` (product generator, C, integer-only)."""
    from opencuda_gb300 import _lib
    L = _lib.load()
    specs = (_lib.hl_scene_params * (index + 1))()
    assert L.hl_synth_spec(kind, seed, index + 1, specs) == 0
    p = specs[index]
    img = np.empty((p.height, p.width), np.uint8)
    assert L.hl_synth_scene(C.byref(p), C.c_void_p(img.ctypes.data), p.width) == 0
    return img


def synth_custom(w: int, h: int, nseg: int, lmin: int, lmax: int, ppm: int,
                 seed: int, nbezier: int = 0) -> np.ndarray:
    from opencuda_gb300 import _lib
    L = _lib.load()
    p = _lib.hl_scene_params(w, h, nseg, lmin, lmax, ppm, nbezier, seed)
    img = np.empty((h, w), np.uint8)
    assert L.hl_synth_scene(C.byref(p), C.c_void_p(img.ctypes.data), w) == 0
    return img


def circle_scene(w: int, h: int, ncircles: int, rmin: int, rmax: int, ppm: int,
                 seed: int) -> np.ndarray:
    """Rings drawn with the integer Bresenham circle (d < 0 rule, so not the
    vote's own step rule), radii in [rmin, rmax], centres anywhere in the
    image, plus ppm salt pixels per million; integer-only."""
    rng = _splitmix(seed)
    img = np.zeros((h, w), np.uint8)
    for _ in range(ncircles):
        r = rmin + next(rng) % (rmax - rmin + 1)
        a, b = next(rng) % w, next(rng) % h
        x, y, d = 0, r, 3 - 2 * r
        pts = []
        while x <= y:
            pts += [(a + x, b + y), (a + x, b - y), (a - x, b + y), (a - x, b - y),
                    (a + y, b + x), (a + y, b - x), (a - y, b + x), (a - y, b - x)]
            if d < 0:
                d += 4 * x + 6
            else:
                d += 4 * (x - y) + 10
                y -= 1
            x += 1
        for px, py in pts:
            if 0 <= px < w and 0 <= py < h:
                img[py, px] = 255
    for _ in range(w * h * ppm // 1_000_000):
        img[next(rng) % h, next(rng) % w] = 255
    return img


# HoughCircle parity cases: the ring scene's recipe, the ROI (None: the whole
# image) and the voted radius range
CIRCLE_CASES = {
    "circ_160x120": dict(w=160, h=120, n=3, dr=(8, 40), ppm=5000, seed=5, roi=None,
                         r=(5, 30)),
    "circ_roi_300x200": dict(w=300, h=200, n=6, dr=(5, 60), ppm=10000, seed=6,
                             roi=(17, 11, 283, 190), r=(5, 50)),
    "circ_r0_97x53": dict(w=97, h=53, n=2, dr=(3, 20), ppm=20000, seed=7,
                          roi=(3, 2, 95, 51), r=(0, 12)),
    "circ_700x330": dict(w=700, h=330, n=5, dr=(60, 100), ppm=5000, seed=8,
                         roi=(5, 7, 690, 325), r=(60, 100)),
    "circ_1024": dict(w=1024, h=1024, n=24, dr=(8, 50), ppm=10000, seed=77, roi=None,
                      r=(5, 50)),
}


def circle_case_image(c: dict) -> np.ndarray:
    return circle_scene(c["w"], c["h"], c["n"], c["dr"][0], c["dr"][1], c["ppm"], c["seed"])


def circle_case_roi(c: dict) -> tuple[int, int, int, int]:
    return tuple(c["roi"]) if c["roi"] else (0, 0, c["w"], c["h"])


def kat(name: str) -> np.ndarray:
    if name == "vertical":
        img = np.zeros((48, 64), np.uint8)
        _line(img, 20, 0, 20, 47)
    elif name == "horizontal":
        img = np.zeros((48, 64), np.uint8)
        _line(img, 0, 30, 63, 30)
    elif name == "diag45":
        img = np.zeros((48, 64), np.uint8)
        _line(img, 5, 5, 40, 40)
    elif name == "antidiag":          # negative rho for theta > 90 deg
        img = np.zeros((48, 64), np.uint8)
        _line(img, 60, 2, 20, 42)
    elif name == "single":
        img = np.zeros((48, 64), np.uint8)
        img[9, 7] = 255
    elif name == "empty":
        img = np.zeros((48, 64), np.uint8)
    elif name == "gray":              # only 255 votes (okano_3_0/HoughLine.cu:125)
        img = np.zeros((48, 64), np.uint8)
        _line(img, 0, 10, 63, 40)
        img[img == 255] = 254
        _line(img, 3, 0, 3, 47)
        img[20:25, 30:35] = 128
    elif name == "roi_scene":
        img = synth_custom(300, 200, 0, 0, 0, 20000, 7)   # salt only
        for seg in [(0, 0, 299, 199), (17, 150, 280, 150), (150, 9, 150, 190),
                    (40, 190, 260, 20)]:
            _line(img, *seg)
    elif name == "ragged":            # widths/heights off the 128x32 tiles
        img = synth_custom(333, 127, 6, 40, 300, 15000, 99)
    else:
        raise KeyError(name)
    return img


# Each case: image source, ROI (x1, y1, x2, y2) or None for the full image,
# detheta, derho, plus threshold / linesmax for the line-level checks.
CASES = {
    "kat_vertical": dict(src=("kat", "vertical"), roi=None, detheta=DEG1, derho=1.0, thr=20, k=4),
    "kat_horizontal": dict(src=("kat", "horizontal"), roi=None, detheta=DEG1, derho=1.0, thr=20, k=4),
    "kat_diag45": dict(src=("kat", "diag45"), roi=None, detheta=DEG1, derho=1.0, thr=20, k=4),
    "kat_antidiag": dict(src=("kat", "antidiag"), roi=None, detheta=DEG1, derho=1.0, thr=20, k=4),
    "kat_single": dict(src=("kat", "single"), roi=None, detheta=DEG1, derho=1.0, thr=0, k=8),
    "kat_empty": dict(src=("kat", "empty"), roi=None, detheta=DEG1, derho=1.0, thr=0, k=8),
    "kat_gray": dict(src=("kat", "gray"), roi=None, detheta=DEG1, derho=1.0, thr=20, k=4),
    "kat_roi": dict(src=("kat", "roi_scene"), roi=(17, 9, 283, 191), detheta=DEG1, derho=1.0, thr=60, k=8),
    "ragged_333x127": dict(src=("kat", "ragged"), roi=None, detheta=DEG1, derho=1.0, thr=40, k=16),
    "ragged_roi_odd": dict(src=("kat", "ragged"), roi=(5, 3, 300, 120), detheta=DEG05, derho=1.0, thr=40, k=16),
    "cfg1_s1234": dict(src=("synth", 1, 1234, 0), roi=None, detheta=DEG1, derho=1.0, thr=100, k=16),
    "cfg1_s1": dict(src=("synth", 1, 1, 0), roi=None, detheta=DEG1, derho=1.0, thr=100, k=16),
    "cfg1_s2": dict(src=("synth", 1, 2, 0), roi=None, detheta=DEG1, derho=1.0, thr=100, k=16),
    "cfg1_derho2": dict(src=("synth", 1, 1234, 0), roi=None, detheta=DEG1, derho=2.0, thr=60, k=16),
    "cfg1_deg05": dict(src=("synth", 1, 1234, 0), roi=None, detheta=DEG05, derho=1.0, thr=100, k=16),
    "cfg2_1024": dict(src=("custom", 1024, 1024, 16, 200, 1000, 20000, 5), roi=None, detheta=DEG025, derho=1.0, thr=150, k=64),
    "cfg2_4096": dict(src=("synth", 2, 1234, 0), roi=None, detheta=DEG025, derho=1.0, thr=300, k=256),
    "cfg3_i0": dict(src=("synth", 3, 1234, 0), roi=None, detheta=DEG05, derho=1.0, thr=None, k=32),
    "cfg3_i1": dict(src=("synth", 3, 1234, 1), roi=None, detheta=DEG05, derho=1.0, thr=None, k=32),
    "cfg3_i2": dict(src=("synth", 3, 1234, 2), roi=None, detheta=DEG05, derho=1.0, thr=None, k=32),
}

# Cases small enough for the CPU test run (the oracle finishes in seconds).
CPU_CASES = [n for n in CASES if n not in ("cfg2_4096",)]


def image(case: dict) -> np.ndarray:
    src = case["src"]
    if src[0] == "kat":
        return kat(src[1])
    if src[0] == "synth":
        return synth(src[1], src[2], src[3])
    if src[0] == "custom":
        return synth_custom(*src[1:])
    raise KeyError(src)


def roi_of(case: dict, img: np.ndarray) -> tuple[int, int, int, int]:
    h, w = img.shape
    return case["roi"] if case["roi"] else (0, 0, w, h)


def threshold(case: dict, img: np.ndarray) -> int:
    """Batched scenes use 0.15 * max(w, h)."""
    if case["thr"] is not None:
        return case["thr"]
    h, w = img.shape
    return int(0.15 * max(w, h))


def point_set(seed: int = 11, n: int = 4096, w: int = 700, h: int = 500):
    """Interleaved int (x, y) list with a point at x = 0 and at y = 0 (so the
    reference's box-extent accumulator height covers every rho), n a multiple
    of 16 (the reference's point grid has no tail check)."""
    rng = _splitmix(seed)
    pts = []
    for (x0, y0, x1, y1) in [(0, 0, w - 1, h - 1), (0, 250, w - 1, 250), (350, 0, 350, h - 1)]:
        m = max(abs(x1 - x0), abs(y1 - y0)) + 1
        for i in range(m):
            pts.append((x0 + (x1 - x0) * i // (m - 1), y0 + (y1 - y0) * i // (m - 1)))
    while len(pts) < n:
        pts.append((next(rng) % w, next(rng) % h))
    xy = np.array(pts[:n], np.int32)
    return xy
