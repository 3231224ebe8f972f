"""HoughCircle on the GPU engine (include/hl_circle.h) against the CPU
oracle (oracle/circle_oracle.c): the (radius, row, column) accumulator bit
for bit, and the ranked, merged circles."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def ring_image(w, h, circles, noise=0.0, seed=0):
    """255 on the pixels within half a pixel of each circle, plus salt."""
    yy, xx = np.mgrid[0:h, 0:w]
    img = np.zeros((h, w), np.uint8)
    for a, b, r in circles:
        img[np.abs(np.hypot(xx - a, yy - b) - r) < 0.5] = 255
    if noise:
        rng = np.random.default_rng(seed)
        img[rng.random((h, w)) < noise] = 255
    return img


CASES = [
    # (w, h, circles, noise, roi, rmin, rmax, threshold, dist, rthres, cmax)
    (160, 120, [(50, 60, 20), (110, 40, 12)], 0.0, None, 5, 30, 30, 10.0, 5, 8),
    (300, 200, [(80, 90, 35), (200, 100, 22), (150, 40, 9)], 0.01, (17, 11, 283, 190),
     5, 50, 40, 50.0, 20, 16),
    (256, 256, [(128, 128, 60), (60, 60, 18)], 0.02, None, 40, 64, 60, 20.0, 8, 12),
    (97, 53, [(40, 26, 10)], 0.0, (3, 2, 95, 51), 0, 12, 10, 5.0, 3, 4),
    # radii near the accumulator tile's size, an ROI over 4 x 3 tiles
    (700, 330, [(100, 100, 80), (400, 200, 95), (600, 150, 70)], 0.005, (5, 7, 690, 325),
     60, 100, 80, 30.0, 10, 8),
]


@pytest.fixture(scope="module")
def hc_mod(cuda):
    from opencuda_gb300.houghcircle import HoughCircle, points_image
    from opencuda_gb300.houghline import Image
    return HoughCircle, Image, points_image


def _roi_arr(img, roi):
    if roi is None:
        return img
    x1, y1, x2, y2 = roi
    return img[y1:y2, x1:x2]


@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}x{c[1]}r{c[5]}-{c[6]}" for c in CASES])
def test_circle_accumulator_bit_exact(hc_mod, case):
    HoughCircle, Image, _ = hc_mod
    w, h, circles, noise, roi, rmin, rmax, thr, dist, rth, cmax = case
    img = ring_image(w, h, circles, noise, seed=w)
    hc = HoughCircle(rmin, rmax, dist, rth, thr)
    acc = hc.accumulator(Image.from_host(img, roi)).cpu().numpy()
    want = O.circle_vote(_roi_arr(img, roi), rmin, rmax)
    assert acc.shape == want.shape
    assert np.array_equal(acc, want)


@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}x{c[1]}r{c[5]}-{c[6]}" for c in CASES])
def test_circles_match_oracle(hc_mod, case):
    HoughCircle, Image, _ = hc_mod
    w, h, circles, noise, roi, rmin, rmax, thr, dist, rth, cmax = case
    img = ring_image(w, h, circles, noise, seed=w)
    hc = HoughCircle(rmin, rmax, dist, rth, thr)
    rc, got = hc.houghcircle(Image.from_host(img, roi), None, cmax)
    assert rc == 0
    want, n = O.houghcircle(_roi_arr(img, roi), rmin, rmax, thr, dist, rth, cmax)
    ox, oy = (roi[0], roi[1]) if roi else (0, 0)
    assert [c.astuple() for c in got] == [(a + ox, b + oy, r, v) for a, b, r, v in want]
    assert len(got) > 0


def test_circles_found_where_drawn(hc_mod):
    HoughCircle, Image, _ = hc_mod
    img = ring_image(200, 160, [(70, 80, 25), (150, 60, 15)])
    hc = HoughCircle(5, 40, 15.0, 6, 40)
    rc, got = hc.houghcircle(Image.from_host(img), None, 4)
    assert rc == 0
    found = {(c.a, c.b, c.radius) for c in got}
    for a, b, r in [(70, 80, 25), (150, 60, 15)]:
        assert any(abs(fa - a) <= 1 and abs(fb - b) <= 1 and abs(fr - r) <= 1
                   for fa, fb, fr in found), (a, b, r, found)


def test_circle_edge_cases(hc_mod):
    from opencuda_gb300 import _lib
    HoughCircle, Image, _ = hc_mod
    empty = Image.from_host(np.zeros((64, 64), np.uint8))
    hc = HoughCircle(5, 20, 10.0, 5, 10)
    assert hc.houghcircle(empty, None, 8) == (0, [])
    # nothing above the threshold
    img = ring_image(100, 100, [(50, 50, 15)])
    assert HoughCircle(5, 20, 10.0, 5, 100000).houghcircle(Image.from_host(img), None, 8) == (0, [])
    # room for no circle
    rc, got = HoughCircle(5, 20, 10.0, 5, 20).houghcircle(Image.from_host(img), None, 0)
    assert rc == 0 and got == []
    # radius_max < radius_min
    bad = HoughCircle(5, 20, 10.0, 5, 20)
    bad.radiusMax = 3
    assert bad.houghcircle(Image.from_host(img), None, 8)[0] == _lib.INVALID_DATA
    # more local maxima above the threshold than the tail ranks: an error,
    # never a silently shortened list
    noisy = ring_image(400, 400, [], noise=0.3, seed=7)
    rc, _ = HoughCircle(5, 8, 10.0, 5, 0).houghcircle(Image.from_host(noisy), None, 8)
    assert rc == _lib.OP_OVERFLOW


def test_circle_guidingset(hc_mod):
    """The coordinate-set path (okano_3_0/HoughCircle.cu:1175-1193): the points
    drawn into a (max x + 2) x (max y + 2) image, then the image path."""
    HoughCircle, Image, points_image = hc_mod
    img = ring_image(150, 130, [(60, 70, 22)])
    ys, xs = np.nonzero(img)
    xy = np.stack([xs, ys], 1)
    hc = HoughCircle(10, 30, 10.0, 5, 40)
    rc, got = hc.houghcircle(None, xy, 4)
    assert rc == 0
    pim = np.zeros((int(ys.max()) + 2, int(xs.max()) + 2), np.uint8)
    pim[ys, xs] = 255
    want, _ = O.houghcircle(pim, 10, 30, 40, 10.0, 5, 4)
    assert [c.astuple() for c in got] == list(want) and got


def test_accumulator_matches_reference_kernel(hc_mod):
    """The GPU accumulator against the hash of the reference's own
    _houghcirImgKer on the committed circle scenes."""
    import json
    import sys
    from pathlib import Path
    HoughCircle, Image, _ = hc_mod
    here = Path(__file__).resolve().parent / "golden"
    sys.path.insert(0, str(here))
    import cases
    gold = json.loads((here / "golden.json").read_text())["circle"]
    for name, c in cases.CIRCLE_CASES.items():
        img = cases.circle_case_image(c)
        rmin, rmax = c["r"]
        acc = HoughCircle(rmin, rmax).accumulator(
            Image.from_host(img, cases.circle_case_roi(c))).cpu().numpy()
        assert O.fnv1a(np.ascontiguousarray(acc)) == gold[name]["fnv_ref_acc"], name


def test_radii_wider_than_the_tiles(hc_mod):
    """Radii 1452-1457 over a 2960 x 400 ROI: every circle crosses many
    accumulator tiles and most of its votes fall outside the ROI; the
    accumulator and the circles against the oracle."""
    HoughCircle, Image, _ = hc_mod
    rng = np.random.default_rng(5)
    img = np.zeros((400, 2960), np.uint8)
    img[rng.random(img.shape) < 3e-4] = 255
    yy, xx = np.mgrid[0:400, 0:2960]
    img[np.abs(np.hypot(xx - 1480, yy - 1655) - 1455) < 0.5] = 255
    acc = HoughCircle(1452, 1457).accumulator(Image.from_host(img)).cpu().numpy()
    want = O.circle_vote(img, 1452, 1457)
    assert np.array_equal(acc, want)
    rc, got = HoughCircle(1452, 1457, 20.0, 3, 3).houghcircle(Image.from_host(img), None, 16)
    want_c, _ = O.houghcircle(img, 1452, 1457, 3, 20.0, 3, 16)
    assert rc == 0 and [c.astuple() for c in got] == list(want_c)


def test_piece_circle(hc_mod):
    """pieceCircle of the Python mirror: 3 x 3 pieces against the oracle on
    each piece's ROI, concatenated in row-major order."""
    HoughCircle, Image, _ = hc_mod
    img = ring_image(330, 240, [(50, 40, 20), (170, 120, 30), (280, 200, 25), (90, 190, 15)],
                     0.01, seed=3)
    im = Image.from_host(img)
    rc, got = HoughCircle(5, 30, 20.0, 5, 20).pieceCircle(im, 3, 12)
    assert rc == 0
    want = []
    for y in range(3):
        for x in range(3):
            x1, y1 = x * 110, y * 80
            w, _ = O.houghcircle(img[y1:y1 + 79, x1:x1 + 109], 5, 30, 20, 20.0, 5, 10)
            want += [(a + x1, b + y1, r, v) for a, b, r, v in w]
    assert [c.astuple() for c in got] == want[:12]
    assert (im.roiX1, im.roiY1, im.roiX2, im.roiY2) == (220, 160, 329, 239)


def test_piece_circle_keeps_pieces_when_one_overflows(hc_mod):
    """A piece with more than 4096 local maxima above the threshold (dense
    noise) fails alone: pieceCircle keeps the other pieces' circles, as the
    reference does (okano_3_0/HoughCircle.cu:1366-1375)."""
    HoughCircle, Image, _ = hc_mod
    from opencuda_gb300 import _lib
    img = ring_image(330, 240, [(50, 40, 20), (170, 120, 30), (280, 200, 25), (90, 190, 15)],
                     0.01, seed=3)
    rng = np.random.default_rng(9)
    img[80:159, 110:219] = np.where(rng.random((79, 109)) < 0.4, 255, 0)   # piece (1, 1)
    hc = HoughCircle(5, 30, 20.0, 5, 20)
    rc, _ = hc.houghcircle(Image.from_host(img, (110, 80, 219, 159)), None, 10)
    assert rc == _lib.OP_OVERFLOW
    rc, got = hc.pieceCircle(Image.from_host(img), 3, 40)
    assert rc == 0
    want = []
    for y in range(3):
        for x in range(3):
            if (x, y) == (1, 1):
                continue
            x1, y1 = x * 110, y * 80
            w, _ = O.houghcircle(img[y1:y1 + 79, x1:x1 + 109], 5, 30, 20, 20.0, 5, 10)
            want += [(a + x1, b + y1, r, v) for a, b, r, v in w]
    assert [c.astuple() for c in got] == want[:40]



def test_random_configurations(hc_mod):
    """Seeded sweep: image sizes 1-400, ROIs covering at least the middle
    third, radius ranges from 0 to 70 (some wider than the ROI), thresholds
    at 20-90% of the ROI's largest count, noise and rings; accumulator and
    circles against the oracle."""
    HoughCircle, Image, _ = hc_mod
    rng = np.random.default_rng(2024)
    found = 0
    for trial in range(24):
        w, h = int(rng.integers(1, 401)), int(rng.integers(1, 301))
        rings = [(int(rng.integers(0, w)), int(rng.integers(0, h)), int(rng.integers(2, 60)))
                 for _ in range(int(rng.integers(1, 6)))]
        img = ring_image(w, h, rings, float(rng.choice([0.0, 0.01, 0.03])),
                         seed=int(rng.integers(1 << 30)))
        x1, y1 = int(rng.integers(0, w // 3 + 1)), int(rng.integers(0, h // 3 + 1))
        x2 = int(rng.integers(max(x1 + 1, 2 * w // 3), w + 1))
        y2 = int(rng.integers(max(y1 + 1, 2 * h // 3), h + 1))
        rmin = int(rng.integers(0, 30))
        rmax = rmin + int(rng.integers(0, 41))
        dist, rth, cm = float(rng.uniform(1, 60)), int(rng.integers(1, 20)), int(rng.integers(0, 20))
        frac = float(rng.uniform(0.2, 0.9))
        im = Image.from_host(img, (x1, y1, x2, y2))
        roi = img[y1:y2, x1:x2]
        want_acc = O.circle_vote(roi, rmin, rmax)
        acc = HoughCircle(rmin, rmax).accumulator(im).cpu().numpy()
        assert np.array_equal(acc, want_acc), (trial, w, h, rmin, rmax)
        thr = int(frac * int(want_acc.max()))
        rc, got = HoughCircle(rmin, rmax, dist, rth, thr).houghcircle(im, None, cm)
        want, n = O.houghcircle(roi, rmin, rmax, thr, dist, rth, cm)
        if n > 4096:
            assert rc == _lib_overflow(), trial
            continue
        assert rc == 0, (trial, rc)
        assert [c.astuple() for c in got] == [(a + x1, b + y1, r, v) for a, b, r, v in want], trial
        found += len(want)
    assert found > 24


def _lib_overflow():
    from opencuda_gb300 import _lib
    return _lib.OP_OVERFLOW


def test_batch_matches_each_roi(hc_mod):
    """hl_circles_batch over ROIs of different images and sizes (one 1 x 1,
    one without edge pixels) against the oracle on each ROI; then a batch in
    which one ROI has more than 4096 candidates: OP_OVERFLOW, that ROI's
    count 0, the others unchanged."""
    HoughCircle, Image, _ = hc_mod
    from opencuda_gb300 import _lib
    a = ring_image(300, 200, [(80, 90, 35), (200, 100, 22), (150, 40, 9)], 0.01, seed=1)
    b = ring_image(160, 120, [(50, 60, 20), (110, 40, 12)], 0.0)
    c = ring_image(700, 330, [(100, 100, 40), (400, 200, 45), (600, 150, 30)], 0.005, seed=2)
    rois = [(a, (17, 11, 283, 190)), (b, None), (c, (5, 7, 690, 325)), (a, (0, 0, 1, 1)),
            (b, (0, 0, 20, 20)), (c, (300, 100, 520, 300))]
    hc = HoughCircle(5, 50, 20.0, 5, 30)
    imgs = [Image.from_host(x, r) for x, r in rois]
    rc, per = hc.houghcircleBatch(imgs, 12)
    assert rc == 0
    for (x, r), got in zip(rois, per):
        x1, y1, x2, y2 = r if r else (0, 0, x.shape[1], x.shape[0])
        want, _ = O.houghcircle(x[y1:y2, x1:x2], 5, 50, 30, 20.0, 5, 12)
        assert [q.astuple() for q in got] == [(p + x1, s + y1, rr, v) for p, s, rr, v in want]
    assert sum(len(g) for g in per) > 5
    noisy = ring_image(400, 400, [], noise=0.3, seed=7)
    hc2 = HoughCircle(5, 8, 10.0, 5, 0)
    rc, per = hc2.houghcircleBatch([Image.from_host(b), Image.from_host(noisy),
                                    Image.from_host(b)], 8)
    assert rc == _lib.OP_OVERFLOW
    want, _ = O.houghcircle(b, 5, 8, 0, 10.0, 5, 8)
    assert per[1] == [] and [q.astuple() for q in per[0]] == list(want)
    assert [q.astuple() for q in per[2]] == list(want)
