"""The HoughCircle oracle on its own (CPU): known circles are found, and the
vote rule's features (the midpoint steps, the axis points voted twice, the
ROI bounds) hold."""
import numpy as np

from oracle import oracle as O


def _ring(w, h, a, b, r):
    yy, xx = np.mgrid[0:h, 0:w]
    img = np.zeros((h, w), np.uint8)
    img[np.abs(np.hypot(xx - a, yy - b) - r) < 0.5] = 255
    return img


def test_single_point_votes_its_midpoint_circle():
    img = np.zeros((41, 41), np.uint8)
    img[20, 20] = 255
    acc = O.circle_vote(img, 10, 10)[0]
    # radius 10 from the centre: the midpoint steps (x < y) in all octants,
    # the four axis points twice (x0 + 0 and x0 - 0 vote the same cell)
    assert acc[30, 20] == 2 and acc[10, 20] == 2 and acc[20, 30] == 2 and acc[20, 10] == 2
    x, y, d, pts = 0, 10, 3 - 20, []
    while x < y:
        pts.append((x, y))
        if d < y:
            d += 4 * x + 6
        else:
            d += 4 * (x - y) + 10
            y -= 1
        x += 1
    assert acc.sum() == 8 * len(pts)
    assert all(acc[20 + yy, 20 + xx] >= 1 for xx, yy in pts)


def test_votes_outside_the_roi_are_dropped():
    img = np.zeros((10, 10), np.uint8)
    img[0, 0] = 255
    acc = O.circle_vote(img, 3, 3)[0]
    assert acc.sum() < 8 * 3 and acc[3, 0] == 2


def test_known_circles_found():
    img = _ring(200, 160, 70, 80, 25) | _ring(200, 160, 150, 60, 15)
    got, n = O.houghcircle(img, 5, 40, 40, 15.0, 6, 4)
    assert n > 0
    for a, b, r in [(70, 80, 25), (150, 60, 15)]:
        assert any(abs(c[0] - a) <= 1 and abs(c[1] - b) <= 1 and abs(c[2] - r) <= 1
                   for c in got), (a, b, r, got)


def _golden_circle():
    import json
    from pathlib import Path
    g = json.loads((Path(__file__).resolve().parent / "golden" / "golden.json").read_text())
    return g["circle"]


def test_oracle_vote_matches_reference_kernel():
    """The oracle's accumulator against the hash of the reference's own
    _houghcirImgKer (okano_3_0/HoughCircle.cu:187-245) on the same scenes,
    recorded on a GB300 by tests/golden/make_golden.py."""
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
    import cases
    gold = _golden_circle()
    assert set(gold) == set(cases.CIRCLE_CASES)
    for name, c in cases.CIRCLE_CASES.items():
        rec = gold[name]
        assert rec["oracle_equal"] and rec["border_zero"], name
        img = cases.circle_case_image(c)
        assert O.fnv1a(img) == rec["fnv_image"], name
        x1, y1, x2, y2 = cases.circle_case_roi(c)
        acc = O.circle_vote(img[y1:y2, x1:x2], *c["r"])
        assert int(acc.sum(dtype=np.int64)) == rec["sum"], name
        assert O.fnv1a(acc) == rec["fnv_ref_acc"], name
