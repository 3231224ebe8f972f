"""GPU parity of the batched path (hl_batch): uneven images in one pipeline
give, image by image, the oracle's lines and hl_plain's lines; CUDA-graph
replay and the autotuner keep the results."""
import math

import numpy as np
import pytest

import cases
from oracle import oracle as O

pytestmark = pytest.mark.gpu

DEG05 = math.pi / 360


@pytest.fixture(scope="module")
def hl_mod(cuda):
    from opencuda_gb300.houghline import HoughLine, Image
    return HoughLine, Image


def _batch_images(n, seed=1234):
    """Uneven seeded scenes of the batched workload (256..2048 per side) plus
    small ragged / ROI cases."""
    imgs = [cases.synth(3, seed, i) for i in range(n)]
    rois = [None] * n
    imgs.append(cases.image(cases.CASES["ragged_333x127"]))
    rois.append(None)
    big = cases.synth(1, 7, 0)
    imgs.append(big)
    rois.append((13, 29, 13 + 300, 29 + 211))
    return imgs, rois


def _thr(img, roi):
    h, w = img.shape if roi is None else (roi[3] - roi[1], roi[2] - roi[0])
    return int(0.15 * max(w, h))


def _oracle(hl, img, roi, thr, k):
    c, s = hl.trig_table()
    if roi is not None:
        x1, y1, x2, y2 = roi
        img = img[y1:y2, x1:x2]
    want, _, _ = O.houghline(img, c, s, DEG05, 1.0, thr, hl.getThresAng(),
                             hl.getThresDis(), k)
    return want


def _dev(Image, img, roi):
    return Image.from_host(img, roi) if roi is not None else Image.from_host(img)


def test_batch_matches_oracle_and_plain(hl_mod):
    HoughLine, Image = hl_mod
    imgs, rois = _batch_images(6)
    thr = [_thr(im, r) for im, r in zip(imgs, rois)]
    hl = HoughLine(detheta=DEG05)
    dev = [_dev(Image, im, r) for im, r in zip(imgs, rois)]
    rc, res = hl.houghLineBatch(dev, 32, thr)
    assert rc == 0 and len(res) == len(imgs)
    for i, (im, r) in enumerate(zip(imgs, rois)):
        want = _oracle(hl, im, r, thr[i], 32)
        assert [l.astuple() for l in res[i]] == want, i
        hl.setThreshold(thr[i])
        rc, single = hl.houghLine(dev[i], None, 32)
        assert rc == 0
        assert [l.astuple() for l in single] == want, i


def test_full_benchmark_batch_matches_plain(hl_mod):
    """The whole benchmarked batch (all 256 uneven images of the batched
    workload, theta step 0.5 deg, threshold 0.15 * max(w, h), top-32) through
    one hl_batch call with graph replay and the autotuned vote shape: every
    image's lines equal hl_plain on that image alone, and every 16th image's
    equal the oracle's."""
    HoughLine, Image = hl_mod
    n = 256
    imgs = [cases.synth(3, 1234, i) for i in range(n)]
    thr = [int(0.15 * max(im.shape)) for im in imgs]
    dev = [Image.from_host(im) for im in imgs]
    hl = HoughLine(detheta=DEG05)
    hl.autotune(dev, 32, thr)
    hl.set_batch_graph(True)
    for _ in range(2):          # the second call replays the captured graph
        rc, res = hl.houghLineBatch(dev, 32, thr)
        assert rc == 0 and len(res) == n
    ref = HoughLine(detheta=DEG05)
    for i in range(n):
        ref.setThreshold(thr[i])
        rc, single = ref.houghLine(dev[i], None, 32)
        assert rc == 0
        assert [l.astuple() for l in res[i]] == [l.astuple() for l in single], i
    for i in range(0, n, 16):
        assert [l.astuple() for l in res[i]] == _oracle(ref, imgs[i], None, thr[i], 32), i


def test_batch_default_threshold_and_small_k(hl_mod):
    HoughLine, Image = hl_mod
    imgs, rois = _batch_images(3, seed=99)
    hl = HoughLine(detheta=DEG05, threshold=120)
    dev = [_dev(Image, im, r) for im, r in zip(imgs, rois)]
    rc, res = hl.houghLineBatch(dev, 5)
    assert rc == 0
    for i, (im, r) in enumerate(zip(imgs, rois)):
        assert [l.astuple() for l in res[i]] == _oracle(hl, im, r, 120, 5), i


def test_batch_graph_replay_follows_new_content(hl_mod):
    HoughLine, Image = hl_mod
    a_imgs, a_rois = _batch_images(4, seed=5)
    b_imgs = [cases.synth(3, 5, i) for i in range(4)]   # same sizes
    b_imgs = [np.flipud(im).copy() for im in b_imgs] + a_imgs[4:]
    thr = [_thr(im, r) for im, r in zip(a_imgs, a_rois)]
    hl = HoughLine(detheta=DEG05)
    assert hl.set_batch_graph(True) == 0
    da = [_dev(Image, im, r) for im, r in zip(a_imgs, a_rois)]
    db = [_dev(Image, im, r) for im, r in zip(b_imgs, a_rois)]
    rc, r1 = hl.houghLineBatch(da, 16, thr)      # captures
    assert rc == 0
    rc, r2 = hl.houghLineBatch(da, 16, thr)      # replays
    assert rc == 0 and r1 == r2
    rc, r3 = hl.houghLineBatch(db, 16, thr)      # replays, other images
    assert rc == 0
    for i, (im, r) in enumerate(zip(b_imgs, a_rois)):
        assert [l.astuple() for l in r3[i]] == _oracle(hl, im, r, thr[i], 16), i
    for i, (im, r) in enumerate(zip(a_imgs, a_rois)):
        assert [l.astuple() for l in r1[i]] == _oracle(hl, im, r, thr[i], 16), i


def test_autotune_keeps_results(hl_mod):
    HoughLine, Image = hl_mod
    imgs, rois = _batch_images(4, seed=3)
    thr = [_thr(im, r) for im, r in zip(imgs, rois)]
    hl = HoughLine(detheta=DEG05)
    dev = [_dev(Image, im, r) for im, r in zip(imgs, rois)]
    best, tried = hl.autotune(dev, 16, thr)
    assert best[0] > 0 and best[1] in (512, 1024) and best[2] > 0
    assert len(tried) >= 4 and min(t[2] for t in tried) == best[2]
    rc, res = hl.houghLineBatch(dev, 16, thr)
    assert rc == 0
    for i, (im, r) in enumerate(zip(imgs, rois)):
        assert [l.astuple() for l in res[i]] == _oracle(hl, im, r, thr[i], 16), i


def test_batch_errors(hl_mod):
    HoughLine, Image = hl_mod
    hl = HoughLine(detheta=DEG05)
    rc, _ = hl.houghLineBatch([], 16)
    assert rc == -1   # INVALID_DATA
    im = cases.synth(3, 1, 0)
    d = Image.from_host(im)
    d.roiX2 = d.width + 1   # ROI outside the image
    rc, _ = hl.houghLineBatch([d], 16)
    assert rc == -1


def test_tiled_cells_one_launch(hl_mod):
    """The HoughRec tiling (okano_3_0/HoughRec.cu:716-760): every cell of a
    piecenum x piecenum grid, ROIs [x c, x c + c - 1), in one batched launch
    equals the per-cell plain call and the oracle on the cell."""
    HoughLine, Image = hl_mod
    img = cases.synth_custom(1600, 1200, 40, 60, 900, 15000, 321)
    hl = HoughLine(detheta=math.pi / 180, threshold=40, thresang=float(np.float32(math.pi / 30)),
                   thresdis=15)
    dimg = Image.from_host(img)
    rc, per_cell = hl.houghLineTiles(dimg, 4, 24)
    assert rc == 0 and len(per_cell) == 16
    cx, cy = 1600 // 4, 1200 // 4
    for y in range(4):
        for x in range(4):
            roi = (x * cx, y * cy, x * cx + cx - 1, y * cy + cy - 1)
            rc1, plain = hl.houghLine(Image(dimg.data, roi), None, 24)
            assert rc1 == 0
            got = [l.astuple() for l in per_cell[y * 4 + x]]
            assert got == [l.astuple() for l in plain]
            c, s = hl.trig_table()
            x1, y1, x2, y2 = roi
            want, _, _ = O.houghline(img[y1:y2, x1:x2], c, s, math.pi / 180, 1.0, 40,
                                     hl.getThresAng(), hl.getThresDis(), 24)
            assert got == want


def test_batch_peak_candidates_and_their_overflow(hl_mod):
    """The batched vote and merge note every bin above its image's
    threshold, and the peak pass then tests only those; past the list's
    room it scans every accumulator.  A 4096 x 4096 image (split blocks,
    merged by the merge launch) with uneven ones, first with thresholds that
    only peaks-to-be clear, then with one image at threshold 0 (millions of
    bins: the list overflows), give hl_plain's lines image by image."""
    HoughLine, Image = hl_mod
    imgs = [cases.synth(2, 1234, 0)] + [cases.synth(3, 77, i) for i in range(3)]
    dev = [Image.from_host(im) for im in imgs]
    for derho in (1.0, 2.0):   # the vote's unit and scaled rho forms
        hl = HoughLine(detheta=DEG05)
        ref = HoughLine(detheta=DEG05)
        assert hl.setDeRho(derho) == 0 and ref.setDeRho(derho) == 0
        for thr in ([300] + [int(0.15 * max(im.shape)) for im in imgs[1:]],
                    [300, 0] + [int(0.15 * max(im.shape)) for im in imgs[2:]]):
            rc, res = hl.houghLineBatch(dev, 24, thr)
            assert rc == 0 and len(res) == len(imgs)
            for i in range(len(imgs)):
                ref.setThreshold(thr[i])
                rc, single = ref.houghLine(dev[i], None, 24)
                assert rc == 0
                assert [l.astuple() for l in res[i]] == [l.astuple() for l in single], \
                    (derho, thr, i)
