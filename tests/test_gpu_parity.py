"""GPU parity: the CUDA path through the C ABI against the CPU oracle (same
GPU-evaluated cos/sin table), bit-exact, and against the golden hashes of
the reference's own vote kernel."""
import ctypes as C
import json
import math
from pathlib import Path

import numpy as np
import pytest

import cases
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


def _golden():
    p = GOLDEN / "golden.json"
    return json.loads(p.read_text()) if p.exists() else None


@pytest.fixture(scope="module")
def hl_mod(cuda):
    from opencuda_gb300.houghline import HoughLine, Image
    return HoughLine, Image


def _oracle_lines(hl, roi, thr, k, det, derho):
    c, s = hl.trig_table()
    return O.houghline(roi, c, s, det, derho, thr, hl.getThresAng(),
                       hl.getThresDis(), k)


@pytest.mark.parametrize("name", cases.CPU_CASES)
def test_accumulator_bit_exact(hl_mod, name):
    HoughLine, Image = hl_mod
    case = cases.CASES[name]
    img = cases.image(case)
    roi = cases.roi_of(case, img)
    hl = HoughLine(detheta=case["detheta"], derho=case["derho"])
    dimg = Image.from_host(img, roi)
    acc, rho_min = hl.accumulator(dimg)
    x1, y1, x2, y2 = roi
    c, s = hl.trig_table()
    want, wmin, dropped = O.vote_image(img[y1:y2, x1:x2], c, s, case["derho"])
    assert dropped == 0 and rho_min == wmin
    got = acc.cpu().numpy()
    assert got.shape == want.shape
    assert np.array_equal(got, want)
    g = _golden()
    if g and name in g["cases"]:
        ref = hl.accumulator_ref_layout(dimg).cpu().numpy()
        assert O.fnv1a(ref) == g["cases"][name]["fnv_ref_acc"]


@pytest.mark.parametrize("name", cases.CPU_CASES)
def test_lines_match_oracle(hl_mod, name):
    HoughLine, Image = hl_mod
    case = cases.CASES[name]
    img = cases.image(case)
    roi = cases.roi_of(case, img)
    thr = cases.threshold(case, img)
    hl = HoughLine(detheta=case["detheta"], derho=case["derho"], threshold=thr)
    rc, lines = hl.houghLine(Image.from_host(img, roi), None, case["k"])
    assert rc == 0
    x1, y1, x2, y2 = roi
    want, linenum, n = _oracle_lines(hl, img[y1:y2, x1:x2], thr, case["k"],
                                     case["detheta"], case["derho"])
    assert [l.astuple() for l in lines] == want


def test_full_4096_against_golden_and_oracle(hl_mod):
    HoughLine, Image = hl_mod
    case = cases.CASES["cfg2_4096"]
    img = cases.image(case)
    hl = HoughLine(detheta=case["detheta"], threshold=case["thr"])
    dimg = Image.from_host(img)
    g = _golden()
    if g and "cfg2_4096" in g["cases"]:
        ref = hl.accumulator_ref_layout(dimg).cpu().numpy()
        assert O.fnv1a(ref) == g["cases"]["cfg2_4096"]["fnv_ref_acc"]
    acc, _ = hl.accumulator(dimg)
    c, s = hl.trig_table()
    want, _, _ = O.vote_image(img, c, s)
    assert np.array_equal(acc.cpu().numpy(), want)
    rc, lines = hl.houghLine(dimg, None, case["k"])
    assert rc == 0
    R, T = want.shape
    pk = O.peaks(want, case["thr"])
    gg = O.geom(T, -(R // 2), R, O.ref_numrho(4096, 4096), case["detheta"],
                hl.getThresDis(), hl.getThresAng())
    wl, _, _ = O.rank_merge(want, gg, pk, case["k"])
    assert [l.astuple() for l in lines] == wl


def test_split_blocks_across_geometries(hl_mod):
    """Heavy (slice, window) blocks are voted in parts that add into their
    accumulator region, which the compaction launch clears: one handle over a
    run of geometries (each a different split plan, the first one twice, the
    accumulator buffer reused) still gives the oracle's accumulator every
    time."""
    HoughLine, Image = hl_mod
    hl = HoughLine(detheta=math.pi / 720)
    c, s = hl.trig_table()
    # derho 3 at 4096 x 4096: a bin could pass 2^16 votes in principle, so
    # the parts keep 32-bit counts (16-bit ones everywhere else)
    seq = [(4096, 4096, 0, 0, 1.0), (4096, 4096, 0, 0, 1.0), (3000, 1800, 0, 0, 1.0),
           (2500, 2500, 300, 512, 1.0), (4096, 4096, 0, 0, 3.0), (4096, 4096, 0, 0, 1.0)]
    for i, (w, h, rows, threads, derho) in enumerate(seq):
        img = cases.synth_custom(w, h, 40, 200, 3000, 20000, 50 + i)
        assert hl.set_vote_shape(rows, threads) == 0
        assert hl.setDeRho(derho) == 0
        acc, _ = hl.accumulator(Image.from_host(img))
        want, _, _ = O.vote_image(img, c, s, derho)
        assert np.array_equal(acc.cpu().numpy(), want), (w, h, rows, threads, derho)


@pytest.mark.parametrize("rows,threads", [(64, 256), (200, 512), (1000, 1024), (1400, 512)])
def test_vote_shapes_agree(hl_mod, rows, threads):
    """Rho windows narrower than the rho range exercise the tile filter."""
    HoughLine, Image = hl_mod
    img = cases.synth_custom(1500, 900, 12, 100, 1200, 15000, 3)
    hl = HoughLine(detheta=cases.DEG05)
    dimg = Image.from_host(img)
    assert hl.set_vote_shape(rows, threads) == 0
    acc, _ = hl.accumulator(dimg)
    c, s = hl.trig_table()
    want, _, _ = O.vote_image(img, c, s)
    assert np.array_equal(acc.cpu().numpy(), want)


def test_compaction_points_and_order(hl_mod):
    HoughLine, Image = hl_mod
    img = cases.kat("ragged")
    roi = (5, 3, 300, 120)
    hl = HoughLine()
    pts, offs, cnt = hl.compact(Image.from_host(img, roi))
    n = int(cnt.item())
    x1, y1, x2, y2 = roi
    sub = img[y1:y2, x1:x2]
    assert n == int((sub == 255).sum())
    p = pts[:n].cpu().numpy().astype(np.uint32)
    xs, ys = (p & 0xFFFF).astype(np.int64), (p >> 16).astype(np.int64)
    assert np.all(sub[ys, xs] == 255)
    # tile-major order (128 x 32 tiles), raster order inside each tile
    tiles_x = (x2 - x1 + 127) // 128
    key = ((ys // 32) * tiles_x + xs // 128) * 4096 + (ys % 32) * 128 + xs % 128
    assert np.all(np.diff(key) > 0)
    o = offs.cpu().numpy()
    assert o[0] == 0 and o[-1] == n and np.all(np.diff(o) >= 0)


@pytest.mark.parametrize("w,h", [(4096, 4096), (8192, 2560), (1000, 37)])
def test_compaction_large_and_fallback(hl_mod, w, h):
    """About one CTA per SM (a cooperative launch) up to the tiles that many
    CTAs can hold, one CTA per 4-tile group beyond (8192 x 2560 has 5120
    tiles): the same points, order and tile offsets either way."""
    HoughLine, Image = hl_mod
    img = cases.synth_custom(w, h, 30, 100, 4000, 25000, 77)
    hl = HoughLine()
    for _ in range(2):
        pts, offs, cnt = hl.compact(Image.from_host(img))
        n = int(cnt.item())
        assert n == int((img == 255).sum())
        p = pts[:n].cpu().numpy().astype(np.uint32)
        xs, ys = (p & 0xFFFF).astype(np.int64), (p >> 16).astype(np.int64)
        assert np.all(img[ys, xs] == 255)
        tiles_x = (w + 127) // 128
        key = ((ys // 32) * tiles_x + xs // 128) * 4096 + (ys % 32) * 128 + xs % 128
        assert np.all(np.diff(key) > 0)
        o = offs.cpu().numpy()
        tile = (ys // 32) * tiles_x + xs // 128
        want = np.searchsorted(tile, np.arange(len(o) - 1))
        assert np.array_equal(o[:-1], want) and o[-1] == n


def test_compaction_unaligned_and_repeat(hl_mod):
    """Misaligned ROI origins take the scalar path; repeated calls reuse the
    epoch-tagged look-back state without clearing it."""
    HoughLine, Image = hl_mod
    img = cases.synth_custom(1000, 700, 10, 50, 600, 30000, 21)
    hl = HoughLine()
    for roi in [(0, 0, 1000, 700), (3, 1, 997, 699), (16, 0, 1000, 700), (1, 5, 2, 6)]:
        for _ in range(2):
            pts, offs, cnt = hl.compact(Image.from_host(img, roi))
            x1, y1, x2, y2 = roi
            assert int(cnt.item()) == int((img[y1:y2, x1:x2] == 255).sum())


def test_points_path_matches_oracle(hl_mod, cuda):
    import torch
    HoughLine, _ = hl_mod
    xy = cases.point_set()
    hl = HoughLine(threshold=30)
    t = torch.from_numpy(xy).to(cuda)
    rc, lines = hl.houghLineCor(t, 16)
    assert rc == 0
    c, s = hl.trig_table()
    ax = float(np.abs(xy[:, 0]).max())
    ay = float(np.abs(xy[:, 1]).max())
    d = int(math.floor(math.sqrt(ax * ax + ay * ay) + 1.0 + 0.5))
    acc, dropped = O.vote_points(xy, c, s, -d, 2 * d + 1)
    assert dropped == 0
    w = int(xy[:, 0].max() - xy[:, 0].min())
    h = int(xy[:, 1].max() - xy[:, 1].min())
    g = O.geom(len(c), -d, 2 * d + 1, O.ref_numrho(w, h), hl.getDeTheta(),
               hl.getThresDis(), hl.getThresAng())
    want, _, _ = O.rank_merge(acc, g, O.peaks(acc, 30), 16)
    assert [l.astuple() for l in lines] == want


def test_stage_c_many_candidates(hl_mod, cuda):
    """More peaks than one finalize chunk (radix-select path) and many vote
    ties: ranking, decode and merge against the oracle."""
    import torch
    HoughLine, _ = hl_mod
    w, h = 400, 300
    hl = HoughLine(threshold=0)
    g = hl.geometry(w, h)
    rng = np.random.default_rng(5)
    acc = rng.integers(0, 6, size=(g.numrho, g.numtheta)).astype(np.int32)
    for linesmax in (16, 300, 5000):
        rc, lines = hl.lines_from_accumulator(torch.from_numpy(acc).to(cuda), w, h,
                                              linesmax)
        assert rc == 0
        gg = O.geom(g.numtheta, g.rho_min, g.numrho, g.ref_numrho, hl.getDeTheta(),
                    hl.getThresDis(), hl.getThresAng())
        want, linenum, n = O.rank_merge(acc, gg, O.peaks(acc, 0), linesmax)
        assert len(O.peaks(acc, 0)) > 1024
        assert [l.astuple() for l in lines] == want


def test_error_codes(hl_mod):
    HoughLine, Image = hl_mod
    hl = HoughLine()
    img = Image.from_host(np.zeros((40, 50), np.uint8))
    assert hl.houghLine(None, None, 4)[0] == -2          # NULL_POINTER
    img.roiX2 = 60                                       # ROI beyond the image
    assert hl.houghLine(img, None, 4)[0] == -1           # INVALID_DATA
    img.roiX2 = img.roiX1                                # empty ROI
    assert hl.houghLine(img, None, 4)[0] == -1
    assert hl.setDeTheta(0.0) == -1
    assert hl.getDeTheta() == math.pi / 180
    ok = Image.from_host(cases.kat("vertical"))
    rc, lines = hl.houghLine(ok, None, 0)
    assert rc == 0 and lines == []


def test_trig_table_matches_golden(hl_mod):
    HoughLine, _ = hl_mod
    p = GOLDEN / "trig_tables.npz"
    if not p.exists():
        pytest.skip("golden tables not generated yet")
    z = np.load(p)
    for det in (cases.DEG1, cases.DEG05, cases.DEG025):
        c, s = HoughLine(detheta=det).trig_table()
        T = len(c)
        assert np.array_equal(c, z[f"cos_T{T}"]) and np.array_equal(s, z[f"sin_T{T}"])


@pytest.mark.parametrize("w,h,det,derho,noise,roi", [
    (512, 512, math.pi / 180, 1.0, 10000, None),          # the 512 x 512 configuration
    (640, 480, math.pi / 180, 1.0, 20000, (7, 3, 631, 470)),
    (333, 127, math.pi / 90, 1.0, 30000, None),            # 3 CTAs of 32 thetas
    (600, 600, math.pi / 256, 1.0, 8000, None),            # 8 CTAs, the most a cluster takes
    (512, 384, math.pi / 180, 2.0, 10000, None),           # rho step 2 (irho = 0.5)
    (1, 1, math.pi / 180, 1.0, 0, None),
])
def test_small_image_single_launch(hl_mod, w, h, det, derho, noise, roi):
    """Small images take one cluster launch (compaction, vote, peaks and the
    tail, the accumulator in shared memory only); its lines must equal the
    multi-launch pipeline's (forced by a vote shape) and the oracle's."""
    HoughLine, Image = hl_mod
    img = cases.synth_custom(w, h, 6, 20, max(w, h) // 2 + 20, noise, w + h)
    if w == 1:
        img[:] = 255
    thr = 30 if w > 1 else 0
    dev = Image.from_host(img, roi)
    hl = HoughLine(detheta=det, derho=derho, threshold=thr)
    rc, small = hl.houghLine(dev, None, 24)
    assert rc == 0 and hl.last_launch_count() == 1
    ref = HoughLine(detheta=det, derho=derho, threshold=thr)
    assert ref.set_vote_shape(1000, 1024) == 0
    rc, multi = ref.houghLine(dev, None, 24)
    assert rc == 0 and ref.last_launch_count() > 1
    x1, y1, x2, y2 = roi if roi else (0, 0, w, h)
    want, _, _ = _oracle_lines(hl, img[y1:y2, x1:x2], thr, 24, det, derho)
    assert [l.astuple() for l in small] == want
    assert [l.astuple() for l in multi] == want
    # a second call on the same handle reuses the cleared candidate counter
    rc, again = hl.houghLine(dev, None, 24)
    assert rc == 0 and [l.astuple() for l in again] == want
