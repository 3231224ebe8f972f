"""The drop-in C++ surface (include/HoughLine.h, Image.h, CoordiSet.h): a
caller written against the reference's class compiles against these headers
and links the library; on the GPU its results equal the oracle's."""
import ctypes as C
import math
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

import cases
from oracle import oracle as O

ROOT = Path(__file__).resolve().parent.parent
BUILD = ROOT / "opencuda_gb300" / "_build"
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def compile_main(name: str = "houghline_class_main") -> Path:
    exe = BUILD / name
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off",
           "-I", str(ROOT / "include"), "-I", os.path.join(CUDA, "include"),
           str(ROOT / "tests" / "cpp" / (name + ".cpp")),
           "-L", str(BUILD), "-lhoughline_gb300",
           f"-Wl,-rpath,{BUILD}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_caller_compiles_and_links():
    assert compile_main().exists()
    assert compile_main("houghcircle_class_main").exists()


def _parse(out: str):
    res = {}
    for line in out.splitlines():
        parts = line.split()
        if len(parts) >= 2 and parts[1] == "line":
            res.setdefault(parts[0] + "_lines", []).append(
                (float.fromhex(parts[2]), int(parts[3]), int(parts[4])))
        elif len(parts) >= 2 and parts[1].startswith("rc="):
            res[parts[0]] = (int(parts[1][3:]), int(parts[2][2:]))
        else:
            res.setdefault("misc", []).append(parts)
    return res


@pytest.mark.gpu
def test_cpp_class_matches_oracle(cuda):
    exe = compile_main()
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    res = _parse(r.stdout)
    img = cases.synth(1, 1234, 0)
    misc = {p[0]: p[1:] for p in res["misc"]}
    assert int(misc["image"][0].split("=")[1]) == O.fnv1a(img)
    from opencuda_gb300.houghline import HoughLine
    c, s = HoughLine().trig_table()
    thr, K = 100, 16
    ta = float(np.float32(math.pi / 180 * 5.0))
    det = math.pi / 180

    want, _, n = O.houghline(img, c, s, det, 1.0, thr, ta, 50, K)
    assert res["plain"] == (0, n)
    assert res["plain_lines"] == [tuple(w) for w in want]
    assert int(misc["migrated"][0].split("=")[1]) >= 0

    roi = img[21:500, 37:480]
    want_roi, _, n = O.houghline(roi, c, s, det, 1.0, thr, ta, 50, K)
    assert res["roi"] == (0, n)
    assert res["roi_lines"] == [tuple(w) for w in want_roi]
    # getGlobalParam: distance += 37 cos(a) + 21 sin(a) in float, truncated
    libm = C.CDLL("libm.so.6")
    libm.cosf.restype = libm.sinf.restype = C.c_float
    libm.cosf.argtypes = libm.sinf.argtypes = [C.c_float]
    glob = []
    for a, d, v in want_roi:
        x = np.float32(d) + np.float32(37) * np.float32(libm.cosf(a))
        x = np.float32(x) + np.float32(21) * np.float32(libm.sinf(a))
        glob.append((a, int(np.float32(x)), v))
    assert res["global_lines"] == glob

    assert res["img"][0] == 0 and res["img_lines"] == res["plain_lines"]
    import json
    g = json.loads((ROOT / "tests" / "golden" / "golden.json").read_text())
    d = misc["drawn"]
    assert d[0] == "512x512"
    # the lines drawn by the reference's own _houghoutKer, same records
    assert [[a, dd] for a, dd, _ in want] == [[np.float32(x), y] for x, y in g["draw"]["lines"]]
    assert int(d[1].split("=")[1]) == g["draw"]["fnv_image"]
    assert int(d[2].split("=")[1]) == g["draw"]["lit"]

    segs = [(0, 0, 511, 511), (100, 50, 400, 50), (17, 300, 480, 120), (5, 5, 5, 400)]
    got_rl = {int(p[1]): int(p[2]) for p in res["misc"] if p[0] == "realline"}
    for i, sg in enumerate(segs):
        _, real = O.real_line(img, *sg, 2.5, 0.05)
        assert got_rl[i] == int(real), (i, sg)

    ys, xs = np.nonzero(img == 255)
    xy = np.stack([xs, ys], axis=1).astype(np.int32)
    ax, ay = float(np.abs(xy[:, 0]).max()), float(np.abs(xy[:, 1]).max())
    D = int(math.floor(math.sqrt(ax * ax + ay * ay) + 1.0 + 0.5))
    acc, _ = O.vote_points(xy, c, s, -D, 2 * D + 1)
    gg = O.geom(len(c), -D, 2 * D + 1,
                O.ref_numrho(int(xs.max() - xs.min()), int(ys.max() - ys.min())),
                det, 50, ta)
    wp, _, n = O.rank_merge(acc, gg, O.peaks(acc, thr), K)
    assert res["points"] == (0, n)
    assert res["points_lines"] == [tuple(w) for w in wp]
    assert ["null=-2"] in res["misc"]      # NULL_POINTER, okano_3_0/HoughLine.cu:640


@pytest.mark.gpu
def test_cpp_circle_class_matches_oracle(cuda, tmp_path):
    """include/HoughCircle.h: houghcircle on an image, on its ROI and on a
    point set, and pieceCircle, against the oracle."""
    exe = compile_main("houghcircle_class_main")
    W, H = 400, 300
    img = cases.circle_scene(W, H, 8, 8, 45, 3000, 21)
    raw = tmp_path / "scene.raw"
    raw.write_bytes(img.tobytes())
    # the same scene with its bottom-right piece replaced by 40% noise: that
    # piece has far more than 4096 local maxima above the threshold
    ov = img.copy()
    rng = np.random.default_rng(5)
    ov[H // 2:, W // 2:] = np.where(rng.random((H - H // 2, W - W // 2)) < 0.4, 255, 0)
    raw_ov = tmp_path / "overflow.raw"
    raw_ov.write_bytes(ov.tobytes())
    r = subprocess.run([str(exe), str(raw), str(W), str(H), str(raw_ov)], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    got, rcn, misc = {}, {}, {}
    for line in r.stdout.splitlines():
        p = line.split()
        if len(p) == 6 and p[1] == "circle":
            got.setdefault(p[0], []).append(tuple(int(v) for v in p[2:]))
        elif len(p) == 3 and p[1].startswith("rc="):
            rcn[p[0]] = (int(p[1][3:]), int(p[2][2:]))
        else:
            misc[p[0]] = p[1:]
    args = (5, 50, 60, 30.0, 10)

    def oracle(a, cm, ox=0, oy=0):
        want, _ = O.houghcircle(a, args[0], args[1], args[2], args[3], args[4], cm)
        return [(x + ox, y + oy, rr, v) for x, y, rr, v in want]

    full = oracle(img, 32)
    assert rcn["full"] == (0, len(full)) and got.get("full", []) == full and full
    roi = oracle(img[30:H - 10, 40:W - 20], 32, 40, 30)
    assert rcn["roi"] == (0, len(roi)) and got.get("roi", []) == roi
    cx, cy, pieces = W // 2, H // 2, []
    for y in range(2):
        for x in range(2):
            x1, y1 = x * cx, y * cy
            pieces += oracle(img[y1:y1 + cy - 1, x1:x1 + cx - 1], 10, x1, y1)
    pieces = pieces[:64]
    assert rcn["piece"] == (0, len(pieces)) and got.get("piece", []) == pieces
    assert misc["lastroi"] == [str(cx), str(cy), str(2 * cx - 1), str(2 * cy - 1)]
    # one overflowing piece: OP_OVERFLOW for that piece alone, the other three
    # pieces' circles kept by pieceCircle (okano_3_0/HoughCircle.cu:1366-1375)
    assert "ovrc=-3" in r.stdout
    kept = []
    for y in range(2):
        for x in range(2):
            if (x, y) != (1, 1):
                x1, y1 = x * cx, y * cy
                kept += oracle(ov[y1:y1 + cy - 1, x1:x1 + cx - 1], 10, x1, y1)
    assert rcn["pieceov"] == (0, len(kept)) and got.get("pieceov", []) == kept
    ys, xs = np.nonzero(img == 255)
    pim = np.zeros((ys.max() + 2, xs.max() + 2), np.uint8)
    pim[ys, xs] = 255
    pts = oracle(pim, 32)
    assert rcn["points"] == (0, len(pts)) and got.get("points", []) == pts
    assert misc["null=-2"] == [] or "null=-2" in r.stdout
    assert misc["defaults"] == ["5", "50", "50", "20", "100"]
    assert misc["setmin=-1"] == ["keep=5"] and misc["setthr=-1"] == ["keep=100"]

