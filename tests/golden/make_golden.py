"""Generate the golden fixtures in this directory on a GB300.

Runs the REFERENCE's own kernels -- _houghlineImgKer, _houghlineCorKer and
_houghoutKer from okano_3_0/HoughLine.cu, and _houghcirImgKer from
okano_3_0/HoughCircle.cu, compiled for sm_103a by oracle/build_ref.sh into
oracle/_ref/ -- on every case of cases.py and records a hash of each result,
plus the cos/sin tables the GPU evaluates (CUDA's cosf/sinf at
theta_k = (float)(k * detheta)).

    python tests/golden/make_golden.py OUT_DIR [--circle-only]

writes OUT_DIR/golden.json and OUT_DIR/trig_tables.npz; the committed copies
in tests/golden/ came from such a run (--circle-only recomputes the circle
records alone, keeping the rest of the committed golden.json).  The
reference's peak kernels _findlocalMaxKer and _findpartmaxKer are never run
(they write outside their buffers).
"""
from __future__ import annotations

import ctypes as C
import json
import math
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(HERE))

import cases  # noqa: E402
from opencuda_gb300 import _lib, build  # noqa: E402
from oracle import oracle as O  # noqa: E402


def trig_tables() -> dict:
    L = _lib.load()
    out = {}
    for name, det in (("T180", cases.DEG1), ("T360", cases.DEG05), ("T720", cases.DEG025)):
        h = C.c_void_p()
        p = _lib.hl_params(det, 1.0, 90, O.default_thresang(), 50)
        _lib.check(L.hl_create(C.byref(h), C.byref(p)), "hl_create")
        T = O.numtheta(det)
        c = np.zeros(T, np.float32)
        s = np.zeros(T, np.float32)
        _lib.check(L.hl_trig_table(h, C.c_void_p(c.ctypes.data), C.c_void_p(s.ctypes.data)))
        L.hl_destroy(h)
        out["cos_" + name] = c
        out["sin_" + name] = s
    return out


def table_for(tables: dict, detheta: float):
    T = O.numtheta(detheta)
    return tables[f"cos_T{T}"], tables[f"sin_T{T}"]


def circle_golden(rr) -> dict:
    """The reference's circle vote on every circle case against the oracle's:
    the reference's buffer has a one-cell zero border per radius plane
    (okano_3_0/HoughCircle.cu:170-179); its interior is the oracle layout."""
    rc = rr.rr_init_circle(str(O.REF_CIRCLE_FATBIN).encode())
    if rc != 0:
        raise RuntimeError("rr_init_circle failed: " + rr.rr_error().decode())
    out = {}
    for name, c in cases.CIRCLE_CASES.items():
        img = cases.circle_case_image(c)
        h, w = img.shape
        x1, y1, x2, y2 = cases.circle_case_roi(c)
        rmin, rmax = c["r"]
        nr, rw, rh = rmax - rmin + 1, x2 - x1, y2 - y1
        ref = np.zeros((nr, rh + 2, rw + 2), np.int32)
        rc = rr.rr_circle_vote(C.c_void_p(img.ctypes.data), w, h, w, x1, y1, x2, y2,
                               rmin, rmax, C.c_void_p(ref.ctypes.data))
        if rc != 0:
            raise RuntimeError(name + ": reference kernel failed: " + rr.rr_error().decode())
        inner = np.ascontiguousarray(ref[:, 1:-1, 1:-1])
        mine = O.circle_vote(np.ascontiguousarray(img[y1:y2, x1:x2]), rmin, rmax)
        rec = {"w": w, "h": h, "roi": [x1, y1, x2, y2], "rmin": rmin, "rmax": rmax,
               "fnv_image": O.fnv1a(img), "fnv_ref_acc": O.fnv1a(inner),
               "sum": int(inner.sum(dtype=np.int64)), "max": int(inner.max()),
               "border_zero": bool(int(ref.sum(dtype=np.int64)) == int(inner.sum(dtype=np.int64))),
               "edge_points": int((img[y1:y2, x1:x2] == 255).sum()),
               "oracle_equal": bool(np.array_equal(mine, inner))}
        out[name] = rec
        print(name, "oracle_equal" if rec["oracle_equal"] else "DIFFERS", rec["sum"])
    return out


def main(out_dir: str, circle_only: bool = False) -> int:
    out = Path(out_dir)
    out.mkdir(parents=True, exist_ok=True)
    build.build_library()
    build.build_oracle()
    runner = build.build_ref_runner()
    rr = C.CDLL(str(runner))
    rr.rr_error.restype = C.c_char_p
    rr.rr_circle_vote.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_long, C.c_int, C.c_int,
                                  C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
    rr.rr_vote_image.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_long, C.c_int,
                                 C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                 C.c_void_p]
    rr.rr_vote_points.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double,
                                  C.c_double, C.c_void_p]
    rr.rr_draw_lines.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                 C.c_int, C.c_void_p]
    rc = rr.rr_init(str(O.REF_FATBIN).encode())
    if rc != 0:
        print("rr_init failed:", rr.rr_error().decode())
        return 1
    if circle_only:
        golden = json.loads((HERE / "golden.json").read_text())
        golden["circle"] = circle_golden(rr)
        with open(out / "golden.json", "w") as f:
            json.dump(golden, f, indent=1, sort_keys=True)
        return 0 if all(r["oracle_equal"] for r in golden["circle"].values()) else 1
    tables = trig_tables()
    np.savez(out / "trig_tables.npz", **tables)
    golden = {"cases": {}, "tables": {}}
    for det in (cases.DEG1, cases.DEG05, cases.DEG025):
        T = O.numtheta(det)
        c, s = table_for(tables, det)
        lc, ls = O.trig_libm(T, det)
        golden["tables"][f"T{T}"] = {
            "fnv_cos": O.fnv1a(c), "fnv_sin": O.fnv1a(s),
            "libm_cos_diff": int((lc != c).sum()), "libm_sin_diff": int((ls != s).sum())}
    for name, case in cases.CASES.items():
        img = cases.image(case)
        h, w = img.shape
        x1, y1, x2, y2 = cases.roi_of(case, img)
        rw, rh = x2 - x1, y2 - y1
        det, derho = case["detheta"], case["derho"]
        T = O.numtheta(det)
        nref = O.ref_numrho(rw, rh, derho)
        cosv, sinv = table_for(tables, det)
        roi = np.ascontiguousarray(img[y1:y2, x1:x2])
        acc, rho_min, dropped = O.vote_image(roi, cosv, sinv, derho)
        # the reference kernel is only run where every vote lands inside its
        # own accumulator rows
        nz = np.nonzero(acc.sum(axis=1))[0]
        off = (nref - 1) // 2
        if len(nz):
            lo, hi = nz[0] + rho_min + off, nz[-1] + rho_min + off
            if lo < 0 or hi >= nref:
                print(f"{name}: skipped, rho rows [{lo},{hi}] outside [0,{nref})")
                continue
        ref = np.zeros((nref + 2, T + 2), np.int32)
        rc = rr.rr_vote_image(C.c_void_p(img.ctypes.data), w, h, w, x1, y1, x2, y2,
                              det, derho, C.c_void_p(ref.ctypes.data))
        if rc != 0:
            print(name, "reference kernel failed:", rr.rr_error().decode())
            return 1
        mine = O.to_ref_layout(acc, rho_min, nref)
        rec = {"w": w, "h": h, "roi": [x1, y1, x2, y2], "detheta": det,
               "derho": derho, "T": T, "ref_numrho": nref,
               "fnv_image": O.fnv1a(img), "fnv_ref_acc": O.fnv1a(ref),
               "sum": int(ref.sum(dtype=np.int64)), "max": int(ref.max()),
               "nnz": int((ref != 0).sum()), "edge_points": int((roi == 255).sum()),
               "oracle_equal": bool(np.array_equal(mine, ref))}
        if not rec["oracle_equal"]:
            d = np.nonzero(mine != ref)
            rec["first_diffs"] = [[int(a), int(b), int(mine[a, b]), int(ref[a, b])]
                                  for a, b in zip(d[0][:8], d[1][:8])]
        golden["cases"][name] = rec
        print(name, "oracle_equal" if rec["oracle_equal"] else "DIFFERS", rec["sum"])
    # coordinate-set path
    xy = cases.point_set()
    w = int(xy[:, 0].max() - xy[:, 0].min())
    hh = int(xy[:, 1].max() - xy[:, 1].min())
    for name, det in (("points_deg1", cases.DEG1), ("points_deg05", cases.DEG05)):
        T = O.numtheta(det)
        nref = O.ref_numrho(w, hh, 1.0)
        ref = np.zeros((nref + 2, T + 2), np.int32)
        rc = rr.rr_vote_points(C.c_void_p(xy.ctypes.data), len(xy), w, hh, det, 1.0,
                               C.c_void_p(ref.ctypes.data))
        if rc != 0:
            print(name, "reference kernel failed:", rr.rr_error().decode())
            return 1
        cosv, sinv = table_for(tables, det)
        off = (nref - 1) // 2
        acc, _ = O.vote_points(xy, cosv, sinv, -off, nref)
        mine = O.to_ref_layout(acc, -off, nref)
        golden["cases"][name] = {"n": len(xy), "box_w": w, "box_h": hh, "detheta": det,
                                 "T": T, "ref_numrho": nref, "fnv_points": O.fnv1a(xy),
                                 "fnv_ref_acc": O.fnv1a(ref),
                                 "sum": int(ref.sum(dtype=np.int64)),
                                 "oracle_equal": bool(np.array_equal(mine, ref))}
        print(name, golden["cases"][name]["oracle_equal"])
    # line drawing: lines of cfg1_s1234 drawn by the reference kernel
    case = cases.CASES["cfg1_s1234"]
    img = cases.image(case)
    cosv, sinv = table_for(tables, case["detheta"])
    lines, _, n = O.houghline(img, cosv, sinv, case["detheta"], 1.0, case["thr"],
                              O.default_thresang(), 50, case["k"])
    ang = np.array([l[0] for l in lines], np.float32)
    dist = np.array([l[2 - 1] for l in lines], np.int32)
    drawn = np.zeros_like(img)
    rc = rr.rr_draw_lines(C.c_void_p(ang.ctypes.data), C.c_void_p(dist.ctypes.data),
                          len(lines), img.shape[1], img.shape[0], 1,
                          C.c_void_p(drawn.ctypes.data))
    if rc != 0:
        print("draw failed:", rr.rr_error().decode())
        return 1
    golden["draw"] = {"case": "cfg1_s1234", "lines": [[float(a), int(d)] for a, d in zip(ang, dist)],
                      "fnv_image": O.fnv1a(drawn), "lit": int((drawn == 255).sum())}
    np.save(out / "draw_cfg1.npy", drawn)
    golden["circle"] = circle_golden(rr)
    with open(out / "golden.json", "w") as f:
        json.dump(golden, f, indent=1, sort_keys=True)
    bad = [n for n, r in golden["cases"].items() if not r["oracle_equal"]]
    print("cases:", len(golden["cases"]), "oracle differs on:", bad)
    return 0


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    if len(args) != 1:
        sys.exit("usage: make_golden.py OUTPUT_DIR [--circle-only]  (run on a GPU host; "
                 "copy OUTPUT_DIR/golden.json next to this script to commit it)")
    sys.exit(main(args[0], circle_only="--circle-only" in sys.argv))
