#!/usr/bin/env python
"""Plain HoughLine throughput on one GB300 (or N, one process per GPU).

Workload: one 4096 x 4096 uint8 binary image per step -- 64 seeded segments of
200-3000 px plus 2% salt (about 0.44 M edge points), theta step 0.25 deg
(T = 720), rho step 1 px over [-5793, 5793] (R = 11587), threshold 300,
top-256 lines: compaction -> vote -> peak NMS -> rank/merge, all on the GPU.

  value : images/s with the image resident in HBM (device time per step,
          CUDA events around each step; L2 flushed between steps, flush not
          timed; the per-stage times come from a separate pass, since stage
          events between the kernels would serialise their launches)
  e2e   : images/s through the C ABI with host buffers: every step copies
          its image from pinned host memory and reads its LineParam records
          back (hl_plain_async; upload and read-back streams, two device image
          and two device result buffers), overlapping the neighbouring steps'
          kernels
  roofline : the vote kernel against the measured shared-memory atomic
          ceiling of this GPU (conflict-free int32 atomicAdd micro-kernel);
          the whole pipeline against measured HBM bandwidth is reported
          beside it
  cpu_baseline : the C transcription of the reference's vote loop + host
          tail (oracle/hough_oracle.c) on this host's cores
  circle : HoughCircle (include/hl_circle.h) at the reference's default
          parameters on a 1024 x 1024 ring scene: device and e2e images/s,
          votes against the shared-memory atomic ceiling, the C restatement
          (oracle/circle_oracle.c) on this host's cores beside it

--impl reference times that CPU transcription alone (the reference's path
has no CPU implementation of its own; its GPU kernels are the K40-era code
this project replaces).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests" / "golden"))

METRIC = "images/s, Gvotes/s: proposal-guided vs plain Hough, 1 GB300, >=99% recall"
DETHETA = math.pi / 720
THRESHOLD = 300
LINESMAX = 256
W = H = 4096


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def reduce_over_ranks(times, votes: float, ws: int, device):
    """Timings: the slowest rank's (max); votes: the whole job's (sum)."""
    import torch
    t = torch.tensor(list(times) + [votes], dtype=torch.float64, device=device)
    if ws > 1:
        import torch.distributed as dist
        tt = t[:-1].clone()
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        vt = t[-1:].clone()
        dist.all_reduce(vt, op=dist.ReduceOp.SUM)
        t = torch.cat([tt, vt])
    return tuple(float(x) for x in t.tolist())


def bench_config(n_gpus: int) -> dict:
    """The workload description both arms print (identical dicts)."""
    return {"workload": "plain HoughLine 4096x4096, T=720, R=11587, thr 300, top-256",
            "images_per_step_per_gpu": 1,
            "parallelism": f"replicas x{n_gpus} (images sharded, no collective)",
            "l2": "flushed between device-timed steps (256 MiB write, not timed)"}


def make_images(rank: int, n: int):
    import cases
    return [cases.synth(2, 1234 + 1000 * rank + i, 0) for i in range(n)]


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text()), "measured"
        except Exception:
            pass
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def ncu_traffic():
    """Per-launch DRAM bytes of the vote kernel from the committed ncu summary."""
    p = ROOT / "profiles" / "vote_kernel_4096.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.strip().startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


class NvmlClockSampler:
    """SM clock and clock-event reasons read from NVML (the driver's
    libnvidia-ml, through ctypes; read-only queries) by a thread every
    millisecond while it runs, so a timed region of a few milliseconds still
    gets samples.  None when NVML is unavailable."""
    SM = 1
    REASONS = {0x8: "hw_slowdown", 0x40: "hw_thermal_slowdown", 0x20: "sw_thermal_slowdown",
               0x4: "sw_power_cap"}

    def __init__(self, torch_device):
        import threading
        self.rows, self.h, self.nv = [], None, None
        try:
            nv = C.CDLL("libnvidia-ml.so.1")
            if nv.nvmlInit_v2() != 0:
                return
            import torch
            pr = torch.cuda.get_device_properties(torch_device)
            h = C.c_void_p()
            bus = getattr(pr, "pci_bus_id", None)
            dom = getattr(pr, "pci_domain_id", 0)
            devid = getattr(pr, "pci_device_id", 0)
            ok = False
            if bus is not None:
                ident = f"{dom:08x}:{bus:02x}:{devid:02x}.0".encode()
                ok = nv.nvmlDeviceGetHandleByPciBusId_v2(ident, C.byref(h)) == 0
            if not ok and nv.nvmlDeviceGetHandleByIndex_v2(
                    int(torch_device.index or 0), C.byref(h)) != 0:
                return
            self.nv, self.h = nv, h
            mx = C.c_uint()
            self.max_mhz = float(mx.value) if nv.nvmlDeviceGetMaxClockInfo(
                h, self.SM, C.byref(mx)) == 0 else None
        except (OSError, AttributeError):
            return
        self.stop_flag = threading.Event()
        self.t = threading.Thread(target=self._run, daemon=True)
        self.t.start()

    def _sample(self):
        mhz, rs = C.c_uint(), C.c_ulonglong()
        if self.nv.nvmlDeviceGetClockInfo(self.h, self.SM, C.byref(mhz)) != 0:
            return
        f = getattr(self.nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.nv.nvmlDeviceGetCurrentClocksThrottleReasons
        r = rs.value if f(self.h, C.byref(rs)) == 0 else 0
        self.rows.append((float(mhz.value), r))

    def _run(self):
        while not self.stop_flag.is_set():
            self._sample()
            time.sleep(0.001)

    def stop(self):
        if self.h is None:
            return None
        self.stop_flag.set()
        self.t.join(timeout=5)
        if not self.rows:
            self._sample()
        if not self.rows:
            return None
        reasons = sorted({n for _, r in self.rows for b, n in self.REASONS.items() if r & b})
        return {"sm_mhz": statistics.median(m for m, _ in self.rows),
                "sm_max_mhz": self.max_mhz, "reasons": reasons, "samples": len(self.rows),
                "source": "NVML every 1 ms during the timed steps"}


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: str):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", gpu_index], stdout=self.f, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = []
        for line in Path(self.f.name).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.f.name)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r)
                          if v.lower().startswith("active")})
        return {"sm_mhz": statistics.median(r[0] for r in rows),
                "sm_max_mhz": max(r[1] for r in rows), "reasons": reasons,
                "samples": len(rows)}


def cpu_reference_images(imgs, budget_s: float, min_images: int = 1):
    """The C transcription of the reference path on all host cores."""
    from oracle import oracle as O
    c, s = O.trig_libm(O.numtheta(DETHETA), DETHETA)
    t0 = time.perf_counter()
    n = votes = 0
    while True:
        img = imgs[n % len(imgs)]
        O.houghline(img, c, s, DETHETA, 1.0, THRESHOLD, O.default_thresang(), 50,
                    LINESMAX)
        votes += int((img == 255).sum()) * O.numtheta(DETHETA)
        n += 1
        el = time.perf_counter() - t0
        if n >= min_images and el >= budget_s:
            break
        if n >= min_images and el / n * (n + 1) > budget_s * 1.5:
            break
    return n, el, votes, O.max_threads()


def batched_workload(L, HoughLine, Image, dev, sp, reps: int, atom_peak: float, cpu: bool):
    """The batched configuration: 256 seeded uneven images (sides 256-2048),
    theta step 0.5 deg, threshold 0.15 * max(w, h) per image, top-32, through
    one hl_batch_async pipeline (CUDA-graph replay, autotuned vote shape);
    images resident in HBM, L2 flushed between batches.  Untimed afterwards:
    every image's batched result against hl_plain on that image, and (in the
    CPU-baseline leg) every 16th image against the C restatement of the
    reference path, timed as the batched CPU baseline."""
    import torch
    import cases
    n, K, det = 256, 32, math.pi / 360
    imgs = [cases.synth(3, 1234, i) for i in range(n)]
    dimgs = [Image.from_host(im, device=dev) for im in imgs]
    thr = [int(0.15 * max(im.shape)) for im in imgs]
    votes = sum(int((im == 255).sum()) for im in imgs) * int(math.pi / det)
    hl = HoughLine(detheta=det)
    best, _ = hl.autotune(dimgs, K, thr, stream=sp)
    hl.set_batch_graph(True)
    descs = (_lib_mod().hl_image_desc * n)(*[d.desc() for d in dimgs])
    th = (C.c_int * n)(*thr)
    lines = torch.empty(n * K * 3, dtype=torch.int32, device=dev)
    counts = torch.zeros(n, dtype=torch.int32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def run():
        rc = L.hl_batch_async(hl.handle, descs, n, th, K, C.c_void_p(lines.data_ptr()),
                              C.c_void_p(counts.data_ptr()), sp)
        if rc != 0:
            raise RuntimeError(f"hl_batch_async returned {rc}")
    for _ in range(3):
        run()
    torch.cuda.synchronize(dev)
    ms = []
    for _ in range(reps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        run()
        e1.record()
        torch.cuda.synchronize(dev)
        ms.append(e0.elapsed_time(e1))
    st = C.c_int()
    L.hl_last_status(hl.handle, C.byref(st), sp)
    if st.value != 0:
        raise RuntimeError(f"batched device status {st.value}")
    t = statistics.median(ms)
    # parity at the benched size: every image's batched lines against hl_plain
    # on that image alone (same handle parameters, that image's threshold)
    T = int(math.pi / det)
    got = lines.view(n, K, 3).cpu().numpy()
    got_n = counts.cpu().numpy()
    ref = HoughLine(detheta=det)
    _lib = _lib_mod()
    out = (_lib.hl_line * K)()
    differ = []
    for i in range(n):
        ref.setThreshold(thr[i])
        lm = C.c_int(K)
        d = dimgs[i].desc()
        rc = L.hl_plain(ref.handle, C.byref(d), C.byref(lm), out, sp)
        if rc != 0:
            raise RuntimeError(f"hl_plain returned {rc}")
        want = np.frombuffer(bytes(out), np.int32).reshape(K, 3)[:lm.value]
        if int(got_n[i]) != lm.value or not np.array_equal(got[i, :lm.value], want):
            differ.append(i)
    pix = int(sum(im.size for im in imgs))
    acc_bytes = sum(4 * T * ref.geometry(im.shape[1], im.shape[0]).numrho for im in imgs)
    res = {"workload": "batched plain HoughLine: 256 uneven images (w, h in [256, 2048]), "
                       "T=360, rho +-diag per image, thr 0.15*max(w,h), top-32",
           "value": n / (t / 1e3), "unit": "images/s", "ms_per_batch": t,
           "gvotes_per_s": votes / (t / 1e3) / 1e9, "pixels": pix,
           "reps": reps, "graph": True, "l2": "flushed between batches",
           "vote_shape": {"window_rows": best[0], "threads": best[1]},
           "matches_plain": not differ, "images_checked_against_plain": n,
           "roofline": {"bound": "smem_atomic", "achieved": votes / (t / 1e3) / 1e12,
                        "peak": atom_peak / 1e12, "unit": "T atomics/s",
                        "frac": votes / (t / 1e3) / atom_peak,
                        "note": "whole batch call (every launch) as the time",
                        "hbm": {"bytes_per_batch": pix + acc_bytes,
                                "achieved_gbs": (pix + acc_bytes) / (t / 1e3) / 1e9,
                                "scope": "images read once + accumulators written once"}}}
    if differ:
        res["differs_from_plain"] = differ[:16]
    if cpu:
        from oracle import oracle as O
        cosv, sinv = ref.trig_table()
        sample = list(range(0, n, 16))
        bad, t0 = [], time.perf_counter()
        for i in sample:
            w_lines, _, _ = O.houghline(imgs[i], cosv, sinv, det, 1.0, thr[i],
                                        ref.getThresAng(), ref.getThresDis(), K)
            a = got[i, :got_n[i]]
            mine = [(float(np.int32(r[0]).view(np.float32)), int(r[1]), int(r[2])) for r in a]
            if mine != [tuple(x) for x in w_lines]:
                bad.append(i)
        tc = time.perf_counter() - t0
        res["matches_oracle"] = not bad
        res["images_checked_against_oracle"] = len(sample)
        res["cpu_baseline"] = {"value": len(sample) / tc, "unit": "images/s",
                               "cores": O.max_threads(), "kind": "port",
                               "sample": f"{len(sample)} of the 256 images (every 16th) through "
                                         "the C restatement of the reference path, OpenMP "
                                         "over theta columns; their lines compared with the "
                                         "batched result"}
    return res


def latency_512(L, HoughLine, Image, dev, reps: int = 300):
    """The 512 x 512 single-image configuration (8 segments, 1% salt, theta
    step 1 deg, threshold 100, top-16): latency-bound.  Host wall time per
    synchronous call through the C ABI (image resident on the device, lines
    returned to the host), for hl_plain (five launches and one copy) and for
    the same image through hl_batch with CUDA-graph replay."""
    import cases
    img = cases.synth(1, 1234, 0)
    d = Image.from_host(img, device=dev)
    hl = HoughLine(detheta=math.pi / 180, threshold=100)
    _lib = _lib_mod()
    desc = d.desc()
    lm = C.c_int()
    out = (_lib.hl_line * 16)()

    def plain():
        lm.value = 16
        rc = L.hl_plain(hl.handle, C.byref(desc), C.byref(lm), out, None)
        if rc != 0:
            raise RuntimeError(f"hl_plain returned {rc}")
    descs = (_lib.hl_image_desc * 1)(desc)
    cnt = (C.c_int * 1)()
    hl.set_batch_graph(True)

    def batched():
        rc = L.hl_batch(hl.handle, descs, 1, None, 16, out, cnt, None)
        if rc != 0:
            raise RuntimeError(f"hl_batch returned {rc}")

    def wall(f):
        for _ in range(20):
            f()
        t0 = time.perf_counter()
        for _ in range(reps):
            f()
        return (time.perf_counter() - t0) / reps * 1e6
    return {"workload": "plain HoughLine 512x512, T=180, R=1449, thr 100, top-16 "
                        "(image on the device, lines to the host, synchronous)",
            "hl_plain_us_per_image": wall(plain),
            "hl_batch_graph_us_per_image": wall(batched), "calls": reps}


def gpu_scenes(L, Image, dev, kind: int, n: int, seed: int):
    """n seeded scenes of a workload spec generated on the GPU (the same
    bytes as the host generator), each in its own pitched buffer."""
    import torch
    _lib = _lib_mod()
    ps = (_lib.hl_scene_params * n)()
    _lib.check(L.hl_synth_spec(kind, seed, n, ps), "hl_synth_spec")
    imgs, descs = [], (_lib.hl_image_desc * n)()
    for i in range(n):
        w, h = ps[i].width, ps[i].height
        pitch = (w + 511) // 512 * 512
        buf = torch.empty((h, pitch), dtype=torch.uint8, device=dev)
        descs[i] = _lib.hl_image_desc(buf.data_ptr(), pitch, w, h, 0, 0, w, h)
        im = Image(buf[:, :w])
        im._buf = buf
        imgs.append(im)
    _lib.check(L.hl_synth_scenes_device(ps, n, descs, None), "hl_synth_scenes_device")
    return imgs


def proposal_selection():
    """The calibrated selection settings saved beside the network weights."""
    from opencuda_gb300.proposal import WEIGHTS
    p = WEIGHTS.with_name("proposal_selection.json")
    return json.loads(p.read_text())


def proposal_workload(L, HoughLine, Image, dev, sp, kind: int, n: int, reps: int,
                      check_counts: bool):
    """Proposal-guided batched HoughLine against the plain batched path on
    the same images: spec 4 = 2048 x 2048 scenes (8-48 segments, 1-4% noise),
    spec 5 = uneven 512-4096 scenes, 30% cluttered.  Theta step 0.5 deg,
    threshold 0.15 * max(w, h), top-32.  Two operating points: `calibrated`
    (local maxima of the coarse heatmap, the 64 best grown by one cell, and
    the confidence fall-back whose threshold was calibrated on held-out
    scenes for 99% top-32 recall) and `no_fallback` (the same selection, no
    fall-back).  Timed with CUDA events around whole batch calls through the
    C ABI, device buffers made once, like the plain call (the proposal call
    synchronises once to decide its fall-back set); recall =
    plain top-32 lines the proposal path also reports, over all images.
    With check_counts, every line the calibrated run reports is checked
    against the plain accumulator of its image (untimed)."""
    import torch
    from opencuda_gb300.proposal import WEIGHTS, HoughNet, proposal_batch
    K, det = 32, math.pi / 360
    imgs = gpu_scenes(L, Image, dev, kind, n, 4321 + kind)
    thr = [int(0.15 * max(im.width, im.height)) for im in imgs]
    hl = HoughLine(detheta=det)
    hl.set_batch_graph(True)
    net = HoughNet()
    net.load(WEIGHTS)
    sel = proposal_selection()
    sel = dict(sel, **sel.get("per_spec", {}).get(str(kind), {}))
    _lib = _lib_mod()
    descs = (_lib.hl_image_desc * n)(*[d.desc() for d in imgs])
    th = (C.c_int * n)(*thr)
    lines = torch.empty(n * K * 3, dtype=torch.int32, device=dev)
    counts = torch.zeros(n, dtype=torch.int32, device=dev)
    base = dict(p_cut=sel["p_cut"], max_props=sel["max_props"], dilate_theta=sel["dilate_theta"],
                dilate_rho=sel["dilate_rho"], top_m=sel["top_m"], nms=bool(sel["nms"]))
    points = {"calibrated": dict(base, p_conf=sel["p_conf"]),
              "no_fallback": dict(base, p_conf=0.0, max_props=90 * 128)}

    def plain():
        rc = L.hl_batch_async(hl.handle, descs, n, th, K, C.c_void_p(lines.data_ptr()),
                              C.c_void_p(counts.data_ptr()), sp)
        if rc != 0:
            raise RuntimeError(f"hl_batch_async returned {rc}")

    def timed(f):
        for _ in range(2):
            f()
        torch.cuda.synchronize(dev)
        ms = []
        for _ in range(reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            f()
            e1.record()
            torch.cuda.synchronize(dev)
            ms.append(e0.elapsed_time(e1))
        return statistics.median(ms)
    t_plain = timed(plain)
    out = {"workload": ("proposal-guided vs plain batched HoughLine: "
                        + ("2048x2048 scenes, 8-48 segments, 1-4% noise" if kind == 4 else
                           "uneven 512-4096 scenes, 30% cluttered")
                        + f", {n} images, T=360, thr 0.15*max(w,h), top-32"),
           "images": n, "plain_images_per_s": n / (t_plain / 1e3),
           "network": sel.get("network", ""), "selection": base,
           "calibration": sel.get("calibration")}
    for name, opts in points.items():
        # timed through the C ABI like the plain call (device buffers made
        # once, no statistics counted); the Python wrapper below, untimed,
        # gives the lines and the statistics
        copts = _lib.hl_proposal_opts(opts["p_cut"], opts["max_props"], opts["dilate_theta"],
                                      opts["dilate_rho"], 0, opts["top_m"],
                                      1 if opts["nms"] else 0, opts["p_conf"])

        def prop(copts=copts):
            rc = L.hl_proposal_batch(hl.handle, net.handle, descs, n, th, K, C.byref(copts),
                                     C.c_void_p(lines.data_ptr()),
                                     C.c_void_p(counts.data_ptr()), None, sp)
            if rc != 0:
                raise RuntimeError(f"hl_proposal_batch returned {rc}")
        t_prop = timed(prop)
        rc, got, st = proposal_batch(hl, net, imgs, K, thr, stream=sp, judge_every=1, **opts)
        if rc != 0:
            raise RuntimeError(f"hl_proposal_batch returned {rc}")
        out[name] = {"p_conf": opts["p_conf"], "images_per_s": n / (t_prop / 1e3),
                     "speedup_vs_plain": t_plain / t_prop,
                     "recall_top32": st["judged_found"] / max(st["judged_lines"], 1),
                     "fallback_rate": st["fallback"] / n,
                     "fallback_confidence": st["fallback_conf"] / n,
                     "windows_per_image": st["windows"] / n,
                     "cells_per_image": st["cells"] / n,
                     "executed_votes_per_image": st["votes"] / n}
        if check_counts and name == "calibrated":
            # every reported line is a peak bin of the plain accumulator with
            # its exact count (the reference decode reports negative rho
            # bins one higher, so d <= 0 may stand for bin d or d - 1)
            bad = checked = 0
            for i, im in enumerate(imgs):
                if not got[i]:
                    continue
                acc, rho_min = hl.accumulator(im)
                R = acc.shape[0]
                ks = [int(round(ln.angle / det)) for ln in got[i]]
                r0 = [min(max(ln.distance - rho_min, 0), R - 1) for ln in got[i]]
                r1 = [min(max(ln.distance - 1 - rho_min, 0), R - 1) for ln in got[i]]
                kt = torch.tensor(ks, device=dev)
                v0 = acc[torch.tensor(r0, device=dev), kt].tolist()
                v1 = acc[torch.tensor(r1, device=dev), kt].tolist()
                for q, ln in enumerate(got[i]):
                    ok = (0 <= ln.distance - rho_min < R and v0[q] == ln.votes) or \
                         (ln.distance <= 0 and 0 <= ln.distance - 1 - rho_min < R and
                          v1[q] == ln.votes)
                    bad += not ok
                    checked += 1
                del acc
            out[name]["exact_counts"] = {"lines_checked": checked, "mismatches": bad,
                                         "images": n}
    return out


def proposal_single_image(L, HoughLine, Image, dev, sp, reps: int):
    """The single-image learned-proposal configuration: one 2048 x 2048 scene
    (8-48 segments, 1-4% noise).  Device time (CUDA events) of the network
    forward alone (occupancy map in HBM) and wall time of one synchronous
    proposal-guided call (calibrated selection) against hl_plain on the same
    image."""
    import torch
    from opencuda_gb300.proposal import WEIGHTS, HoughNet, proposal_batch
    K, det = 32, math.pi / 360
    img = gpu_scenes(L, Image, dev, 4, 1, 4325)
    thr = [int(0.15 * max(img[0].width, img[0].height))]
    hl = HoughLine(detheta=det)
    net = HoughNet()
    net.load(WEIGHTS)
    sel = proposal_selection()
    sel = dict(sel, **sel.get("per_spec", {}).get("4", {}))
    opts = dict(p_cut=sel["p_cut"], max_props=sel["max_props"], dilate_theta=sel["dilate_theta"],
                dilate_rho=sel["dilate_rho"], top_m=sel["top_m"], nms=bool(sel["nms"]),
                p_conf=sel["p_conf"])
    occ, geo = net.occupancy(hl, img)
    fs = torch.cuda.Stream(dev)
    for _ in range(5):
        net.forward(occ, geo, stream=fs)
    torch.cuda.synchronize(dev)
    ms = []
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(fs)
        net.forward(occ, geo, stream=fs)
        e1.record(fs)
        fs.synchronize()
        ms.append(e0.elapsed_time(e1))

    def wall(f):
        for _ in range(5):
            f()
        t0 = time.perf_counter()
        for _ in range(reps):
            f()
        return (time.perf_counter() - t0) / reps * 1e6
    hl.setThreshold(thr[0])
    plain_us = wall(lambda: hl.houghLine(img[0], None, K))
    prop_us = wall(lambda: proposal_batch(hl, net, img, K, thr, stream=sp, **opts))
    rc, _, st = proposal_batch(hl, net, img, K, thr, stream=sp, **opts)
    return {"workload": "learned proposal, one 2048x2048 scene (8-48 segments, 1-4% noise), "
                        "T=360, top-32", "network_forward_us": statistics.median(ms) * 1e3,
            "proposal_call_us": prop_us, "hl_plain_us": plain_us,
            "fell_back": bool(st.get("fallback", 0)), "calls": reps,
            "timing": "network: CUDA events, device time; calls: host wall time, synchronous"}


def circle_workload(L, Image, dev, sp, atom_peak: float, reps: int, cpu: bool):
    """HoughCircle::houghcircle at the reference's default parameters (radii
    5-50, distThres 50, rThres 20, cirThreshold 100), circleMax 32, on a
    1024 x 1024 scene of 24 rings (radii 8-50) and 1% salt.  Device: CUDA
    events around the synchronous hl_circles call (compaction, tile vote +
    local maxima, tail, result copy) with the image resident and L2 flushed
    between calls.  e2e: host wall time from the host image (pinned) through
    the upload, hl_circles and the circles on the host.  The votes are the
    accumulator's sum (the in-ROI midpoint votes), counted once untimed."""
    import torch
    import cases
    from opencuda_gb300.houghcircle import HoughCircle
    from oracle import oracle as O
    host = cases.circle_scene(1024, 1024, 24, 8, 50, 10000, 77)
    h, w = host.shape
    img = Image.from_host(host, device=dev)
    pinned = torch.from_numpy(host).pin_memory()
    hc = HoughCircle()
    cm = 32
    votes = int(hc.accumulator(img, stream=sp).sum().item())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    for _ in range(3):
        rc, got = hc.houghcircle(img, None, cm, stream=sp)
    if rc != 0:
        raise RuntimeError(f"hl_circles returned {rc}")
    torch.cuda.synchronize(dev)
    ms = []
    for _ in range(reps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        hc.houghcircle(img, None, cm, stream=sp)
        e1.record()
        torch.cuda.synchronize(dev)
        ms.append(e0.elapsed_time(e1))
    t = statistics.median(ms)
    dst = img.data
    e2e = []
    for _ in range(reps):
        flush.zero_()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        dst.copy_(pinned, non_blocking=True)
        rc, got = hc.houghcircle(img, None, cm, stream=sp)
        e2e.append((time.perf_counter() - t0) * 1e3)
    te = statistics.median(e2e)
    out = {"workload": "HoughCircle 1024x1024, 24 rings r 8-50 + 1% salt, radii 5-50, "
                       "distThres 50, rThres 20, cirThreshold 100, circleMax 32",
           "value": 1e3 / t, "unit": "images/s", "ms_per_image": t,
           "e2e": {"value": 1e3 / te, "unit": "images/s", "ms_per_image": te,
                   "h2d_bytes_per_step": int(host.nbytes),
                   "d2h_bytes_per_step": 16 * (cm + 1)},
           "edge_pixels": int((host == 255).sum()), "votes": votes, "circles": len(got),
           "roofline": {"bound": "smem_atomic", "achieved": votes / (t / 1e3) / 1e12,
                        "peak": atom_peak / 1e12, "unit": "T atomics/s",
                        "frac": votes / (t / 1e3) / atom_peak,
                        "note": "whole call (all launches and the result copy) as the time"},
           "reps": reps, "l2": "flushed between calls"}
    # pieceCircle: 4 x 4 pieces of the same scene as one hl_circles_batch call,
    # against the pieces looped through hl_circles
    pieces = []
    for y in range(4):
        for x in range(4):
            pieces.append(Image(img.data, (x * 256, y * 256, x * 256 + 255, y * 256 + 255)))
    for _ in range(3):
        hc.houghcircleBatch(pieces, 10, stream=sp)
    bt, lt = [], []
    for _ in range(reps):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        rc, _ = hc.houghcircleBatch(pieces, 10, stream=sp)
        bt.append((time.perf_counter() - t0) * 1e3)
        t0 = time.perf_counter()
        for pc in pieces:
            hc.houghcircle(pc, None, 10, stream=sp)
        lt.append((time.perf_counter() - t0) * 1e3)
    if rc != 0:
        raise RuntimeError(f"hl_circles_batch returned {rc}")
    out["pieces"] = {"workload": "pieceCircle 4 x 4 of the same scene (256 x 256 pieces, "
                                 "ROI [x*c, x*c + c - 1)), 10 circles per piece",
                     "batch_ms": statistics.median(bt), "loop_ms": statistics.median(lt),
                     "timing": "host wall time of synchronous calls, image resident"}
    if cpu:
        t0 = time.perf_counter()
        want, _ = O.houghcircle(host, 5, 50, 100, 50.0, 20, cm)
        tc = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": 1 / tc, "unit": "images/s", "cores": O.max_threads(),
                               "kind": "port",
                               "sample": "1 image through the C restatement (vote with OpenMP "
                                         "over radii, local maxima, sort, merge)"}
        out["matches_oracle"] = [c.astuple() for c in got] == list(want)
    return out


def _lib_mod():
    from opencuda_gb300 import _lib
    return _lib


def run_reference(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return 0
    from opencuda_gb300 import build
    build.build_oracle()
    imgs = make_images(0, 2)
    for _ in range(max(args.warmup, 0)):
        cpu_reference_images(imgs, 0.0)
    n, el, votes, cores = cpu_reference_images(imgs, 0.0, min_images=args.steps)
    ips = n / el
    line = {"impl": "reference", "metric": METRIC, "value": ips, "unit": "images/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": el / n * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int32 votes, f32 rho", "data": "synthetic",
            "gvotes_per_s": votes / el / 1e9,
            "config": bench_config(args.gpus),
            "cpu_baseline": {"value": ips, "unit": "images/s", "cores": cores, "kind": "port",
                             "sample": f"{n} full 4096x4096 images (vote + peaks + host tail), "
                                       "OpenMP over theta columns"},
            "e2e": {"value": ips, "unit": "images/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_gb300(args):
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    from opencuda_gb300 import _lib, build
    build.build_library()
    L = _lib.load()
    from opencuda_gb300.houghline import HoughLine, Image

    if args.circle_only:
        stream = torch.cuda.current_stream(dev)
        sp = C.c_void_p(stream.cuda_stream)
        atom = C.c_double()
        _lib.check(L.hl_measure_smem_atomic_peak(2000, C.byref(atom), sp), "atomic peak")
        out = circle_workload(L, Image, dev, sp, atom.value, max(args.steps, 5),
                              ws == 1 and not args.no_cpu_baseline)
        if rank == 0:
            print(json.dumps({"circle": out}))
        return 0

    if args.proposal_only:
        stream = torch.cuda.current_stream(dev)
        sp = C.c_void_p(stream.cuda_stream)
        out = {"proposal": [proposal_workload(L, HoughLine, Image, dev, sp, 4, 128, 5, False),
                            proposal_workload(L, HoughLine, Image, dev, sp, 5, 1024, 3, True)],
               "proposal_single": proposal_single_image(L, HoughLine, Image, dev, sp, 50)}
        if rank == 0:
            print(json.dumps(out))
        return 0

    if args.batched_only:
        stream = torch.cuda.current_stream(dev)
        sp = C.c_void_p(stream.cuda_stream)
        atom = C.c_double()
        _lib.check(L.hl_measure_smem_atomic_peak(2000, C.byref(atom), sp), "atomic peak")
        out = batched_workload(L, HoughLine, Image, dev, sp, max(args.steps, 5), atom.value,
                               ws == 1 and not args.no_cpu_baseline)
        if rank == 0:
            print(json.dumps({"batched": out}))
        return 0

    imgs_host = make_images(rank, 4)
    hl = HoughLine(detheta=DETHETA, threshold=THRESHOLD)
    g = hl.geometry(W, H)
    T = g.numtheta
    dimgs = [Image.from_host(im, device=dev) for im in imgs_host]
    npts = [int((im == 255).sum()) for im in imgs_host]
    stream = torch.cuda.current_stream(dev)
    sp = C.c_void_p(stream.cuda_stream)
    lines_dev = torch.empty(LINESMAX * 3, dtype=torch.int32, device=dev)
    count_dev = torch.zeros(1, dtype=torch.int32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def step(i):
        d = dimgs[i % len(dimgs)].desc()
        rc = L.hl_plain_async(hl.handle, C.byref(d), LINESMAX,
                              C.c_void_p(lines_dev.data_ptr()),
                              C.c_void_p(count_dev.data_ptr()), sp)
        if rc != 0:
            raise RuntimeError(f"hl_plain_async returned {rc}")

    # warm-up (also grows the workspace once)
    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize(dev)
    st = C.c_int()
    _lib.check(L.hl_last_status(hl.handle, C.byref(st), sp), "hl_last_status")
    if st.value != 0:
        raise RuntimeError(f"device status {st.value}")
    launches_per_step = hl.last_launch_count()

    # shared-memory atomic ceiling of this GPU (micro-kernel)
    atom = C.c_double()
    _lib.check(L.hl_measure_smem_atomic_peak(2000, C.byref(atom), sp), "atomic peak")

    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    gpu_index = os.environ.get("CUDA_VISIBLE_DEVICES", str(local)).split(",")[local] \
        if os.environ.get("CUDA_VISIBLE_DEVICES") else str(local)
    clocks = NvmlClockSampler(dev)
    if clocks.h is None:
        clocks = ClockSampler(gpu_index)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    t_wall = time.perf_counter()
    for i in range(args.steps):
        flush.zero_()                       # L2 flush, outside the timed events
        evs[i][0].record(stream)
        step(i)
        evs[i][1].record(stream)
    torch.cuda.synchronize(dev)
    if ws > 1:
        torch.distributed.barrier()
    t_wall = time.perf_counter() - t_wall
    ck = clocks.stop()
    dev_ms = sum(a.elapsed_time(b) for a, b in evs)
    # per-stage times in a separate pass: the stage events sit between the
    # kernels, where they would keep each kernel from launching while its
    # predecessor drains, so they stay out of the timed steps
    stage = (C.c_double * 4)()
    calls = C.c_int()
    _lib.check(L.hl_profile(hl.handle, 1), "hl_profile")
    for i in range(min(args.steps, 100)):
        flush.zero_()
        step(i)
    torch.cuda.synchronize(dev)
    _lib.check(L.hl_profile_read(hl.handle, stage, C.byref(calls)), "hl_profile_read")
    L.hl_profile(hl.handle, 0)
    votes = sum(npts[i % len(npts)] * T for i in range(args.steps))
    # e2e through the public API, pipelined: every step copies its image from
    # pinned host memory (upload stream) and reads its line count and lines
    # back to pinned host memory (read-back stream); two device image buffers
    # and two device result buffers let the upload of step i+1 and the
    # read-back of step i overlap the kernels.  Timed from the first copy to the
    # last read-back, on the device.
    pinned = [torch.from_numpy(im).pin_memory() for im in imgs_host]
    copy_stream = torch.cuda.Stream(dev)   # uploads
    back_stream = torch.cuda.Stream(dev)   # read-backs (in order behind their pipelines)
    stg = [torch.empty((H, W), dtype=torch.uint8, device=dev) for _ in range(2)]
    stg_img = [Image(t) for t in stg]
    ready = [torch.cuda.Event() for _ in range(2)]     # image b uploaded
    done = [torch.cuda.Event() for _ in range(2)]      # pipeline of buffer b finished
    fetched = [torch.cuda.Event() for _ in range(2)]   # results of buffer b read back
    # results: LINESMAX records then the count, one read-back per step
    res_dev = [torch.empty(LINESMAX * 3 + 1, dtype=torch.int32, device=dev) for _ in range(2)]
    res_host = [torch.empty(LINESMAX * 3 + 1, dtype=torch.int32).pin_memory() for _ in range(2)]

    def e2e_run(nsteps, start_ev=None):
        for i in range(nsteps):
            b = i % 2
            with torch.cuda.stream(copy_stream):
                if start_ev is not None and i == 0:
                    copy_stream.wait_event(start_ev)
                if i >= 2:
                    copy_stream.wait_event(done[b])
                stg[b].copy_(pinned[i % len(pinned)], non_blocking=True)
                ready[b].record(copy_stream)
            stream.wait_event(ready[b])
            if i >= 2:
                stream.wait_event(fetched[b])
            d = stg_img[b].desc()
            rc = L.hl_plain_async(hl.handle, C.byref(d), LINESMAX,
                                  C.c_void_p(res_dev[b].data_ptr()),
                                  C.c_void_p(res_dev[b].data_ptr() + 4 * LINESMAX * 3), sp)
            if rc != 0:
                raise RuntimeError(f"hl_plain_async returned {rc}")
            done[b].record(stream)
            with torch.cuda.stream(back_stream):
                back_stream.wait_event(done[b])
                res_host[b].copy_(res_dev[b], non_blocking=True)
                fetched[b].record(back_stream)

    e2e_run(args.warmup)
    torch.cuda.synchronize(dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    e2e_run(args.steps, start_ev=e0)
    stream.wait_stream(back_stream)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    e2e_ms = e0.elapsed_time(e1)
    _lib.check(L.hl_last_status(hl.handle, C.byref(st), sp), "hl_last_status")
    if st.value != 0:
        raise RuntimeError(f"device status {st.value} in the end-to-end run")
    # the last step's read-back equals the same image through the device path
    last = args.steps - 1
    chk = torch.empty(LINESMAX * 3 + 1, dtype=torch.int32, device=dev)
    d = dimgs[last % len(dimgs)].desc()
    _lib.check(L.hl_plain_async(hl.handle, C.byref(d), LINESMAX, C.c_void_p(chk.data_ptr()),
                                C.c_void_p(chk.data_ptr() + 4 * LINESMAX * 3), sp),
               "hl_plain_async")
    torch.cuda.synchronize(dev)
    got, want = res_host[last % 2], chk.cpu()
    n = int(want[-1])
    if int(got[-1]) != n or not torch.equal(got[:3 * min(n, LINESMAX)], want[:3 * min(n, LINESMAX)]):
        raise RuntimeError("end-to-end read-back differs from the device path")

    dev_ms, e2e_ms, vote_ms, votes_all = reduce_over_ranks(
        [dev_ms, e2e_ms, stage[1]], float(votes), ws, dev)
    if rank != 0:
        if ws > 1:
            torch.distributed.destroy_process_group()
        return 0

    images = args.steps * ws
    value = images / (dev_ms / 1e3)
    peaks, peak_kind = measured_peaks()
    n_avg = sum(npts[i % len(npts)] for i in range(args.steps)) / args.steps
    vote_launch_s = vote_ms / 1e3 / max(calls.value, 1)
    atomics_per_launch = n_avg * T
    achieved_atom = atomics_per_launch / vote_launch_s
    b_alg_step = W * H + 4.0 * T * g.numrho          # image once + accumulator once
    pipe_s = dev_ms / 1e3 / args.steps
    hbm_gbs = b_alg_step / pipe_s / 1e9
    traffic = ncu_traffic()
    line = {
        "metric": METRIC, "value": value, "unit": "images/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "int32 votes, f32 rho (bit-exact)", "data": "synthetic",
        "gvotes_per_s": votes_all / (dev_ms / 1e3) / 1e9,
        "config": bench_config(ws),
        "edge_points_avg": n_avg,
        "stage_ms_avg": {"compact": stage[0] / max(calls.value, 1),
                         "vote": stage[1] / max(calls.value, 1),
                         "peaks": stage[2] / max(calls.value, 1),
                         "finalize": stage[3] / max(calls.value, 1)},
        "roofline": {"kernel": "hl_vote_kernel", "bound": "smem_atomic",
                     "achieved": achieved_atom / 1e9, "peak": atom.value / 1e9,
                     "unit": "Gatomic/s", "frac": achieved_atom / atom.value,
                     "peak_source": "measured on this GPU: conflict-free shared int32 atomicAdd micro-kernel",
                     "units_per_launch": atomics_per_launch,
                     "traffic": traffic,
                     "hbm": {"achieved": hbm_gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                             "frac": hbm_gbs / peaks["hbm_gbs"], "peak_source": peak_kind,
                             "bytes_per_step": b_alg_step, "scope": "whole pipeline"}},
        "e2e": {"value": images / (e2e_ms / 1e3), "unit": "images/s",
                "h2d_bytes_per_step": W * H,
                "d2h_bytes_per_step": 4 + 12 * LINESMAX,
                "pipeline": "upload and read-back streams, 2 device image and 2 device result buffers: the "
                            "H2D of step i+1 and the D2H of step i overlap the kernels; "
                            "no L2 flush (each image arrives by H2D)"},
        "gpu_launches": launches_per_step * args.steps,
        "clocks": ck,
        "wall_s_timed_loop": t_wall,
    }
    line["latency_512"] = latency_512(L, HoughLine, Image, dev)
    if not args.no_batch:
        line["batched"] = batched_workload(L, HoughLine, Image, dev, sp, min(max(args.steps, 5), 50),
                                           atom.value, ws == 1 and not args.no_cpu_baseline)
    if not args.no_batch and not args.no_proposal:
        line["proposal"] = [proposal_workload(L, HoughLine, Image, dev, sp, 4, 128, 5, False),
                            proposal_workload(L, HoughLine, Image, dev, sp, 5, 1024, 3, True)]
        line["proposal_single"] = proposal_single_image(L, HoughLine, Image, dev, sp, 50)
    if not args.no_circle:
        line["circle"] = circle_workload(L, Image, dev, sp, atom.value,
                                         min(max(args.steps, 5), 50),
                                         ws == 1 and not args.no_cpu_baseline)
    if ws == 1 and not args.no_cpu_baseline:
        n, el, v, cores = cpu_reference_images(imgs_host, args.cpu_budget)
        line["cpu_baseline"] = {"value": n / el, "unit": "images/s", "cores": cores,
                                "kind": "port", "gvotes_per_s": v / el / 1e9,
                                "sample": f"{n} full 4096x4096 images through the C "
                                          "transcription of the reference vote loop + "
                                          "host tail, OpenMP over theta columns"}
    else:
        line["cpu_baseline"] = None
    print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-budget", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true",
                    help="skip the batched (256 uneven images) measurement")
    ap.add_argument("--no-circle", action="store_true",
                    help="skip the HoughCircle measurement")
    ap.add_argument("--circle-only", action="store_true",
                    help="only the HoughCircle measurement (its own JSON line)")
    ap.add_argument("--batched-only", action="store_true",
                    help="only the batched 256-image measurement (its own JSON line)")
    ap.add_argument("--no-proposal", action="store_true",
                    help="skip the proposal-guided measurements")
    ap.add_argument("--proposal-only", action="store_true",
                    help="only the proposal-guided measurements (their own JSON line)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gb300":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
