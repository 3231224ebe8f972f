"""Train the proposal network on the GPU with the project's own kernels.

    python -m opencuda_gb300.train_proposal --images 200000 --out weights.npy

Every batch is generated on the GPU (hl_synth_scenes_device, seeded scenes:
three quarters 2048 x 2048 images with 8-48 segments and 1-4% noise, one
quarter uneven 512-4096 images of which 30% are cluttered), labelled by the
plain method itself (hl_batch: the top-32 lines per image, threshold
0.15 * max(w, h), theta step 0.5 deg), pooled to 256 x 256 occupancy maps and
fed to hl_net_train_step (forward and backward kernels of hl_cnn.cu, Adam).
Labels come only from the plain method; the images never leave the GPU,
only the line lists that the coarse targets are built from.

After training, a held-out set calibrates the confidence fall-back
(--calibrate N: the threshold that brings the top-32 recall, fall-backs
included, to 99%) and measures the top-32 recall of the proposal-guided path
against the plain method for a grid of selection settings (one JSON line
per setting).
"""
from __future__ import annotations

import argparse
import json
import math
import sys
import time

import numpy as np

from . import _lib
from .houghline import HoughLine, Image
from .proposal import HoughNet, line_targets, proposal_batch

DET = math.pi / 360
K = 32


class SceneGen:
    """GPU scene batches in pitched device buffers reused across calls."""

    def __init__(self, maxside: int = 4096, batch: int = 32):
        import torch
        self.L = _lib.load()
        self.pitch = (maxside + 511) // 512 * 512
        self.buf = torch.empty((batch, maxside, self.pitch), dtype=torch.uint8, device="cuda")
        self.batch = batch

    def make(self, specs):
        n = len(specs)
        assert n <= self.batch
        ps = (_lib.hl_scene_params * n)(*specs)
        descs = (_lib.hl_image_desc * n)()
        imgs = []
        for i, p in enumerate(specs):
            descs[i] = _lib.hl_image_desc(self.buf[i].data_ptr(), self.pitch, p.width,
                                          p.height, 0, 0, p.width, p.height)
            imgs.append(Image(self.buf[i, : p.height, : p.width]))
        _lib.check(self.L.hl_synth_scenes_device(ps, n, descs, None), "hl_synth_scenes_device")
        return imgs


def specs_for(seed: int, start: int, n: int, frac_2048: float = 0.75):
    """Scene parameters of images start .. start + n - 1 of a run: the batch's
    own seed (seed, start) draws n scenes of each kind and a seeded coin per
    image picks the kind, so every (seed, index) names one scene."""
    L = _lib.load()
    bseed = (seed * 1000003 + start) & 0xFFFFFFFFFFFF
    s4 = (_lib.hl_scene_params * n)()
    s5 = (_lib.hl_scene_params * n)()
    _lib.check(L.hl_synth_spec(4, bseed, n, s4))
    _lib.check(L.hl_synth_spec(5, bseed, n, s5))
    rng = np.random.default_rng(bseed)
    return [s4[i] if rng.random() < frac_2048 else s5[i] for i in range(n)]


def thresholds(imgs):
    return [int(0.15 * max(im.width, im.height)) for im in imgs]


def train(args) -> HoughNet:
    import torch
    hl = HoughLine(detheta=DET)
    net = HoughNet(seed=args.seed)
    gen = SceneGen(batch=args.batch)
    steps = max(1, args.images // args.batch)
    t0 = time.time()
    losses = []
    for step in range(steps):
        imgs = gen.make(specs_for(args.seed, step * args.batch, args.batch))
        rc, lines = hl.houghLineBatch(imgs, K, thresholds(imgs))
        _lib.check(rc, "hl_batch")
        occ, geo = net.occupancy(hl, imgs)
        tgt = torch.from_numpy(line_targets(lines, geo)).cuda()
        lr = args.lr * (0.5 * (1 + math.cos(math.pi * step / steps)))   # cosine decay
        losses.append(net.train_step(occ, geo, tgt, lr, args.pos_weight))
        if step % max(1, steps // 20) == 0 or step == steps - 1:
            print(json.dumps({"step": step, "images": (step + 1) * args.batch,
                              "loss": float(np.mean(losses[-50:])), "lr": lr,
                              "s": round(time.time() - t0, 1)}), flush=True)
    return net


def evaluate(net: HoughNet, n: int, seed: int, settings, frac_2048: float = 0.75):
    """Top-32 recall and fall-back rate on held-out scenes per setting:
    (p_cut, max_props, dilate_theta, dilate_rho, top_m)."""
    hl = HoughLine(detheta=DET)
    gen = SceneGen(batch=32)
    rows = []
    for (p_cut, max_props, dt, dr, top_m) in settings:
        found = total = fb = wins = votes = 0
        for start in range(0, n, 32):
            imgs = gen.make(specs_for(seed, start, min(32, n - start), frac_2048))
            rc, _, st = proposal_batch(hl, net, imgs, K, thresholds(imgs), p_cut=p_cut,
                                       max_props=max_props, dilate_theta=dt, dilate_rho=dr,
                                       judge_every=1, top_m=top_m, nms=True)
            _lib.check(rc, "hl_proposal_batch")
            found += st["judged_found"]
            total += st["judged_lines"]
            fb += st["fallback"]
            wins += st["windows"]
            votes += st["votes"]
        rows.append({"p_cut": p_cut, "max_props": max_props, "dilate_theta": dt,
                     "dilate_rho": dr, "top_m": top_m, "recall": found / max(total, 1),
                     "fallback_rate": fb / n, "windows_per_image": wins / n,
                     "votes_per_image": votes / n, "images": n})
        print(json.dumps(rows[-1]), flush=True)
    return rows


def selection_confidence(net: HoughNet, hl, imgs, top_m: int):
    """Per image, the logit of the best local maximum of the coarse heatmap
    that a top_m selection leaves out (-inf when there is none): the value
    hl_proposal_batch's confidence test compares with logit(p_conf)."""
    import torch
    import torch.nn.functional as F
    occ, geo = net.occupancy(hl, imgs)
    z = net.forward(occ, geo)
    mx = F.max_pool2d(F.pad(z[:, None], (1, 1, 1, 1), value=-1e30), 3, 1)[:, 0]
    cand = torch.where(z >= mx, z, torch.full_like(z, -3e38)).reshape(len(imgs), -1)
    k = min(top_m + 1, cand.shape[1])
    return torch.topk(cand, k, dim=1).values[:, -1].cpu().numpy()


def calibrate(net: HoughNet, n: int, seed: int, top_m: int, dilate_theta: int,
              dilate_rho: int, target: float = 0.99, frac_2048: float = 0.75) -> dict:
    """Choose the confidence threshold on held-out scenes: run the proposal
    path with the confidence test off, record each image's top-32 recall
    against the plain method and its confidence value, then take the
    highest threshold whose fall-backs (recall 1 for those images) bring the
    overall recall to the target."""
    hl = HoughLine(detheta=DET)
    gen = SceneGen(batch=32)
    conf, found, lines = [], [], []
    for start in range(0, n, 32):
        imgs = gen.make(specs_for(seed, start, min(32, n - start), frac_2048))
        thr = thresholds(imgs)
        rc, plain = hl.houghLineBatch(imgs, K, thr)
        _lib.check(rc, "hl_batch")
        rc, prop, st = proposal_batch(hl, net, imgs, K, thr, p_cut=0.9, max_props=400,
                                      dilate_theta=dilate_theta, dilate_rho=dilate_rho,
                                      top_m=top_m, nms=True)
        _lib.check(rc, "hl_proposal_batch")
        conf.extend(selection_confidence(net, hl, imgs, top_m).tolist())
        for a, b in zip(plain, prop):
            got = {l.astuple() for l in b}
            lines.append(len(a))
            found.append(sum(l.astuple() in got for l in a))
    conf, found, lines = np.array(conf), np.array(found), np.array(lines)
    total = max(int(lines.sum()), 1)
    best = None
    for z in sorted(set(conf.tolist()), reverse=True) + [-3e38]:
        fb = conf >= z
        rec = (lines[fb].sum() + found[~fb].sum()) / total
        if rec >= target:
            best = (z, rec, float(fb.mean()))
            break
    z, rec, fbr = best if best else (-3e38, 1.0, 1.0)
    p = float(1.0 / (1.0 + math.exp(-z))) if z > -80 else 1e-6
    out = {"top_m": top_m, "dilate_theta": dilate_theta, "dilate_rho": dilate_rho, "nms": 1,
           "p_cut": 0.9, "max_props": 400, "p_conf": min(max(p, 1e-6), 0.999999),
           "calibration": {"images": int(n), "seed": seed, "frac_2048": frac_2048,
                           "target_recall": target,
                           "recall": float(rec), "fallback_rate": fbr,
                           "recall_without_fallback": float(found.sum() / total)}}
    print(json.dumps(out), flush=True)
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--images", type=int, default=200000)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--pos-weight", type=float, default=40.0)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--out", default=None)
    ap.add_argument("--eval", type=int, default=256)
    ap.add_argument("--weights", default=None,
                    help="skip training: load these weights (for --calibrate)")
    ap.add_argument("--calibrate", type=int, default=0,
                    help="held-out images for the confidence threshold (0: none)")
    ap.add_argument("--top-m", type=int, default=64)
    ap.add_argument("--dilate-theta", type=int, default=1)
    ap.add_argument("--dilate-rho", type=int, default=1)
    ap.add_argument("--selection-out", default=None,
                    help="write the calibrated selection settings (JSON) here")
    ap.add_argument("--frac-2048", type=float, default=0.75,
                    help="calibration scenes: fraction of 2048 x 2048 scenes (spec 4); "
                         "the rest uneven 512-4096 scenes, 30%% cluttered (spec 5)")
    args = ap.parse_args(argv)
    if args.weights:
        net = HoughNet()
        net.load(args.weights)
    else:
        net = train(args)
    if args.out:
        np.save(args.out, net.get_params())
    if args.calibrate > 0:
        sel = calibrate(net, args.calibrate, 77777, args.top_m, args.dilate_theta,
                        args.dilate_rho, frac_2048=args.frac_2048)
        if args.selection_out:
            with open(args.selection_out, "w") as f:
                json.dump(sel, f, indent=1)
    if args.eval > 0:
        settings = [(0.9, 400, 0, 1, 48), (0.9, 400, 0, 1, 64), (0.9, 400, 1, 1, 64),
                    (0.9, 400, 0, 1, 96), (0.9, 400, 1, 1, 96), (0.5, 600, 1, 1, 128)]
        evaluate(net, args.eval, 99991, settings)
    return 0


if __name__ == "__main__":
    sys.exit(main())
