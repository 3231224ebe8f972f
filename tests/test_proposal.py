"""GPU checks of the proposal-guided path's exactness: with every coarse cell
proposed it must reproduce the plain method bit for bit (window votes, peak
rule, ranking and merge); with the fall-back forced it is the plain method;
the judged recall counts agree."""
import math

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu
DEG05 = math.pi / 360


@pytest.fixture(scope="module")
def env(cuda):
    from opencuda_gb300.houghline import HoughLine, Image
    from opencuda_gb300.proposal import HoughNet, proposal_batch
    return HoughLine, Image, HoughNet, proposal_batch


def _images(Image, n=3, seed=21):
    imgs = [cases.synth(3, seed, i) for i in range(n)]
    imgs.append(cases.synth(1, 5, 0))
    return imgs, [Image.from_host(im) for im in imgs]


def _plain(HoughLine, dev, thr, K):
    hl = HoughLine(detheta=DEG05)
    rc, res = hl.houghLineBatch(dev, K, thr)
    assert rc == 0
    return [[l.astuple() for l in r] for r in res]


def test_all_cells_proposed_equals_plain(env):
    HoughLine, Image, HoughNet, proposal_batch = env
    imgs, dev = _images(Image)
    thr = [int(0.15 * max(im.shape)) for im in imgs]
    want = _plain(HoughLine, dev, thr, 24)
    hl = HoughLine(detheta=DEG05)
    net = HoughNet(seed=3)
    rc, got, st = proposal_batch(hl, net, dev, 24, thr, p_cut=1e-6, max_props=90 * 128,
                                 dilate_rho=0, judge_every=1)
    assert rc == 0 and st["fallback"] == 0
    assert [[l.astuple() for l in r] for r in got] == want
    assert st["judged"] == len(imgs) and st["judged_found"] == st["judged_lines"]
    assert st["windows"] == len(imgs) * 90 * 128


def test_forced_fallback_is_plain(env):
    HoughLine, Image, HoughNet, proposal_batch = env
    imgs, dev = _images(Image, n=2, seed=8)
    thr = [int(0.15 * max(im.shape)) for im in imgs]
    want = _plain(HoughLine, dev, thr, 16)
    hl = HoughLine(detheta=DEG05)
    net = HoughNet(seed=4)
    rc, got, st = proposal_batch(hl, net, dev, 16, thr, p_cut=1e-6, max_props=0)
    assert rc == 0 and st["fallback"] == len(imgs)
    assert [[l.astuple() for l in r] for r in got] == want


def test_reported_lines_carry_exact_votes(env):
    """With few proposals, every reported line is a peak of the full
    accumulator with its exact count."""
    HoughLine, Image, HoughNet, proposal_batch = env
    imgs, dev = _images(Image, n=2, seed=13)
    thr = [int(0.15 * max(im.shape)) for im in imgs]
    hl = HoughLine(detheta=DEG05)
    net = HoughNet(seed=5)
    rc, got, st = proposal_batch(hl, net, dev, 16, thr, p_cut=0.02, max_props=400)
    assert rc == 0
    for i, (im, d) in enumerate(zip(imgs, dev)):
        if not got[i]:
            continue
        acc, rho_min = hl.accumulator(d)
        a = acc.cpu().numpy()
        T = a.shape[1]
        for ln in got[i]:
            k = int(round(ln.angle / DEG05))
            # the reference decode reports negative rho bins one higher
            cand = [ln.distance - rho_min, ln.distance - 1 - rho_min]
            assert any(0 <= j < a.shape[0] and a[j, k] == ln.votes for j in cand), (i, ln)
