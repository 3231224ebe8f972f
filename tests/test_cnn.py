"""GPU parity of the proposal network's tensor-core convolution against the
CPU oracle (oracle/cnn_oracle.py): BF16 operands, FP32 accumulation; outputs
rounded to BF16 must match the oracle within one BF16 step."""
import ctypes as C

import numpy as np
import pytest

from oracle import cnn_oracle as CO

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib(cuda):
    from opencuda_gb300 import _lib
    return _lib.load()


def _dev_bf16(torch, a):
    return torch.from_numpy(CO.bf16_bits(a).view(np.int16).copy()).cuda()


def _run_conv(lib, torch, x, w, bias, stride, relu, mode=0, out_hw=None):
    B, H, W, cin = x.shape
    cout = w.shape[0]
    dx = _dev_bf16(torch, x)
    dw = _dev_bf16(torch, w)
    db = torch.from_numpy(np.asarray(bias, np.float32)).cuda() if bias is not None else None
    if mode == 0:
        Ho, Wo = (H - 1) // stride + 1, (W - 1) // stride + 1
    else:
        Ho, Wo = 2 * H, 2 * W
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    if cout == 1 and mode == 0:
        y = torch.full((B, Ho, Wo), -7.0, dtype=torch.float32, device="cuda")
        rc = lib.hl_cnn_conv3x3(C.c_void_p(dx.data_ptr()), C.c_void_p(dw.data_ptr()),
                                C.c_void_p(db.data_ptr()) if db is not None else None,
                                None, C.c_void_p(y.data_ptr()), B, H, W, cin, cout, stride,
                                int(relu), mode, C.c_void_p(st.data_ptr()), None)
        assert rc == 0
        torch.cuda.synchronize()
        assert int(st.item()) == 0
        return y.cpu().numpy()[..., None]
    y = torch.full((B, Ho, Wo, 32), 12345, dtype=torch.int16, device="cuda")
    rc = lib.hl_cnn_conv3x3(C.c_void_p(dx.data_ptr()), C.c_void_p(dw.data_ptr()),
                            C.c_void_p(db.data_ptr()) if db is not None else None,
                            C.c_void_p(y.data_ptr()), None, B, H, W, cin, cout, stride,
                            int(relu), mode, C.c_void_p(st.data_ptr()), None)
    assert rc == 0
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    out = CO.from_bf16_bits(y.cpu().numpy().view(np.uint16))
    assert np.all(out[..., cout:] == 0.0)
    return out[..., :cout]


def _close(got, ref, bf16_out=True):
    ref = ref.astype(np.float32)
    if bf16_out:
        tol = np.abs(ref) * 2.0 ** -7 + 1e-5
    else:
        tol = np.abs(ref) * 1e-5 + 1e-4
    bad = np.abs(got - ref) > tol
    assert not bad.any(), (np.argwhere(bad)[:5], got[bad][:5], ref[bad][:5])


@pytest.mark.parametrize("cin,cout,stride,relu,B,H,W", [
    (32, 32, 1, True, 2, 37, 29),
    (32, 32, 2, False, 3, 33, 40),
    (1, 32, 2, True, 2, 64, 50),
    (1, 32, 1, False, 1, 17, 23),
])
def test_conv_forward(lib, cin, cout, stride, relu, B, H, W):
    import torch
    rng = np.random.default_rng(cin * 100 + stride + H)
    x = CO.bf16_round(rng.standard_normal((B, H, W, cin)).astype(np.float32))
    w = CO.bf16_round((rng.standard_normal((cout, 9 * cin)) * 0.2).astype(np.float32))
    bias = rng.standard_normal(cout).astype(np.float32) * 0.1
    got = _run_conv(lib, torch, x, w, bias, stride, relu)
    ref = CO.conv3x3(x, w, bias, stride, relu)
    _close(got, ref)


def test_conv_one_channel_output(lib):
    import torch
    rng = np.random.default_rng(5)
    x = CO.bf16_round(rng.standard_normal((2, 31, 26, 32)).astype(np.float32))
    w = CO.bf16_round((rng.standard_normal((1, 288)) * 0.1).astype(np.float32))
    got = _run_conv(lib, torch, x, w, np.array([0.25], np.float32), 1, False)
    ref = CO.conv3x3(x, w, [0.25], 1, False)
    _close(got, ref, bf16_out=False)


def test_conv_stride2_input_gradient(lib):
    import torch
    rng = np.random.default_rng(9)
    H, W = 34, 22          # forward input size (even)
    dy = CO.bf16_round(rng.standard_normal((2, H // 2, W // 2, 32)).astype(np.float32))
    w = CO.bf16_round((rng.standard_normal((32, 288)) * 0.2).astype(np.float32))
    wt = CO.transpose_weights(w)
    got = _run_conv(lib, torch, dy, wt, None, 2, False, mode=1)
    ref = CO.conv3x3_dx(dy, w, H, W, stride=2)
    _close(got, ref)


def test_conv_stride1_input_gradient_is_a_convolution():
    """dx of a stride-1 conv = conv with flipped, transposed weights (the
    identity the backward pass uses)."""
    rng = np.random.default_rng(2)
    dy = rng.standard_normal((1, 9, 7, 32))
    w = rng.standard_normal((32, 288))
    wf = w.reshape(32, 3, 3, 32)[:, ::-1, ::-1, :].reshape(32, 288)
    ref = CO.conv3x3_dx(dy, w, 9, 7, 1)
    got = CO.conv3x3(dy, CO.transpose_weights(wf))
    assert np.allclose(got, ref)


def _occ_problem(seed, B=2):
    rng = np.random.default_rng(seed)
    occ = np.zeros((B, 256, 256), np.float32)
    for b in range(B):
        for _ in range(6):       # a few lines of occupancy ~1/8
            y0, x0 = rng.integers(0, 256, 2)
            ang = rng.random() * np.pi
            for tt in range(-150, 150):
                y = int(y0 + tt * np.sin(ang))
                x = int(x0 + tt * np.cos(ang))
                if 0 <= y < 256 and 0 <= x < 256:
                    occ[b, y, x] = 0.125
        occ[b] += (rng.random((256, 256)) < 0.02) * 0.015625
    occ = CO.bf16_round(occ)
    geos = [(32.0, -2896.0, 128 / 5793.0, 64, 64), (16.0, -1448.0, 128 / 2897.0, 64, 50)][:B]
    return occ, geos


def test_network_forward_matches_oracle(lib):
    import torch
    from opencuda_gb300.proposal import HoughNet
    occ, geos = _occ_problem(3)
    net = HoughNet(seed=7)
    p = net.get_params()
    dev = _dev_bf16(torch, occ)
    z = net.forward(dev, HoughNet.geos(geos)).cpu().numpy()
    zr, H, e, acts, bins = CO.net_forward(occ, geos, p.astype(np.float64))
    err = np.abs(z - zr)
    assert err.max() <= 1e-2 * max(1.0, np.abs(zr).max()), err.max()


def test_network_gradients_match_oracle(lib):
    import torch
    from opencuda_gb300.proposal import HoughNet
    occ, geos = _occ_problem(4)
    net = HoughNet(seed=11)
    p = net.get_params()
    rng = np.random.default_rng(5)
    target = (rng.random((2, 90, 128)) < 0.005).astype(np.float32)
    dev = _dev_bf16(torch, occ)
    loss = net.train_step(dev, HoughNet.geos(geos), torch.from_numpy(target).cuda(), 0.0, 30.0)
    g = net.get_grads()
    assert np.array_equal(net.get_params(), p)       # lr = 0 leaves the weights
    lref, gref = CO.net_loss_grads(occ, geos, p.astype(np.float64), target, 30.0)
    assert abs(loss - lref) <= 1e-3 * abs(lref) + 1e-5
    o = 0
    for ci, co, _, _ in CO.LAYERS:
        for n in (co * 9 * ci, co):
            a, b = g[o:o + n], gref[o:o + n]
            rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
            assert rel < 0.05, (o, n, rel)
            o += n
    assert np.allclose(g[o:], gref[o:], rtol=1e-3, atol=1e-6)


def test_occupancy_matches_numpy(lib):
    """The network's input: the fraction of 255-pixels in every f x f cell
    (f = ceil(max(w, h) / 256)), as BF16, for ROIs of odd sizes and offsets
    (rows not 4-byte aligned) and whole images."""
    import math
    import torch
    from opencuda_gb300.houghline import HoughLine, Image
    from opencuda_gb300.proposal import HoughNet
    rng = np.random.default_rng(12)
    cases = []
    for (h, w, roi) in ((517, 333, None), (1030, 2047, (3, 5, 3 + 1999, 5 + 1001)),
                        (4096, 4093, None), (700, 701, (1, 2, 1 + 613, 2 + 597))):
        img = np.where(rng.random((h, w)) < 0.07, 255, rng.integers(0, 255, (h, w))).astype(np.uint8)
        cases.append((img, roi))
    hl = HoughLine(detheta=math.pi / 360)
    net = HoughNet(seed=1)
    dev = [Image.from_host(im, roi) if roi else Image.from_host(im) for im, roi in cases]
    occ, _ = net.occupancy(hl, dev)
    got = occ.cpu().numpy().view(np.uint16)
    for b, (img, roi) in enumerate(cases):
        sub = img if roi is None else img[roi[1]:roi[3], roi[0]:roi[2]]
        h, w = sub.shape
        f = max(1, (max(w, h) + 255) // 256)
        want = np.zeros((256, 256), np.float32)
        edge = (sub == 255).astype(np.int64)
        for i in range(min(256, (h + f - 1) // f)):
            for j in range(min(256, (w + f - 1) // f)):
                want[i, j] = edge[i * f:(i + 1) * f, j * f:(j + 1) * f].sum() / float(f * f)
        wb = CO.bf16_bits(want).view(np.uint16)
        assert np.array_equal(got[b], wb), b
