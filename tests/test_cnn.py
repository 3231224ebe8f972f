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
