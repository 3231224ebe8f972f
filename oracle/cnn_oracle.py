"""CPU oracle of the proposal network (test infrastructure only).

There is no reference for the learned stage: these numpy functions restate
the network's arithmetic -- BF16 operands, exact products, sums in float64
(the kernels sum in FP32, so results agree to FP32 rounding) -- and give
finite-difference checks of the gradients.  Layouts follow the kernels:
activations NHWC, weights [Cout][tap * Cin + ci] with tap = ky * 3 + kx.
"""
from __future__ import annotations

import numpy as np


def bf16_round(a: np.ndarray) -> np.ndarray:
    """float32 -> nearest bfloat16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(a, np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    r = (b + 0x7FFF + ((b >> 16) & 1)) >> 16
    return (r.astype(np.uint32) << 16).view(np.float32)


def bf16_bits(a: np.ndarray) -> np.ndarray:
    """bfloat16 bit patterns (uint16) of bf16_round(a)."""
    return (bf16_round(a).view(np.uint32) >> 16).astype(np.uint16)


def from_bf16_bits(u: np.ndarray) -> np.ndarray:
    return (np.asarray(u, np.uint32) << 16).view(np.float32)


def conv3x3(x: np.ndarray, w: np.ndarray, bias=None, stride: int = 1,
            relu: bool = False) -> np.ndarray:
    """x [B,H,W,Cin], w [Cout, 9*Cin] -> y [B,Ho,Wo,Cout] (float64 sums)."""
    B, H, W, Cin = x.shape
    Cout = w.shape[0]
    Ho, Wo = (H - 1) // stride + 1, (W - 1) // stride + 1
    xp = np.zeros((B, H + 2, W + 2, Cin), np.float64)
    xp[:, 1:H + 1, 1:W + 1, :] = x
    wk = w.astype(np.float64).reshape(Cout, 3, 3, Cin)
    y = np.zeros((B, Ho, Wo, Cout), np.float64)
    for ky in range(3):
        for kx in range(3):
            patch = xp[:, ky:ky + stride * (Ho - 1) + 1:stride,
                       kx:kx + stride * (Wo - 1) + 1:stride, :]
            y += patch @ wk[:, ky, kx, :].T
    if bias is not None:
        y += np.asarray(bias, np.float64)
    if relu:
        y = np.maximum(y, 0.0)
    return y


def conv3x3_dx(dy: np.ndarray, w: np.ndarray, H: int, W: int,
               stride: int = 1) -> np.ndarray:
    """Input gradient of conv3x3: dy [B,Ho,Wo,Cout], w [Cout, 9*Cin]."""
    B, Ho, Wo, Cout = dy.shape
    Cin = w.shape[1] // 9
    wk = w.astype(np.float64).reshape(Cout, 3, 3, Cin)
    dxp = np.zeros((B, H + 2, W + 2, Cin), np.float64)
    for ky in range(3):
        for kx in range(3):
            dxp[:, ky:ky + stride * (Ho - 1) + 1:stride,
                kx:kx + stride * (Wo - 1) + 1:stride, :] += dy @ wk[:, ky, kx, :]
    return dxp[:, 1:H + 1, 1:W + 1, :]


def conv3x3_dw(x: np.ndarray, dy: np.ndarray, stride: int = 1) -> np.ndarray:
    """Weight gradient [Cout, 9*Cin] of conv3x3."""
    B, H, W, Cin = x.shape
    _, Ho, Wo, Cout = dy.shape
    xp = np.zeros((B, H + 2, W + 2, Cin), np.float64)
    xp[:, 1:H + 1, 1:W + 1, :] = x
    dw = np.zeros((Cout, 3, 3, Cin), np.float64)
    for ky in range(3):
        for kx in range(3):
            patch = xp[:, ky:ky + stride * (Ho - 1) + 1:stride,
                       kx:kx + stride * (Wo - 1) + 1:stride, :]
            dw[:, ky, kx, :] = np.einsum("bhwo,bhwi->oi", dy, patch)
    return dw.reshape(Cout, 9 * Cin)


def transpose_weights(w: np.ndarray) -> np.ndarray:
    """w [Cout, 9*Cin] -> w' [Cin, 9*Cout], w'[ci][tap][co] = w[co][tap][ci]
    (the weights of the stride-2 input-gradient gather)."""
    Cout = w.shape[0]
    Cin = w.shape[1] // 9
    return w.reshape(Cout, 9, Cin).transpose(2, 1, 0).reshape(Cin, 9 * Cout)


# ---- the whole proposal network ------------------------------------------
# (cin, cout, stride, relu) per layer; input 256 x 256 x 1 -> evidence 64 x 64
LAYERS = [(1, 32, 2, True), (32, 32, 2, True), (32, 32, 1, True),
          (32, 32, 1, True), (32, 32, 1, True), (32, 1, 1, False)]
HEAD_T, HEAD_R = 90, 128


def n_params() -> int:
    return sum(co * 9 * ci + co for ci, co, _, _ in LAYERS) + 2


def unpack(p: np.ndarray):
    """flat parameters -> [(W [cout, 9 cin], b [cout]) per layer], alpha, beta"""
    out, o = [], 0
    for ci, co, _, _ in LAYERS:
        w = p[o:o + co * 9 * ci].reshape(co, 9 * ci)
        o += co * 9 * ci
        b = p[o:o + co]
        o += co
        out.append((w, b))
    return out, float(p[o]), float(p[o + 1])


def head_trig():
    t = (np.arange(HEAD_T, dtype=np.float64) + 0.5) * np.pi / HEAD_T
    return np.cos(t).astype(np.float32), np.sin(t).astype(np.float32)


def head_bins(geo, ev: int) -> np.ndarray:
    """bins [T, ev, ev] (int, -1 outside the ROI's evidence cells) of one
    image geometry geo = (cell, rho_min, inv_rw, qh, qw), every float
    operation rounded to float32 as the kernel does."""
    cell, rho_min, inv_rw, qh, qw = geo
    f32 = np.float32
    c, s = head_trig()
    q = np.arange(ev, dtype=np.float32)
    xs = (q + f32(0.5)).astype(f32) * f32(cell)
    ys = xs.copy()
    out = np.full((HEAD_T, ev, ev), -1, np.int64)
    for t in range(HEAD_T):
        rho = (xs[None, :] * c[t]).astype(f32) + (ys[:, None] * s[t]).astype(f32)
        rho = rho.astype(f32)
        v = ((rho - f32(rho_min)).astype(f32) * f32(inv_rw)).astype(f32)
        r = np.clip(np.floor(v).astype(np.int64), 0, HEAD_R - 1)
        out[t, :qh, :qw] = r[:qh, :qw]
    return out


def net_forward(occ: np.ndarray, geos, p: np.ndarray, exact: bool = False):
    """occ [B, S, S] -> logits [B, T, R], head sums, evidence, activations.
    exact=False rounds weights and stored activations to bf16 as the GPU
    does; exact=True keeps float64 (for finite differences)."""
    layers, alpha, beta = unpack(np.asarray(p, np.float64))
    rnd = (lambda a: a.astype(np.float64)) if exact else \
        (lambda a: bf16_round(a.astype(np.float32)).astype(np.float64))
    x = rnd(occ)[..., None]
    acts = [x]
    for l, ((ci, co, st, relu), (w, b)) in enumerate(zip(LAYERS, layers)):
        y = conv3x3(x, rnd(w), b, st, relu)
        if l < len(LAYERS) - 1:
            y = rnd(y)
        acts.append(y)
        x = y
    e = acts[-1][..., 0]
    B, ev = e.shape[0], e.shape[1]
    H = np.zeros((B, HEAD_T, HEAD_R), np.float64)
    bins = [head_bins(g, ev) for g in geos]
    for b in range(B):
        for t in range(HEAD_T):
            m = bins[b][t] >= 0
            np.add.at(H[b, t], bins[b][t][m], e[b][m])
    return alpha * H + beta, H, e, acts, bins


def net_loss_grads(occ, geos, p, target, wpos: float, exact: bool = False):
    """Loss and flat gradient (float64) of the weighted BCE (mean over
    cells) through the whole network."""
    layers, alpha, beta = unpack(np.asarray(p, np.float64))
    rnd = (lambda a: a.astype(np.float64)) if exact else \
        (lambda a: bf16_round(a.astype(np.float32)).astype(np.float64))
    z, H, e, acts, bins = net_forward(occ, geos, p, exact)
    n = z.size
    sg = 1.0 / (1.0 + np.exp(-z))
    y = target
    loss = -np.sum(wpos * y * np.log(sg) + (1 - y) * np.log(1 - sg)) / n
    dz = (wpos * y * (sg - 1) + (1 - y) * sg) / n
    grads = []
    dalpha, dbeta = np.sum(dz * H), np.sum(dz)
    dH = alpha * dz
    B, ev = e.shape[0], e.shape[1]
    de = np.zeros_like(e)
    for b in range(B):
        for t in range(HEAD_T):
            m = bins[b][t] >= 0
            de[b][m] += dH[b, t][bins[b][t][m]]
    g = de[..., None]
    for l in range(len(LAYERS) - 1, -1, -1):
        ci, co, st, relu = LAYERS[l]
        w, _ = layers[l]
        if relu:
            g = g * (acts[l + 1] > 0)
        xin = acts[l]
        dw = conv3x3_dw(xin, g, st)
        db = g.sum(axis=(0, 1, 2))
        grads.append((dw, db))
        if l > 0:
            g = conv3x3_dx(g, rnd(w), xin.shape[1], xin.shape[2], st)
    grads = grads[::-1]
    flat = np.concatenate([np.concatenate([dw.ravel(), db.ravel()]) for dw, db in grads] +
                          [np.array([dalpha, dbeta])])
    return loss, flat
