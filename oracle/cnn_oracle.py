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
