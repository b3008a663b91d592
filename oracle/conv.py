"""TEST INFRASTRUCTURE: float64 numpy reference of the learned preconditioner's
operators (3x3x3 zero-padded convolution forward, data gradient and weight
gradient in channels-last layout; 2x average pooling; nearest upsampling), used
to check the tcgen05 kernels and their gradients.  The learned network has no
counterpart in the reference solver, so these are restated from the definitions.

Tap order: tap = (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1), dz/dy/dx in {-1, 0, 1}
along D/H/W.  Weights are [C_out, 27, C_in].
"""
from __future__ import annotations

import numpy as np


def _taps():
    for tap in range(27):
        yield tap, tap // 9 - 1, (tap // 3) % 3 - 1, tap % 3 - 1


def _shift(x, dz, dy, dx):
    """out[b, d, h, w] = x[b, d + dz, h + dy, w + dx] with zeros outside."""
    B, D, H, W, C = x.shape
    out = np.zeros_like(x)
    d0, d1 = max(0, -dz), min(D, D - dz)
    h0, h1 = max(0, -dy), min(H, H - dy)
    w0, w1 = max(0, -dx), min(W, W - dx)
    out[:, d0:d1, h0:h1, w0:w1] = x[:, d0 + dz:d1 + dz, h0 + dy:h1 + dy, w0 + dx:w1 + dx]
    return out


def conv_fwd(x, w, bias=None, relu=False):
    x = np.asarray(x, np.float64)
    w = np.asarray(w, np.float64)
    y = np.zeros(x.shape[:4] + (w.shape[0],))
    for tap, dz, dy, dx in _taps():
        y += _shift(x, dz, dy, dx) @ w[:, tap, :].T
    if bias is not None:
        y += bias
    return np.maximum(y, 0.0) if relu else y


def conv_dgrad(gy, w):
    gy = np.asarray(gy, np.float64)
    w = np.asarray(w, np.float64)
    gx = np.zeros(gy.shape[:4] + (w.shape[2],))
    for tap, dz, dy, dx in _taps():
        gx += _shift(gy, -dz, -dy, -dx) @ w[:, tap, :]
    return gx


def conv_wgrad(x, gy):
    x = np.asarray(x, np.float64)
    gy = np.asarray(gy, np.float64)
    gw = np.zeros((gy.shape[-1], 27, x.shape[-1]))
    G = gy.reshape(-1, gy.shape[-1])
    for tap, dz, dy, dx in _taps():
        gw[:, tap, :] = G.T @ _shift(x, dz, dy, dx).reshape(-1, x.shape[-1])
    return gw


def avgpool2(x):
    B, D, H, W, C = x.shape
    return x.reshape(B, D // 2, 2, H // 2, 2, W // 2, 2, C).mean(axis=(2, 4, 6))


def upsample2(x):
    return x.repeat(2, axis=1).repeat(2, axis=2).repeat(2, axis=3)


def bf16(a):
    """Round float32 values to bfloat16 (round to nearest even) and return float64."""
    a = np.asarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unet_loss(spec, weights, r, k, target, k_shift, k_scale, real_in=2):
    """Float64 forward of the learned preconditioner's U-Net and its MSE loss
    (same graph as fluxcore3d_gb300.learned.UNetPreconditioner: packed 8-channel
    input, avg-pool down, nearest-upsample + concat up, output channel 0)."""
    r = np.asarray(r, np.float64)
    B = r.shape[0]
    rms = np.sqrt((r.reshape(B, -1) ** 2).mean(axis=1)) + 1e-30
    x = np.zeros(r.shape + (8,))
    x[..., 0] = r / rms[:, None, None, None]
    x[..., 1] = (np.log(np.maximum(np.asarray(k, np.float64), 1e-30)) - k_shift) * k_scale
    W = {s[0]: w for s, w in zip(spec, weights)}
    R = {s[0]: s[3] for s in spec}

    def conv(name, inp):
        return conv_fwd(inp, W[name], relu=R[name])
    ya = conv("a", x)
    yb = conv("b", ya)
    yc = conv("c", avgpool2(yb))
    yd = conv("d", yc)
    ye = conv("e", avgpool2(yd))
    yf = conv("f", ye)
    yg = conv("g", np.concatenate([upsample2(yf), yd], axis=-1))
    yh = conv("h", yg)
    yi = conv("i", np.concatenate([upsample2(yh), yb], axis=-1))
    yj = conv("j", yi)
    t = np.asarray(target, np.float64) / rms[:, None, None, None]
    return float(((yj[..., 0] - t) ** 2).mean())
