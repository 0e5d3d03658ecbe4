"""NumPy restatement of the denoiser U-Net -- TEST INFRASTRUCTURE ONLY.

The CPU oracle of ``ohao_dn_*`` (include/ohao_dn.h): the same graph, the same
BF16 storage points (activations, weights, the gradient operands of the
weight and data GEMMs) and FP64 arithmetic in between, so that the device's
tensor-core convolutions (FP32 accumulation) can be checked layer by layer
and end to end. Layout: activations [n, h, w, c8], weights [cout, 9, cin]
with tap = 3 * dy + dx (dy, dx in 0..2 for offsets -1..1).
"""
from __future__ import annotations

import numpy as np

CHANNELS = (32, 48, 64, 96, 128)


ROUND = True   # False: exact FP64 everywhere (for finite-difference checks of this file)


def bf16(x):
    """Round to bfloat16 (nearest even) and return as float64."""
    if not ROUND:
        return np.asarray(x, np.float64)
    f = np.ascontiguousarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def round8(c):
    return (c + 7) // 8 * 8


def layer_specs():
    """[(name, in0, in1, up0, cin_used, cout, relu)] in execution order with
    pools as ("pool", src, None, ...). Tensor 0 is the packed input."""
    specs = []
    tensors = [("x", 0, 16)]            # (name, level, c8)

    def conv(name, in0, in1, up0, cout, relu=True, cin_used=None):
        lvl = tensors[in0][1] - 1 if up0 else tensors[in0][1]
        cin8 = tensors[in0][2] + (tensors[in1][2] if in1 is not None else 0)
        specs.append(("conv", name, in0, in1, up0, cin_used or cin8, cin8, cout, relu, len(tensors)))
        tensors.append((name, lvl, round8(cout)))
        return len(tensors) - 1

    def pool(src):
        specs.append(("pool", tensors[src][0] + "_pool", src, None, False, 0, 0, 0, False, len(tensors)))
        tensors.append((tensors[src][0] + "_pool", tensors[src][1] + 1, tensors[src][2]))
        return len(tensors) - 1

    cur, skips = 0, []
    for l in range(5):
        a = conv(f"e{l}a", cur, None, False, CHANNELS[l], cin_used=12 if l == 0 else None)
        e = conv(f"e{l}", a, None, False, CHANNELS[l])
        if l < 4:
            skips.append(e)
            cur = pool(e)
        else:
            cur = e
    for l in (3, 2, 1, 0):
        a = conv(f"d{l}a", cur, skips[l], True, CHANNELS[l])
        cur = conv(f"d{l}", a, None, False, CHANNELS[l])
    conv("out", cur, None, False, 3, relu=False)
    return specs, tensors


def unflatten_params(p):
    """Flat parameter vector (ohao_dn_get_params layout) -> [(W[cout,9,cin], b[cout])]."""
    specs, _ = layer_specs()
    out, off = [], 0
    for s in specs:
        if s[0] != "conv":
            continue
        cin, cout = s[5], s[7]
        n = cout * 9 * cin
        W = np.asarray(p[off:off + n], np.float64).reshape(cout, 9, cin)
        off += n
        b = np.asarray(p[off:off + cout], np.float64)
        off += cout
        out.append((W, b))
    assert off == len(p)
    return out


def flatten_grads(gs):
    return np.concatenate([np.concatenate([gW.reshape(-1), gb]) for gW, gb in gs])


def _shift(x, dy, dx):
    """out[:, y, x] = x[:, y + dy, x + dx] with zero padding."""
    n, h, w, c = x.shape
    out = np.zeros_like(x)
    ys, yd = (slice(dy, h), slice(0, h - dy)) if dy >= 0 else (slice(0, h + dy), slice(-dy, h))
    xs, xd = (slice(dx, w), slice(0, w - dx)) if dx >= 0 else (slice(0, w + dx), slice(-dx, w))
    out[:, yd, xd] = x[:, ys, xs]
    return out


def conv3x3(x, W, b):
    """x [n,h,w,cin8], W [cout,9,cin] (cin <= cin8) -> [n,h,w,cout] (FP64)."""
    cin = W.shape[2]
    out = np.zeros(x.shape[:3] + (W.shape[0],))
    for tap in range(9):
        dy, dx = tap // 3 - 1, tap % 3 - 1
        out += _shift(x[..., :cin], dy, dx) @ W[:, tap, :].T
    return out + b


def conv3x3_dgrad(dz, W, cin8):
    """d x [n,h,w,cin8] of conv3x3 given dZ [n,h,w,cout]."""
    cin = W.shape[2]
    dx = np.zeros(dz.shape[:3] + (cin8,))
    for tap in range(9):
        dy_, dx_ = tap // 3 - 1, tap % 3 - 1
        dx[..., :cin] += _shift(dz @ W[:, tap, :], -dy_, -dx_)
    return dx


def conv3x3_wgrad(x, dz, cin):
    """dW [cout,9,cin] = sum over pixels of dZ * shifted x."""
    cout = dz.shape[-1]
    gW = np.zeros((cout, 9, cin))
    dzf = dz.reshape(-1, cout)
    for tap in range(9):
        dy, dx = tap // 3 - 1, tap % 3 - 1
        gW[:, tap, :] = dzf.T @ _shift(x[..., :cin], dy, dx).reshape(-1, cin)
    return gW


def pool2(x):
    n, h, w, c = x.shape
    return x.reshape(n, h // 2, 2, w // 2, 2, c).max(axis=(2, 4))


def pool2_bwd(x, dy):
    """Gradient to the first maximum of each 2x2 window (dy, dx order)."""
    n, h, w, c = x.shape
    xr = x.reshape(n, h // 2, 2, w // 2, 2, c).transpose(0, 1, 3, 2, 4, 5).reshape(n, h // 2, w // 2, 4, c)
    arg = np.argmax(xr, axis=3)
    dx = np.zeros_like(xr)
    np.put_along_axis(dx, arg[:, :, :, None, :], dy[:, :, :, None, :], axis=3)
    return dx.reshape(n, h // 2, w // 2, 2, 2, c).transpose(0, 1, 3, 2, 4, 5).reshape(n, h, w, c)


def up2(x):
    return x.repeat(2, axis=1).repeat(2, axis=2)


def up2_bwd(d):
    n, h, w, c = d.shape
    return d.reshape(n, h // 2, 2, w // 2, 2, c).sum(axis=(2, 4))


def forward(x, params):
    """Network forward on the packed input x [n,h,w,16] (BF16 values).
    Returns the list of tensors (BF16-rounded activations, FP64 output)."""
    specs, tensors = layer_specs()
    T = [x]
    li = 0
    for s in specs:
        if s[0] == "pool":
            T.append(pool2(T[s[2]]))
            continue
        _, name, in0, in1, up0, cin, cin8, cout, relu, _ = s
        xin = up2(T[in0]) if up0 else T[in0]
        if in1 is not None:
            xin = np.concatenate([xin, T[in1]], axis=-1)
        W, b = params[li]
        li += 1
        y = conv3x3(xin, bf16(W), b)
        c8 = round8(cout)
        if relu:
            y = bf16(np.maximum(y, 0.0))
        yp = np.zeros(y.shape[:3] + (c8,))
        yp[..., :cout] = y
        T.append(yp)
    return T


DISPLAY_WEIGHT = 1.0


def display_tf(x):
    """pow(ACES(x / 2), 1/2.2) and its slope (evaluated at ACES >= 1e-3)."""
    u = 0.5 * np.maximum(x, 0.0)
    num = u * (2.51 * u + 0.03)
    den = u * (2.43 * u + 0.59) + 0.14
    a = num / den
    da = ((5.02 * u + 0.03) * den - num * (4.86 * u + 0.59)) / (den * den) * 0.5
    ac = np.maximum(a, 1e-3)
    slope = np.where(a >= 1.0, 0.0, (1.0 / 2.2) * ac ** (1.0 / 2.2) / ac * da)
    return np.where(a >= 1.0, 1.0, np.maximum(a, 0.0) ** (1.0 / 2.2)), slope


DEMOD_EPS = 0.04
Y_MAX = 30.0   # output cap in log1p space


def demod(aov):
    """Albedo modulation m per pixel and channel: first-hit albedo + DEMOD_EPS
    on surface hits, 1 on background pixels."""
    hit = aov[..., 7:8] > 0.5
    return np.where(hit, np.maximum(aov[..., 0:3], 0.0) + DEMOD_EPS, 1.0)


def l1_loss_grad(out, target_lin, aov):
    """|out - log1p(t / m)| + DISPLAY_WEIGHT |D(m expm1(min(out, Y_MAX))) - D(t)|
    per channel (out in demodulated log1p space, m = demod(aov), D the
    display transform), mean and d out."""
    tl = np.maximum(target_lin, 0.0)
    m = demod(aov)
    y = out[..., :3]
    d = y - np.log1p(tl / m)
    e = np.where(y > 0, np.expm1(np.clip(y, 0.0, Y_MAX)), 0.0)
    dx, slope = display_tf(e * m)
    dd = dx - display_tf(tl)[0]
    cnt = d.size
    g = np.zeros_like(out)
    live = (y > 0) & (y < Y_MAX)
    g[..., :3] = (np.sign(d) + DISPLAY_WEIGHT * np.where(live, np.sign(dd) * slope * m * (e + 1.0), 0.0)) / cnt
    return (np.abs(d).sum() + DISPLAY_WEIGHT * np.abs(dd).sum()) / cnt, g


def unpack(out, aov):
    """Linear radiance from the network output and the AOV image."""
    return np.expm1(np.clip(out[..., :3], 0.0, Y_MAX)) * demod(aov)


def backward(T, params, d_out):
    """Parameter gradients [(gW, gb)] and tensor gradients, with the device's
    BF16 rounding of the GEMM operands (dZ, activations, weights)."""
    specs, tensors = layer_specs()
    G = [np.zeros_like(t) for t in T]
    G[-1] = d_out
    convs = [s for s in specs if s[0] == "conv"]
    grads = [None] * len(convs)
    li = len(convs)
    for s in reversed(specs):
        if s[0] == "pool":
            G[s[2]] += pool2_bwd(T[s[2]], G[s[9]])
            continue
        li -= 1
        _, name, in0, in1, up0, cin, cin8, cout, relu, outi = s
        W, b = params[li]
        dY = G[outi][..., :cout]
        y = T[outi][..., :cout]
        dz_full = dY * (y > 0) if relu else dY
        gb = dz_full.reshape(-1, cout).sum(axis=0)
        dz = bf16(dz_full)
        xin = up2(T[in0]) if up0 else T[in0]
        if in1 is not None:
            xin = np.concatenate([xin, T[in1]], axis=-1)
        gW = conv3x3_wgrad(xin, dz, cin)
        grads[li] = (gW, gb)
        if in0 != 0:
            dx = conv3x3_dgrad(dz, bf16(W), cin8)
            c0 = T[in0].shape[-1]
            G[in0] += up2_bwd(dx[..., :c0]) if up0 else dx[..., :c0]
            if in1 is not None:
                G[in1] += dx[..., c0:]
    return grads, G


def pack(rad, aov):
    """Network input [h, w, 16] from RGBA radiance and the 12-float AOV image."""
    h, w = rad.shape[:2]
    x = np.zeros((h, w, 16))
    x[..., 0:3] = np.log1p(np.maximum(rad[..., :3], 0.0) / demod(aov))
    x[..., 3:9] = aov[..., 0:6]
    x[..., 9] = np.where(aov[..., 7] > 0.5, 1.0 / (1.0 + np.maximum(aov[..., 6], 0.0)), 0.0)
    x[..., 10:12] = aov[..., 8:10]
    return bf16(x)
