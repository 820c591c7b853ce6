"""CPU fp32 restatement of the learned surrogate's network (test infrastructure).

The same U-Net as simplewinderosion_gb300/surrogate.py, forward and backward
in numpy float32, used by the tests as the checker of the CUDA building
blocks (csrc/swe_surrogate.cu) and of the GPU gradients. Layout NHWC; 3x3
convolutions with zero padding, weights [cout, 3, 3, cin]; GELU in its erf
form; 2x2 average pooling; nearest 2x upsampling; additive skips.
Nothing here is called by the product.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

# (name, cin, cout) in the order the surrogate lists its layers
LAYERS = [("in", 16, 32), ("e0", 32, 32), ("d1", 32, 64), ("d2", 64, 96), ("d3", 96, 128), ("b3", 128, 128),
          ("u2", 128, 96), ("u1", 96, 64), ("u0", 64, 32), ("out", 32, 16)]


def bf16(a: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def conv3x3(x, w, b=None):
    n, h, wd, cin = x.shape
    cout = w.shape[0]
    xp = np.zeros((n, h + 2, wd + 2, cin), np.float32)
    xp[:, 1:-1, 1:-1] = x
    y = np.zeros((n, h, wd, cout), np.float32)
    for di in range(3):
        for dj in range(3):
            y += np.einsum("nhwc,oc->nhwo", xp[:, di:di + h, dj:dj + wd], w[:, di, dj, :], optimize=True)
    if b is not None:
        y += b
    return y


def conv3x3_grads(x, w, dy):
    """(dx, dw, db) of y = conv3x3(x, w) + b."""
    n, h, wd, cin = x.shape
    xp = np.zeros((n, h + 2, wd + 2, cin), np.float32)
    xp[:, 1:-1, 1:-1] = x
    dw = np.zeros_like(w)
    dxp = np.zeros_like(xp)
    for di in range(3):
        for dj in range(3):
            dw[:, di, dj, :] = np.einsum("nhwo,nhwc->oc", dy, xp[:, di:di + h, dj:dj + wd], optimize=True)
            dxp[:, di:di + h, dj:dj + wd] += np.einsum("nhwo,oc->nhwc", dy, w[:, di, dj, :], optimize=True)
    return dxp[:, 1:-1, 1:-1], dw, dy.sum(axis=(0, 1, 2))


def gelu(v):
    return (0.5 * v * (1.0 + erf(v / np.sqrt(2.0)))).astype(np.float32)


def gelu_grad(v):
    return (0.5 * (1.0 + erf(v / np.sqrt(2.0))) + v * np.exp(-0.5 * v * v) / np.sqrt(2.0 * np.pi)).astype(np.float32)


def pool2(x):
    n, h, wd, c = x.shape
    return x.reshape(n, h // 2, 2, wd // 2, 2, c).mean(axis=(2, 4)).astype(np.float32)


def pool2_bwd(dy):
    return (np.repeat(np.repeat(dy, 2, axis=1), 2, axis=2) * 0.25).astype(np.float32)


def up2(x):
    return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def up2_bwd(dy):
    n, h, wd, c = dy.shape
    return dy.reshape(n, h // 2, 2, wd // 2, 2, c).sum(axis=(2, 4)).astype(np.float32)


def pack_input(height, wind_xz, ref=None):
    """swe_nn_pack_input; with ref, swe_nn_pack_input_centered (each map moved
    so that its mean height is ref)."""
    n, h, wd = height.shape
    x = np.zeros((n, h, wd, 16), np.float32)
    if ref is None:
        x[..., 0] = (height - np.float32(0.25)) * np.float32(4.0)
    else:
        m = height.reshape(n, -1).astype(np.float64).mean(axis=1).astype(np.float32)[:, None, None]
        x[..., 0] = ((height - m) + (np.float32(ref) - np.float32(0.25))) * np.float32(4.0)
    x[..., 1] = wind_xz[:, 0, None, None]
    x[..., 2] = wind_xz[:, 1, None, None]
    return x


def forward(params, x):
    """params: name -> (w, b). Returns (prediction [n,h,w], cache)."""
    c = {}

    def conv_act(name, inp):
        w, b = params[name]
        pre = conv3x3(inp, w, b)
        c[name] = (inp, pre)
        return gelu(pre)

    a_in = conv_act("in", x)
    s0 = conv_act("e0", a_in)
    s1 = conv_act("d1", pool2(s0))
    s2 = conv_act("d2", pool2(s1))
    s3 = conv_act("d3", pool2(s2))
    b3 = conv_act("b3", s3)
    d2 = conv_act("u2", up2(b3)) + s2
    d1 = conv_act("u1", up2(d2)) + s1
    d0 = conv_act("u0", up2(d1)) + s0
    w, b = params["out"]
    out = conv3x3(d0, w, b)
    c["out"] = (d0, out)
    return out[..., 0], c


def backward(params, cache, dpred):
    """Gradients (name -> (dw, db)) from d loss / d prediction [n,h,w]."""
    grads = {}
    d0, out = cache["out"]
    dout = np.zeros_like(out)
    dout[..., 0] = dpred
    dd0, dw, db = conv3x3_grads(d0, params["out"][0], dout)
    grads["out"] = (dw, db)

    def back(name, dact):
        inp, pre = cache[name]
        dpre = dact * gelu_grad(pre)
        dinp, dw, db = conv3x3_grads(inp, params[name][0], dpre)
        grads[name] = (dw, db)
        return dinp

    ds0 = dd0.copy()
    dd1 = up2_bwd(back("u0", dd0))
    ds1 = dd1.copy()
    dd2 = up2_bwd(back("u1", dd1))
    ds2 = dd2.copy()
    db3 = up2_bwd(back("u2", dd2))
    ds3 = back("b3", db3)
    ds2 += pool2_bwd(back("d3", ds3))
    ds1 += pool2_bwd(back("d2", ds2))
    ds0 += pool2_bwd(back("d1", ds1))
    da_in = back("e0", ds0)
    back("in", da_in)
    return grads
