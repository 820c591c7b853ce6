"""Learned surrogate: a BF16 U-Net that predicts the height change of a
terrain after a fixed number of erode cycles.

The network (channels 32/64/96/128 over four levels, 3x3 convolutions, GELU,
2x2 average pooling, nearest 2x upsampling, additive skips) runs on the
library's own kernels (csrc/swe_surrogate.cu, through the C ABI in
include/swe.h): tensor-core implicit-GEMM convolutions with fp32
accumulation, BF16 weights and activations, fp32 master weights and Adam.
Torch provides device memory and the stream only.

Training pairs come from the erosion path itself (`make_pairs`: ensembles of
seeded fBm terrains with random winds, eroded by swe_batch_erode in PARALLEL
mode, the plain GPU method), and the erosion path stays the judge: `Rollout` advances a terrain by
predicted jumps and, every `judge_every` jumps, runs the plain method over
the same jump and rejects the surrogate (falling back to the plain method)
once a prediction's height RMSE exceeds the bound.

Input: 16 channels per cell (height, the wind direction's x and z, zeros);
output channel 0 is the height change times `Surrogate.scale`. Map sides
must be multiples of 8.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import Field, Mode, Params, World, batch_erode, lib, wind_direction, _check

# (name, cin, cout) in forward order
LAYERS = [("in", 16, 32), ("e0", 32, 32), ("d1", 32, 64), ("d2", 64, 96), ("d3", 96, 128), ("b3", 128, 128),
          ("u2", 128, 96), ("u1", 96, 64), ("u0", 64, 32), ("out", 32, 16)]

_P = ctypes.c_void_p
_bound = False


def _bind():
    global _bound
    if _bound:
        return
    L = lib
    i64, f32, i32 = ctypes.c_int64, ctypes.c_float, ctypes.c_int
    L.swe_nn_conv3x3.argtypes = [_P, _P, _P, _P, i32, i32, i32, i32, i32, _P]
    L.swe_nn_conv3x3_flip.argtypes = [_P, _P, i32, i32, _P]
    L.swe_nn_conv3x3_tc_pack.argtypes = [_P, _P, i32, i32, i32, _P]
    L.swe_nn_conv3x3_tc.argtypes = [_P, _P, _P, _P, _P, i32, i32, i32, i32, i32, _P]
    L.swe_nn_status.argtypes = [ctypes.POINTER(ctypes.c_uint32)]
    L.swe_nn_conv3x3_wgrad_tc.argtypes = [_P, _P, _P, _P, i32, i32, i32, i32, i32, _P]
    L.swe_nn_conv3x3_wgrad.argtypes = [_P, _P, _P, _P, i32, i32, i32, i32, i32, _P]
    L.swe_nn_gelu.argtypes = [_P, _P, i64, _P]
    L.swe_nn_gelu_bwd.argtypes = [_P, _P, _P, i64, _P]
    L.swe_nn_pool2.argtypes = [_P, _P, i32, i32, i32, i32, i32, _P]
    L.swe_nn_up2.argtypes = [_P, _P, i32, i32, i32, i32, i32, _P]
    L.swe_nn_add.argtypes = [_P, _P, _P, i64, _P]
    L.swe_nn_pack_input.argtypes = [_P, _P, _P, i32, i32, i32, _P]
    L.swe_nn_pack_input_centered.argtypes = [_P, _P, _P, _P, i32, i32, i32, f32, _P]
    L.swe_nn_mse.argtypes = [_P, _P, f32, _P, _P, i64, i32, f32, _P]
    L.swe_nn_channel0.argtypes = [_P, _P, i64, i32, f32, _P]
    L.swe_nn_adam.argtypes = [_P, _P, _P, _P, _P, i64, f32, f32, f32, f32, i32, _P]
    L.swe_nn_to_bf16.argtypes = [_P, _P, i64, _P]
    _bound = True


def _p(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


class Ops:
    """The building blocks on torch tensors (bf16 NHWC activations)."""

    def __init__(self, torch, device):
        _bind()
        self.torch = torch
        self.device = device

    @property
    def s(self):
        return ctypes.c_void_p(self.torch.cuda.current_stream(self.device).cuda_stream)

    def empty(self, *shape, dtype=None):
        return self.torch.empty(shape, dtype=dtype or self.torch.bfloat16, device=self.device)

    def conv(self, x, w16, b, cout):
        n, h, wd, cin = x.shape
        y = self.empty(n, h, wd, cout)
        _check(lib.swe_nn_conv3x3(_p(x), _p(w16), _p(b), _p(y), n, h, wd, cin, cout, self.s))
        return y

    def pack_tc(self, w16, flip=False):
        """Weights [cout,3,3,cin] packed for the tensor-core convolution
        (flip: for the input gradient)."""
        cout, _, _, cin = w16.shape
        wp = self.empty(9 * cin * cout)
        _check(lib.swe_nn_conv3x3_tc_pack(_p(w16), _p(wp), cin, cout, 1 if flip else 0, self.s))
        return wp

    def conv_tc(self, x, wp, b, cout, act=False):
        """Tensor-core convolution of x with packed weights; with act, also
        returns GELU of the output (fused into the epilogue)."""
        n, h, wd, cin = x.shape
        y = self.empty(n, h, wd, cout)
        a = self.empty(n, h, wd, cout) if act else None
        _check(lib.swe_nn_conv3x3_tc(_p(x), _p(wp), _p(b), _p(y), _p(a), n, h, wd, cin, cout, self.s))
        return (y, a) if act else y

    def wgrad_tc(self, x, dy, dw, db):
        """Tensor-core weight gradient (and bias gradient) ADDED to dw, db."""
        n, h, wd, cin = x.shape
        _check(lib.swe_nn_conv3x3_wgrad_tc(_p(x), _p(dy), _p(dw), _p(db), n, h, wd, cin, dy.shape[3], self.s))

    @staticmethod
    def tc_ok(h, wd, cin, cout) -> bool:
        """Whether the tensor-core convolution takes this shape."""
        if cin % 16 or cout % 16 or cout > 256 or cin < 16 or cout < 16:
            return False
        tw = 128
        while tw > 1 and wd % tw:
            tw //= 2
        return tw >= 8 and h % (128 // tw) == 0

    def status(self) -> int:
        """Raises if a tensor-core kernel gave up on a wait (synchronises)."""
        self.torch.cuda.synchronize(self.device)
        v = ctypes.c_uint32()
        _check(lib.swe_nn_status(ctypes.byref(v)))
        return v.value

    def conv_dx(self, dy, w16, cin):
        n, h, wd, cout = dy.shape
        wf = self.empty(cin, 3, 3, cout)
        _check(lib.swe_nn_conv3x3_flip(_p(w16), _p(wf), cin, cout, self.s))
        dx = self.empty(n, h, wd, cin)
        _check(lib.swe_nn_conv3x3(_p(dy), _p(wf), None, _p(dx), n, h, wd, cout, cin, self.s))
        return dx

    def wgrad(self, x, dy, dw, db):
        n, h, wd, cin = x.shape
        _check(lib.swe_nn_conv3x3_wgrad(_p(x), _p(dy), _p(dw), _p(db), n, h, wd, cin, dy.shape[3], self.s))

    def gelu(self, pre):
        y = self.empty(*pre.shape)
        _check(lib.swe_nn_gelu(_p(pre), _p(y), pre.numel(), self.s))
        return y

    def gelu_bwd(self, pre, dact):
        y = self.empty(*pre.shape)
        _check(lib.swe_nn_gelu_bwd(_p(pre), _p(dact), _p(y), pre.numel(), self.s))
        return y

    def pool(self, x):
        n, h, wd, c = x.shape
        y = self.empty(n, h // 2, wd // 2, c)
        _check(lib.swe_nn_pool2(_p(x), _p(y), n, h, wd, c, 0, self.s))
        return y

    def pool_bwd(self, dy):
        n, h, wd, c = dy.shape
        dx = self.empty(n, 2 * h, 2 * wd, c)
        _check(lib.swe_nn_pool2(_p(dy), _p(dx), n, 2 * h, 2 * wd, c, 1, self.s))
        return dx

    def up(self, x):
        n, h, wd, c = x.shape
        y = self.empty(n, 2 * h, 2 * wd, c)
        _check(lib.swe_nn_up2(_p(x), _p(y), n, h, wd, c, 0, self.s))
        return y

    def up_bwd(self, dy):
        n, h, wd, c = dy.shape
        dx = self.empty(n, h // 2, wd // 2, c)
        _check(lib.swe_nn_up2(_p(dy), _p(dx), n, h // 2, wd // 2, c, 1, self.s))
        return dx

    def add(self, a, b):
        y = self.empty(*a.shape)
        _check(lib.swe_nn_add(_p(a), _p(b), _p(y), a.numel(), self.s))
        return y

    def pack(self, height, wind_xz, ref=None):
        """The network input; with `ref`, every map's heights are first moved
        so that its mean is ref (swe_nn_pack_input_centered)."""
        n, h, wd = height.shape
        x = self.empty(n, h, wd, 16)
        if ref is None:
            _check(lib.swe_nn_pack_input(_p(height), _p(wind_xz), _p(x), n, h, wd, self.s))
        else:
            means = self.torch.empty(n, dtype=self.torch.float32, device=self.device)
            _check(lib.swe_nn_pack_input_centered(_p(height), _p(wind_xz), _p(means), _p(x), n, h, wd, float(ref),
                                                  self.s))
        return x


class Surrogate:
    """The U-Net, its fp32 master weights, bf16 copies, gradients and Adam
    moments. `scale`: the height change is predicted as change * scale.
    `height_ref`: every input map is moved by a constant so that its mean
    height is height_ref (the erosion rules see only height differences, so
    the change over a jump does not depend on that constant); training and
    prediction both see terrains at that level."""

    HEIGHT_REF = 0.35  # about the mean height of the training terrains

    def __init__(self, device="cuda", seed=0, scale=100.0, use_tc=True, height_ref=HEIGHT_REF):
        import torch
        self.torch = torch
        self.use_tc = use_tc  # tensor-core (tcgen05) convolutions where the shape allows
        self.device = torch.device(device)
        self.ops = Ops(torch, self.device)
        self.scale = float(scale)
        self.height_ref = float(height_ref)
        rs = np.random.RandomState(seed)
        self.w, self.b, self.w16 = {}, {}, {}
        for name, cin, cout in LAYERS:
            fan_in = 9 * (3 if name == "in" else cin)
            std = math.sqrt(2.0 / fan_in) * (0.1 if name == "out" else 1.0)
            w = (rs.standard_normal((cout, 3, 3, cin)) * std).astype(np.float32)
            if name == "in":
                w[..., 3:] = 0.0  # the padding channels carry zeros
            self.w[name] = torch.from_numpy(w).to(self.device)
            self.b[name] = torch.zeros(cout, dtype=torch.float32, device=self.device)
        self.gw = {k: torch.zeros_like(v) for k, v in self.w.items()}
        self.gb = {k: torch.zeros_like(v) for k, v in self.b.items()}
        self.m = {k: torch.zeros_like(v) for k, v in list(self.w.items())}
        self.v = {k: torch.zeros_like(v) for k, v in list(self.w.items())}
        self.mb = {k: torch.zeros_like(v) for k, v in self.b.items()}
        self.vb = {k: torch.zeros_like(v) for k, v in self.b.items()}
        self.t = 0
        self.sync_bf16()

    def sync_bf16(self):
        self._packed = {}
        for k, w in self.w.items():
            if k not in self.w16:
                self.w16[k] = self.ops.empty(*w.shape)
            _check(lib.swe_nn_to_bf16(_p(w), _p(self.w16[k]), w.numel(), self.ops.s))

    def state(self) -> dict:
        out = {"scale": np.float32(self.scale), "height_ref": np.float32(self.height_ref)}
        for k in self.w:
            out[f"w_{k}"] = self.w[k].cpu().numpy()
            out[f"b_{k}"] = self.b[k].cpu().numpy()
        return out

    def load(self, state: dict):
        self.scale = float(state["scale"])
        if "height_ref" in state:
            self.height_ref = float(state["height_ref"])
        for k in self.w:
            self.w[k].copy_(self.torch.from_numpy(np.asarray(state[f"w_{k}"], np.float32)))
            self.b[k].copy_(self.torch.from_numpy(np.asarray(state[f"b_{k}"], np.float32)))
        self.sync_bf16()

    # ---- the convolutions: tensor-core kernels where the shape allows ----
    def _packed_w(self, name, flip):
        key = (name, flip)
        if key not in self._packed:
            self._packed[key] = self.ops.pack_tc(self.w16[name], flip)
        return self._packed[key]

    def _conv(self, name, inp, act):
        """(pre, GELU(pre)) with act, else pre."""
        o = self.ops
        n, h, wd, cin = inp.shape
        cout = self.b[name].numel()
        if self.use_tc and o.tc_ok(h, wd, cin, cout):
            return o.conv_tc(inp, self._packed_w(name, False), self.b[name], cout, act=act)
        pre = o.conv(inp, self.w16[name], self.b[name], cout)
        return (pre, o.gelu(pre)) if act else pre

    def _conv_dx(self, name, dy, cin):
        o = self.ops
        n, h, wd, cout = dy.shape
        if self.use_tc and o.tc_ok(h, wd, cout, cin):
            return o.conv_tc(dy, self._packed_w(name, True), None, cin)
        return o.conv_dx(dy, self.w16[name], cin)

    def _wgrad(self, name, inp, dy):
        o = self.ops
        n, h, wd, cin = inp.shape
        cout = dy.shape[3]
        if self.use_tc and o.tc_ok(h, wd, cin, cin) and cout % 16 == 0 and cout <= 128 and cin <= 128:
            o.wgrad_tc(inp, dy, self.gw[name], self.gb[name])
        else:
            o.wgrad(inp, dy, self.gw[name], self.gb[name])

    # ---- forward / backward ----
    def forward(self, x):
        """x: bf16 [n,h,w,16]. Returns the output tensor [n,h,w,16] and the
        cache of the backward pass."""
        o = self.ops
        cache = {}

        def conv_act(name, inp):
            pre, act = self._conv(name, inp, True)
            cache[name] = (inp, pre)
            return act

        a_in = conv_act("in", x)
        s0 = conv_act("e0", a_in)
        s1 = conv_act("d1", o.pool(s0))
        s2 = conv_act("d2", o.pool(s1))
        s3 = conv_act("d3", o.pool(s2))
        b3 = conv_act("b3", s3)
        d2 = o.add(conv_act("u2", o.up(b3)), s2)
        d1 = o.add(conv_act("u1", o.up(d2)), s1)
        d0 = o.add(conv_act("u0", o.up(d1)), s0)
        out = self._conv("out", d0, False)
        cache["out"] = (d0, out)
        return out, cache

    def backward(self, cache, dout):
        """Adds the gradients of every weight and bias from d loss / d out."""
        o = self.ops
        d0, _ = cache["out"]
        self._wgrad("out", d0, dout)
        dd0 = self._conv_dx("out", dout, 32)

        def back(name, dact):
            inp, pre = cache[name]
            dpre = o.gelu_bwd(pre, dact)
            self._wgrad(name, inp, dpre)
            return self._conv_dx(name, dpre, inp.shape[3]) if name != "in" else None

        dd1 = o.up_bwd(back("u0", dd0))
        dd2 = o.up_bwd(back("u1", dd1))
        db3 = o.up_bwd(back("u2", dd2))
        ds3 = back("b3", db3)
        ds2 = o.add(dd2, o.pool_bwd(back("d3", ds3)))
        ds1 = o.add(dd1, o.pool_bwd(back("d2", ds2)))
        ds0 = o.add(dd0, o.pool_bwd(back("d1", ds1)))
        da_in = back("e0", ds0)
        back("in", da_in)

    def zero_grad(self):
        for k in self.gw:
            self.gw[k].zero_()
            self.gb[k].zero_()

    def adam(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.t += 1
        s = self.ops.s
        for k in self.w:
            _check(lib.swe_nn_adam(_p(self.w[k]), _p(self.gw[k]), _p(self.m[k]), _p(self.v[k]), _p(self.w16[k]),
                                   self.w[k].numel(), lr, b1, b2, eps, self.t, s))
            _check(lib.swe_nn_adam(_p(self.b[k]), _p(self.gb[k]), _p(self.mb[k]), _p(self.vb[k]), None,
                                   self.b[k].numel(), lr, b1, b2, eps, self.t, s))
        self._packed = {}  # the bf16 weights changed

    # ---- training and prediction ----
    def train_step(self, height, wind_xz, target_dh, lr=1e-3):
        """One Adam step on a batch: height fp32 [n,h,w], wind_xz fp32 [n,2],
        target_dh fp32 [n,h,w] (unscaled). Returns the mean squared error of
        the scaled prediction."""
        torch = self.torch
        x = self.ops.pack(height, wind_xz, self.height_ref)
        out, cache = self.forward(x)
        dout = self.ops.empty(*out.shape)
        loss = torch.zeros(1, dtype=torch.float32, device=self.device)
        m = out.shape[0] * out.shape[1] * out.shape[2]
        _check(lib.swe_nn_mse(_p(out), _p(target_dh), self.scale, _p(dout), _p(loss), m, 16, 1.0 / m, self.ops.s))
        self.zero_grad()
        self.backward(cache, dout)
        self.adam(lr)
        return float(loss.item()) / m

    def predict(self, height, wind_xz):
        """Predicted height change, fp32 [n,h,w]."""
        torch = self.torch
        x = self.ops.pack(height, wind_xz, self.height_ref)
        out, _ = self.forward(x)
        n, h, wd, _ = out.shape
        ch0 = torch.empty((n, h, wd), dtype=torch.float32, device=self.device)
        _check(lib.swe_nn_channel0(_p(out), _p(ch0), n * h * wd, 16, 1.0 / self.scale, self.ops.s))
        return ch0


# map-side divisor of each layer's resolution
_LEVEL = {"in": 1, "e0": 1, "d1": 2, "d2": 4, "d3": 8, "b3": 8, "u2": 4, "u1": 2, "u0": 1, "out": 1}


def conv_flops(n, h, w, backward=False) -> float:
    """Multiply-add FLOPs (2 per MAC, padded channels included) of the
    network's convolutions for n maps of h x w: the forward pass, or the
    forward pass plus the input and weight gradients of a training step."""
    total = 0.0
    for name, cin, cout in LAYERS:
        f = 2.0 * cin * cout * 9 * n * (h // _LEVEL[name]) * (w // _LEVEL[name])
        total += f
        if backward:
            total += f * (1 if name == "in" else 2)
    return total


def make_pairs(count, size=256, cycles=50, particles=1000, seed=0, chunk=2048, mode=Mode.PARALLEL,
               erosion_seed=0):
    """Training pairs from the erosion path: `count` seeded fBm terrains
    (8 octaves, base frequency 1/64, persistence uniform in [0.4, 0.6], in
    [0, 0.5], plus 0.1 +- 0.02 sediment) with random wind angles, each eroded
    for `cycles` cycles of `particles` particles by swe_batch_erode (mode
    PARALLEL, the default) or swe_batch_erode_ordered (ORDERED);
    `erosion_seed` changes the erosion's random numbers and not the
    terrains. Returns (h0 [count,size,size], wind_xz [count,2], dh
    [count,size,size]) as float32 numpy arrays."""
    rs = np.random.RandomState(seed)
    h0 = np.empty((count, size, size), np.float32)
    dh = np.empty((count, size, size), np.float32)
    wind = np.empty((count, 2), np.float32)
    for first in range(0, count, chunk):
        k = min(chunk, count - first)
        worlds = []
        for i in range(k):
            ang = rs.uniform(0.0, 2.0 * np.pi)
            pers = rs.uniform(0.4, 0.6)
            wx, wy, wz = wind_direction(float(np.cos(ang)), 0.0, float(np.sin(ang)))
            wind[first + i] = (wx, wz)
            w = World(size, params=Params(pspeed=(wx, wy, wz)),
                      seed=int(seed * 1000003 + first + i + 1 + erosion_seed * 7777777))
            w.terrain(seed=int(seed * 7919 + first + i + 1), octaves=8, base_freq=1.0 / 64.0, persistence=pers,
                      sediment=0.1, sediment_jitter=0.02)
            worlds.append(w)
        for i, w in enumerate(worlds):
            h0[first + i] = w.height
        batch_erode(worlds, cycles, particles, mode=mode)
        for i, w in enumerate(worlds):
            w.sync()
            dh[first + i] = w.height - h0[first + i]
            w.close()
    return h0, wind, dh


def predict_tiled(model: "Surrogate", h, wind_xz, tile: int = 256, halo: int = 32, batch: int = 16):
    """The surrogate's height change for a large map h [n, n] (float32,
    host), applied in tile x tile pieces, each predicted from a window with
    `halo` cells of context on every side that the map has (windows at the
    map edge are shifted inward so that they stay tile + 2 halo wide; the
    map's own edge is then the window's edge, as in training). Only each
    window's central tile is kept."""
    torch = model.torch
    nx, nz = h.shape
    win = tile + 2 * halo
    if nx < win or nz < win:
        return predict_map_whole(model, h, wind_xz)
    out = np.empty((nx, nz), np.float32)
    jobs = []
    for x0 in range(0, nx, tile):
        for z0 in range(0, nz, tile):
            wx0 = min(max(x0 - halo, 0), nx - win)
            wz0 = min(max(z0 - halo, 0), nz - win)
            jobs.append((x0, z0, wx0, wz0))
    for k in range(0, len(jobs), batch):
        part = jobs[k:k + batch]
        hb = np.stack([h[wx0:wx0 + win, wz0:wz0 + win] for _, _, wx0, wz0 in part]).astype(np.float32)
        wd = torch.tensor([list(wind_xz)] * len(part), dtype=torch.float32, device=model.device)
        pred = model.predict(torch.from_numpy(hb).to(model.device), wd).cpu().numpy()
        for (x0, z0, wx0, wz0), p in zip(part, pred):
            tx, tz = min(tile, nx - x0), min(tile, nz - z0)
            out[x0:x0 + tx, z0:z0 + tz] = p[x0 - wx0:x0 - wx0 + tx, z0 - wz0:z0 - wz0 + tz]
    return out


def predict_map_whole(model: "Surrogate", h, wind_xz):
    """The surrogate's height change for one whole map h (float32, host)."""
    torch = model.torch
    hd = torch.from_numpy(np.ascontiguousarray(h[None], np.float32)).to(model.device)
    wd = torch.tensor([list(wind_xz)], dtype=torch.float32, device=model.device)
    return model.predict(hd, wd)[0].cpu().numpy()


def rmse(a, b) -> float:
    return float(np.sqrt(np.mean((np.asarray(a, np.float64) - np.asarray(b, np.float64)) ** 2)))


class Rollout:
    """Advances one terrain by jumps of `cycles` erode cycles: predicted by
    the surrogate, with the plain method (PARALLEL, `particles` per cycle)
    run over every `judge_every`-th jump as correction and judge. A jump whose
    prediction misses the plain result by more than `bound` (height RMSE
    relative to the plain result's height range) rejects the surrogate: it
    and every later jump use the plain method. `world` (default: a new World
    of the given size, wind and seed) is the terrain's holder and the plain
    method's runner."""

    def __init__(self, model: Surrogate, size, wind, cycles=50, particles=1000, seed=1, judge_every=4, bound=0.01,
                 world=None):
        self.model, self.size, self.cycles, self.particles = model, size, cycles, particles
        self.wind = wind_direction(*wind)
        self.judge_every, self.bound = judge_every, bound
        self.world = world if world is not None else World(size, params=Params(pspeed=self.wind), seed=seed)
        self.rejected = False
        self.jumps = 0
        self.judged = []  # relative RMSE of each judged jump

    def start(self, height):
        self.world.upload(Field.HEIGHT, np.asarray(height, np.float32))

    def predict_change(self, h):
        """The surrogate's height change over one jump, for the map h."""
        torch = self.model.torch
        hd = torch.from_numpy(np.ascontiguousarray(h[None], dtype=np.float32)).to(self.model.device)
        wd = torch.tensor([[self.wind[0], self.wind[2]]], dtype=torch.float32, device=self.model.device)
        return self.model.predict(hd, wd)[0].cpu().numpy()

    def step(self):
        """One jump; returns the terrain after it."""
        h = self.world.height
        self.jumps += 1
        judge = self.rejected or self.jumps % self.judge_every == 0
        pred = None if self.rejected else h + self.predict_change(h)
        if judge:
            self.world.erode(self.particles, self.cycles, mode=Mode.PARALLEL)
            plain = self.world.height
            if pred is not None:
                rel = rmse(pred, plain) / max(float(plain.max() - plain.min()), 1e-12)
                self.judged.append(rel)
                if rel > self.bound:
                    self.rejected = True
            return plain
        self.world.upload(Field.HEIGHT, pred.astype(np.float32))
        return pred

    def close(self):
        self.world.close()
