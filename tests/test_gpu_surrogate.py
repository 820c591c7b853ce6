"""The learned surrogate's CUDA building blocks and the network's GPU
gradients against the CPU fp32 restatement (oracle/surrogate_ref.py), on
bf16-representable inputs:
- convolution, its input gradient (flip + convolution) and its weight and
  bias gradients: within the bf16 rounding of the output (2^-8 relative) plus
  accumulation-order noise;
- GELU, pooling, upsampling and their adjoints: within bf16 rounding;
- whole-network weight gradients (bf16 activations through ten layers):
  within 5e-2 relative (Frobenius) per layer;
- training lowers the loss, and a network trained on erosion pairs made by
  the plain method predicts held-out pairs better than the method without
  it (no change), which is what the network gains.
"""
import numpy as np
import pytest

from oracle import surrogate_ref as R

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def dev(a):
    return torch.from_numpy(R.bf16(np.asarray(a, np.float32))).cuda().to(torch.bfloat16)


def host(t):
    return t.float().cpu().numpy()


def close(got, want, rel=2 ** -7, atol=1e-3):
    err = np.abs(got - want)
    assert np.all(err <= rel * np.abs(want) + atol), float((err - rel * np.abs(want)).max())


@pytest.fixture(scope="module")
def ops():
    from simplewinderosion_gb300 import surrogate
    return surrogate.Ops(torch, torch.device("cuda", 0))


@pytest.mark.parametrize("shape", [(2, 10, 12, 32, 48), (1, 7, 5, 16, 16), (3, 16, 16, 96, 128)])
def test_conv_forward_and_gradients(ops, shape):
    n, h, w, cin, cout = shape
    rs = np.random.RandomState(cin + cout)
    x = R.bf16(rs.standard_normal((n, h, w, cin)))
    wt = R.bf16(rs.standard_normal((cout, 3, 3, cin)) * np.sqrt(2.0 / (9 * cin)))
    b = rs.standard_normal(cout).astype(np.float32)
    dy = R.bf16(rs.standard_normal((n, h, w, cout)))
    y = host(ops.conv(dev(x), dev(wt), torch.from_numpy(b).cuda(), cout))
    close(y, R.conv3x3(x, wt, b))
    dx_want, dw_want, db_want = R.conv3x3_grads(x, wt, dy)
    close(host(ops.conv_dx(dev(dy), dev(wt), cin)), dx_want)
    dw = torch.zeros((cout, 3, 3, cin), dtype=torch.float32, device="cuda")
    db = torch.zeros(cout, dtype=torch.float32, device="cuda")
    ops.wgrad(dev(x), dev(dy), dw, db)
    close(dw.cpu().numpy(), dw_want, rel=1e-4, atol=1e-3)
    close(db.cpu().numpy(), db_want, rel=1e-4, atol=1e-3)


def test_elementwise_blocks(ops):
    rs = np.random.RandomState(3)
    x = R.bf16(rs.standard_normal((2, 8, 6, 32)) * 2)
    d = R.bf16(rs.standard_normal((2, 8, 6, 32)))
    close(host(ops.gelu(dev(x))), R.gelu(x))
    close(host(ops.gelu_bwd(dev(x), dev(d))), d * R.gelu_grad(x))
    close(host(ops.pool(dev(x))), R.pool2(x))
    close(host(ops.pool_bwd(dev(R.pool2(x)))), R.pool2_bwd(R.bf16(R.pool2(x))))
    close(host(ops.up(dev(x))), R.up2(x))
    close(host(ops.up_bwd(dev(R.up2(d)))), R.up2_bwd(R.up2(d)))
    close(host(ops.add(dev(x), dev(d))), x + d)
    hgt = rs.uniform(0, 0.6, (2, 8, 6)).astype(np.float32)
    wind = np.asarray([[0.6, 0.8], [-1.0, 0.0]], np.float32)
    close(host(ops.pack(torch.from_numpy(hgt).cuda(), torch.from_numpy(wind).cuda())), R.pack_input(hgt, wind))
    shifted = (hgt - np.float32(3.0)).astype(np.float32)
    close(host(ops.pack(torch.from_numpy(shifted).cuda(), torch.from_numpy(wind).cuda(), ref=0.35)),
          R.pack_input(shifted, wind, ref=0.35))


def test_gelu_and_its_derivative_over_every_bf16_input(ops):
    """The device GELU (Abramowitz & Stegun 7.1.26 for the normal CDF) on
    every bf16 value in [-12, 12] against the exact erf form in float64: the
    bf16 result is within one bf16 step of the exact value (or 1e-6 of it
    where the value underflows), and so is the derivative path."""
    import math
    bits = np.arange(0, 1 << 16, dtype=np.uint32).astype(np.uint16)
    v = (bits.astype(np.uint32) << 16).view(np.float32)
    v = v[np.isfinite(v) & (np.abs(v) <= 12.0)]
    v = v[: len(v) // 8 * 8].astype(np.float32)
    erf = np.vectorize(math.erf)
    exact = 0.5 * v.astype(np.float64) * (1.0 + erf(v.astype(np.float64) / math.sqrt(2.0)))
    got = host(ops.gelu(dev(v.reshape(-1, 8)))).reshape(-1).astype(np.float64)
    step = np.maximum(np.abs(exact) * 2.0 ** -7, 1e-6)
    assert np.all(np.abs(got - exact) <= step), float(np.max(np.abs(got - exact) / step))
    ones = np.ones_like(v)
    dexact = 0.5 * (1.0 + erf(v.astype(np.float64) / math.sqrt(2.0))) + v * np.exp(-0.5 * v.astype(np.float64) ** 2) / math.sqrt(2 * math.pi)
    dgot = host(ops.gelu_bwd(dev(v.reshape(-1, 8)), dev(ones.reshape(-1, 8)))).reshape(-1).astype(np.float64)
    dstep = np.maximum(np.abs(dexact) * 2.0 ** -7, 1e-6)
    assert np.all(np.abs(dgot - dexact) <= dstep), float(np.max(np.abs(dgot - dexact) / dstep))


def test_prediction_does_not_depend_on_the_height_level():
    """The erosion rules see heights only through differences; the
    surrogate's input is centred on its reference level, so a terrain and the
    same terrain 2.5 lower get the same predicted change (within the bf16
    rounding of the centred input)."""
    from simplewinderosion_gb300 import surrogate
    m = surrogate.Surrogate(seed=8)
    rs = np.random.RandomState(9)
    h = rs.uniform(0, 0.6, (2, 32, 32)).astype(np.float32)
    wind = torch.from_numpy(np.asarray([[0.6, 0.8], [-1.0, 0.0]], np.float32)).cuda()
    a = m.predict(torch.from_numpy(h).cuda(), wind).cpu().numpy()
    b = m.predict(torch.from_numpy((h - np.float32(2.5)).astype(np.float32)).cuda(), wind).cpu().numpy()
    assert np.abs(a - b).max() <= 0.05 * np.abs(a).max() + 1e-4


def _model_and_reference(seed=4):
    from simplewinderosion_gb300 import surrogate
    m = surrogate.Surrogate(seed=seed)
    # the oracle gets the bf16 weights the kernels use, and the fp32 biases
    params = {k: (host(m.w16[k]), m.b[k].cpu().numpy()) for k in m.w}
    return m, params


def test_network_gradients_match_the_cpu_restatement():
    from simplewinderosion_gb300 import lib, surrogate
    m, params = _model_and_reference()
    rs = np.random.RandomState(5)
    hgt = rs.uniform(0, 0.6, (2, 16, 16)).astype(np.float32)
    wind = np.asarray([[0.6, 0.8], [-1.0, 0.0]], np.float32)
    tgt = (rs.standard_normal((2, 16, 16)) * 0.01).astype(np.float32)
    x = m.ops.pack(torch.from_numpy(hgt).cuda(), torch.from_numpy(wind).cuda())
    out, cache = m.forward(x)
    pred_want, rcache = R.forward(params, R.pack_input(hgt, wind))
    pred = host(out)[..., 0]
    assert np.abs(pred - pred_want).max() <= 5e-2 * np.abs(pred_want).max() + 1e-3
    # d loss / d pred from the GPU prediction, fed to both backward passes
    dout = m.ops.empty(*out.shape)
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    n = hgt.size
    assert lib.swe_nn_mse(surrogate._p(out), surrogate._p(torch.from_numpy(tgt).cuda()), m.scale, surrogate._p(dout),
                          surrogate._p(loss), n, 16, 1.0 / n, m.ops.s) == 0
    dpred = host(dout)[..., 0]
    assert np.allclose(dpred, R.bf16(2.0 * (R.bf16(pred) - tgt * m.scale) / n), rtol=2 ** -7, atol=1e-7)
    m.zero_grad()
    m.backward(cache, dout)
    grads = R.backward(params, rcache, dpred)
    for name, _, _ in R.LAYERS:
        for got, want in ((m.gw[name].cpu().numpy(), grads[name][0]), (m.gb[name].cpu().numpy(), grads[name][1])):
            rel = np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-12)
            assert rel < 5e-2, (name, rel)


def test_training_lowers_the_loss():
    from simplewinderosion_gb300 import surrogate
    m = surrogate.Surrogate(seed=6, scale=1.0)
    rs = np.random.RandomState(7)
    # a learnable map: the change is a fixed multiple of the local relief
    h = rs.uniform(0, 0.5, (8, 32, 32)).astype(np.float32)
    blur = (np.roll(h, 1, 1) + np.roll(h, -1, 1) + np.roll(h, 1, 2) + np.roll(h, -1, 2)) / 4
    dh = (0.5 * (blur - h)).astype(np.float32)
    wind = np.tile(np.asarray([[1.0, 0.0]], np.float32), (8, 1))
    hd, wd, td = (torch.from_numpy(a).cuda() for a in (h, wind, dh))
    losses = [m.train_step(hd, wd, td, lr=2e-3) for _ in range(150)]
    assert np.mean(losses[-10:]) < 0.5 * np.mean(losses[:3]), (losses[:3], losses[-10:])


def test_trained_network_beats_no_change_on_held_out_erosion_pairs():
    from simplewinderosion_gb300 import surrogate
    h0, wind, dh = surrogate.make_pairs(192, size=64, cycles=20, particles=1024, seed=11)
    train, test = slice(0, 160), slice(160, 192)
    m = surrogate.Surrogate(seed=12, scale=1.0 / max(float(dh[train].std()), 1e-6))
    hd, wd, td = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (h0, wind, dh))
    rs = np.random.RandomState(13)
    for _ in range(400):
        idx = torch.from_numpy(rs.randint(0, 160, 32)).cuda()
        m.train_step(hd[idx].contiguous(), wd[idx].contiguous(), td[idx].contiguous(), lr=1e-3)
    pred = m.predict(hd[test].contiguous(), wd[test].contiguous()).cpu().numpy()
    err_net = surrogate.rmse(pred, dh[test])
    err_none = surrogate.rmse(0.0 * dh[test], dh[test])
    print(f"held-out RMSE of the change: network {err_net:.3e}, no change {err_none:.3e}")
    assert err_net < err_none
