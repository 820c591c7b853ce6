"""The CPU restatement of the surrogate network (oracle/surrogate_ref.py),
which checks the CUDA kernels and GPU gradients, checked itself: its
analytic gradients against central finite differences, for one convolution
and for the whole U-Net, and its bf16 rounding against the definition."""
import numpy as np

from oracle import surrogate_ref as R


def _loss(pred, r):
    return float(np.sum(pred.astype(np.float64) * r))


def test_bf16_rounding_is_nearest_even():
    a = np.asarray([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.0e-3], np.float32)
    b = R.bf16(a)
    assert b[0] == 1.0 and b[1] == 1.0  # a tie rounds to even
    assert b[2] == np.float32(1.0 + 2 ** -7)
    assert b[3] == -2.5
    assert abs(b[4] - 3.0e-3) <= 3.0e-3 * 2 ** -8


def test_conv_gradients_by_finite_differences():
    rs = np.random.RandomState(0)
    x = rs.standard_normal((2, 6, 5, 4)).astype(np.float32)
    w = (rs.standard_normal((3, 3, 3, 4)) * 0.3).astype(np.float32)
    b = rs.standard_normal(3).astype(np.float32)
    r = rs.standard_normal((2, 6, 5, 3))
    dx, dw, db = R.conv3x3_grads(x, w, r.astype(np.float32))
    eps = 1e-2
    for arr, grad in ((x, dx), (w, dw), (b, db)):
        for _ in range(8):
            idx = tuple(rs.randint(0, s) for s in arr.shape)
            old = arr[idx]
            arr[idx] = old + eps
            lp = _loss(R.conv3x3(x, w, b), r)
            arr[idx] = old - eps
            lm = _loss(R.conv3x3(x, w, b), r)
            arr[idx] = old
            fd = (lp - lm) / (2 * eps)
            assert abs(fd - grad[idx]) <= 1e-3 * max(1.0, abs(fd)), (idx, fd, grad[idx])


def test_network_gradients_by_finite_differences():
    rs = np.random.RandomState(1)
    params = {}
    for name, cin, cout in R.LAYERS:
        params[name] = ((rs.standard_normal((cout, 3, 3, cin)) * np.sqrt(2.0 / (9 * cin))).astype(np.float32),
                        (rs.standard_normal(cout) * 0.05).astype(np.float32))
    h = rs.uniform(0.0, 0.6, (2, 8, 8)).astype(np.float32)
    x = R.pack_input(h, np.asarray([[0.6, 0.8], [-1.0, 0.0]], np.float32))
    r = rs.standard_normal((2, 8, 8))
    pred, cache = R.forward(params, x)
    grads = R.backward(params, cache, r.astype(np.float32))
    eps = 1e-2
    for name in ("in", "d1", "b3", "u1", "out"):
        for k in (0, 1):
            arr, grad = params[name][k], grads[name][k]
            for _ in range(3):
                idx = tuple(rs.randint(0, s) for s in arr.shape)
                if name == "in" and k == 0:
                    idx = idx[:3] + (rs.randint(0, 3),)  # the inputs' non-zero channels
                old = arr[idx]
                arr[idx] = old + eps
                lp = _loss(R.forward(params, x)[0], r)
                arr[idx] = old - eps
                lm = _loss(R.forward(params, x)[0], r)
                arr[idx] = old
                fd = (lp - lm) / (2 * eps)
                assert abs(fd - grad[idx]) <= 2e-2 * max(1.0, abs(fd)), (name, k, idx, fd, grad[idx])


def test_centred_input_moves_each_map_to_the_reference_level():
    """pack_input with ref (swe_nn_pack_input_centered's restatement): each
    map's height channel has mean (ref - 0.25) * 4, and a terrain and the
    same terrain lowered by a constant pack alike (to float rounding)."""
    rs = np.random.RandomState(4)
    h = rs.uniform(0.0, 0.6, (3, 16, 12)).astype(np.float32)
    wind = np.asarray([[0.6, 0.8], [-1.0, 0.0], [0.0, 1.0]], np.float32)
    x = R.pack_input(h, wind, ref=0.35)
    means = x[..., 0].reshape(3, -1).astype(np.float64).mean(axis=1)
    assert np.allclose(means, (0.35 - 0.25) * 4.0, atol=1e-6)
    y = R.pack_input((h - np.float32(2.5)).astype(np.float32), wind, ref=0.35)
    assert np.allclose(x[..., 0], y[..., 0], atol=1e-5)
    assert np.array_equal(x[..., 1:], y[..., 1:])
    # without ref the packing is the plain affine map
    z = R.pack_input(h, wind)
    assert np.array_equal(z[..., 0], (h - np.float32(0.25)) * np.float32(4.0))
