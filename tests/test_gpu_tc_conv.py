"""The Blackwell tensor-core convolution (tcgen05.mma, TMEM accumulators,
TMA-fed tiles; swe_nn_conv3x3_tc) against the CPU fp32 restatement
(oracle/surrogate_ref.py) on bf16-representable inputs, forward (with bias
and the fused GELU) and input gradient (flipped packing), within the bf16
rounding of the output (2^-7 relative) plus accumulation-order noise. The
shapes cover every map width class (one tile per row pair or less, 128, 256),
channel counts 16..128 (k-blocks of 16 and 32 channels), an odd number of
128-pixel tiles (a CTA with one tile) and the network's own layers."""
import numpy as np
import pytest

from oracle import surrogate_ref as R

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def dev(a):
    return torch.from_numpy(R.bf16(np.asarray(a, np.float32))).cuda().to(torch.bfloat16)


def host(t):
    return t.float().cpu().numpy()


def close(got, want, rel=2 ** -7, atol=2e-3):
    err = np.abs(got - want)
    assert np.all(err <= rel * np.abs(want) + atol), float((err - rel * np.abs(want)).max())


@pytest.fixture(scope="module")
def ops():
    from simplewinderosion_gb300 import surrogate
    return surrogate.Ops(torch, torch.device("cuda", 0))


@pytest.mark.parametrize("shape", [
    (1, 8, 16, 16, 16),     # one tile: a CTA with one M tile; 8 rows of 16 pixels per tile
    (2, 16, 32, 32, 48),    # 4 rows x 32 pixels per tile; K-blocks of 16 for the gradient (48 channels)
    (1, 4, 256, 32, 32),    # half a row of 256 per tile
    (2, 8, 64, 96, 96),     # 2 rows x 64 per tile, 96 channels
    (1, 32, 32, 128, 128),  # the network's deepest level
    (1, 6, 128, 64, 16),    # the output layer's shape class (16 out)
    (1, 4, 320, 32, 32),    # a 320 wide window: tiles of 2 rows x 64 pixels, 5 per row pair
    (1, 8, 48, 16, 32),     # tiles of 8 rows x 16 pixels, 3 per row octet
])
def test_tc_conv_forward_and_input_gradient(ops, shape):
    n, h, w, cin, cout = shape
    rs = np.random.RandomState(cin * 7 + cout)
    x = R.bf16(rs.standard_normal((n, h, w, cin)))
    wt = R.bf16(rs.standard_normal((cout, 3, 3, cin)) * np.sqrt(2.0 / (9 * cin)))
    b = rs.standard_normal(cout).astype(np.float32)
    dy = R.bf16(rs.standard_normal((n, h, w, cout)))
    w16 = dev(wt)
    y, a = ops.conv_tc(dev(x), ops.pack_tc(w16), torch.from_numpy(b).cuda(), cout, act=True)
    yh = host(y)
    close(yh, R.conv3x3(x, wt, b))
    close(host(a), R.gelu(yh))
    dx_want, _, _ = R.conv3x3_grads(x, wt, dy)
    dx = ops.conv_tc(dev(dy), ops.pack_tc(w16, flip=True), None, cin)
    close(host(dx), dx_want)
    assert ops.status() == 0


@pytest.mark.parametrize("shape", [
    (8, 64, 256, 32, 96),   # 512 tile pairs: every CTA of the persistent grid takes 3-4, two accumulator sets
    (5, 64, 256, 16, 256),  # 320 pairs with 256 output channels: one accumulator set, reused in turn
    (4, 64, 256, 64, 32),   # the tap-per-k-block scheme (64-channel rows) with several units per CTA
])
def test_tc_conv_persistent_many_units(ops, shape):
    """More units (pairs of 128-pixel tiles) than CTAs: each CTA runs the
    stage ring through several units and reuses its TMEM accumulator sets;
    both unit schemes (vertically adjacent tiles sharing one input box per
    dx, and one tap-shifted box per tile and tap) are taken."""
    n, h, w, cin, cout = shape
    rs = np.random.RandomState(cin + cout)
    x = R.bf16(rs.standard_normal((n, h, w, cin)))
    wt = R.bf16(rs.standard_normal((cout, 3, 3, cin)) * np.sqrt(2.0 / (9 * cin)))
    b = rs.standard_normal(cout).astype(np.float32)
    y, a = ops.conv_tc(dev(x), ops.pack_tc(dev(wt)), torch.from_numpy(b).cuda(), cout, act=True)
    yh = host(y)
    close(yh, R.conv3x3(x, wt, b))
    close(host(a), R.gelu(yh))
    assert ops.status() == 0


def test_tc_conv_equals_warp_level_conv_closely(ops):
    """Same inputs through the tensor-core kernel and the warp-level mma.sync
    kernel: both accumulate bf16 products in fp32; outputs agree within one
    bf16 rounding step."""
    rs = np.random.RandomState(11)
    n, h, w, cin, cout = 2, 16, 128, 32, 64
    x = dev(rs.standard_normal((n, h, w, cin)))
    w16 = dev(rs.standard_normal((cout, 3, 3, cin)) * 0.1)
    b = torch.from_numpy(rs.standard_normal(cout).astype(np.float32)).cuda()
    y1 = host(ops.conv_tc(x, ops.pack_tc(w16), b, cout))
    y2 = host(ops.conv(x, w16, b, cout))
    close(y1, y2, rel=2 ** -7, atol=1e-3)


@pytest.mark.parametrize("shape", [
    (1, 8, 16, 16, 32),     # the input layer's channel class (16 in, 32 out)
    (2, 16, 32, 32, 16),    # 16 out: 112 padded rows of the 128-row MMA are never stored
    (1, 4, 256, 64, 32),    # 3 taps per CTA row (64 input channels)
    (3, 16, 16, 96, 128),   # 8 rows x 16 pixels per tile
    (1, 32, 32, 128, 128),
    (1, 4, 320, 32, 32),
])
def test_tc_weight_gradient(ops, shape):
    n, h, w, cin, cout = shape
    rs = np.random.RandomState(cin * 5 + cout)
    x = R.bf16(rs.standard_normal((n, h, w, cin)))
    wt = R.bf16(rs.standard_normal((cout, 3, 3, cin)) * np.sqrt(2.0 / (9 * cin)))
    dy = R.bf16(rs.standard_normal((n, h, w, cout)))
    _, dw_want, db_want = R.conv3x3_grads(x, wt, dy)
    dw = torch.zeros((cout, 3, 3, cin), dtype=torch.float32, device="cuda")
    db = torch.zeros(cout, dtype=torch.float32, device="cuda")
    ops.wgrad_tc(dev(x), dev(dy), dw, db)
    close(dw.cpu().numpy(), dw_want, rel=1e-4, atol=2e-3)
    close(db.cpu().numpy(), db_want, rel=1e-4, atol=2e-3)
    assert ops.status() == 0
