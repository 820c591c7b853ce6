"""The large-domain long run's pieces on the GPU at reduced size: the tiled
application of the surrogate (256^2 tiles predicted from windows with
32-cell halos, windows at the map edge shifted inward) stitches exactly the
central tiles of the windows' own predictions, ragged last tiles included;
and a short surrogate-accelerated run with the plain method over every
second jump compares itself with the plain-only run after each judged jump."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def model():
    from simplewinderosion_gb300.surrogate import Surrogate
    return Surrogate(seed=9)


def test_tiled_prediction_stitches_window_centres(model):
    from simplewinderosion_gb300 import terrain
    from simplewinderosion_gb300.surrogate import predict_map_whole, predict_tiled
    nx, nz, tile, halo = 640, 576, 256, 32
    h = (terrain.normalise(terrain.fbm(nx, nz, 3, 1.0 / 128)) + 0.1).astype(np.float32)
    wind = (0.6, -0.8)
    got = predict_tiled(model, h, wind, tile, halo)
    win = tile + 2 * halo
    for x0 in range(0, nx, tile):
        for z0 in range(0, nz, tile):
            wx0 = min(max(x0 - halo, 0), nx - win)
            wz0 = min(max(z0 - halo, 0), nz - win)
            p = predict_map_whole(model, np.ascontiguousarray(h[wx0:wx0 + win, wz0:wz0 + win]), wind)
            tx, tz = min(tile, nx - x0), min(tile, nz - z0)
            want = p[x0 - wx0:x0 - wx0 + tx, z0 - wz0:z0 - wz0 + tz]
            assert np.array_equal(got[x0:x0 + tx, z0:z0 + tz], want), (x0, z0)
    model.ops.status()


def test_short_accelerated_run_judges_itself(model):
    from simplewinderosion_gb300.longrun import long_run
    rec = long_run(model, size=512, jumps=4, judge_every=2, seed=3, log=lambda *_: None)
    judged = [s for s in rec["steps"] if s["by"] == "plain"]
    assert [s["jump"] for s in judged] == [2, 4]
    for s in judged:
        assert np.isfinite(s["rel_rmse"]) and s["rel_rmse"] >= 0.0
        assert np.isfinite(s["spectrum_rms_log10"])
    assert rec["seconds"]["plain_only"] > 0 and rec["speedup_vs_plain_only"] > 0
