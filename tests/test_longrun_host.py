"""The long run's host-side pieces on the CPU: the tiled application of a
surrogate (tiles predicted from windows with halos, windows at the map edge
shifted inward so that they stay full size) reproduces a pointwise model
exactly, ragged last tiles included, and takes each tile from a window that
holds its halo wherever the map has one; the comparison's radial spectrum
and RMSE behave as their definitions say."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from simplewinderosion_gb300.longrun import compare, log_radial_spectrum
from simplewinderosion_gb300.surrogate import predict_tiled


class _PointwiseModel:
    """Stands in for the network: predicts 2 h + the window's wind x, cell
    by cell, and records the windows it was given."""

    def __init__(self):
        self.torch = torch
        self.device = torch.device("cpu")
        self.windows = []

    def predict(self, hb, wd):
        self.windows.append(tuple(hb.shape))
        return 2.0 * hb + wd[:, 0, None, None]


@pytest.mark.parametrize("nx,nz", [(640, 576), (320, 320), (700, 333)])
def test_tiled_prediction_of_a_pointwise_model_is_exact(nx, nz):
    rs = np.random.RandomState(nx + nz)
    h = rs.uniform(0.0, 1.0, (nx, nz)).astype(np.float32)
    m = _PointwiseModel()
    got = predict_tiled(m, h, (0.25, -0.5), tile=256, halo=32, batch=4)
    assert got.shape == (nx, nz)
    assert np.array_equal(got, (2.0 * h + np.float32(0.25)).astype(np.float32))
    # every window is a full 320 x 320 window
    assert all(s[1:] == (320, 320) for s in m.windows)
    tiles = -(-nx // 256) * -(-nz // 256)
    assert sum(s[0] for s in m.windows) == tiles


def test_a_small_map_is_predicted_whole():
    h = np.zeros((200, 300), np.float32)
    m = _PointwiseModel()
    got = predict_tiled(m, h, (1.0, 0.0), tile=256, halo=32)
    assert m.windows == [(1, 200, 300)] and np.all(got == 1.0)


def test_compare_and_spectrum():
    rs = np.random.RandomState(3)
    a = rs.standard_normal((128, 128))
    c = compare(a, a)
    assert c["rel_rmse"] == 0.0 and c["spectrum_rms_log10"] == 0.0 and c["mean_diff"] == 0.0
    c = compare(a + 1.5, a)
    assert abs(c["mean_diff"] - 1.5) < 1e-12
    assert c["spectrum_rms_log10"] < 1e-9  # the spectrum is of the mean-free map
    # a wave of period 16 cells puts its power at radius 1/16 of the sampling rate
    x = np.arange(128)
    wave = np.sin(2 * np.pi * x / 16)[:, None] * np.ones(128)[None, :]
    s = log_radial_spectrum(wave, bins=48)
    assert int(np.argmax(s)) == int(1 / 16 / 0.5 * 48)
