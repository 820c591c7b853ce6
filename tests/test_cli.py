"""The headless app loop (SimpleWindErosion.cpp:27-34, 211-231): arguments
and the PPM writer on the CPU, a short run with exports on the GPU."""
import numpy as np
import pytest

from simplewinderosion_gb300 import cli


def test_defaults_are_the_app_cadence():
    a = cli.parse_args([])
    assert a.seed is None and a.size == 512 and a.particles == 0 and a.mode == "parallel"
    a = cli.parse_args(["42", "--size", "64", "--frames", "2"])
    assert a.seed == 42 and a.size == 64 and a.frames == 2
    with pytest.raises(SystemExit):
        cli.parse_args(["--every", "0"])
    assert cli.parse_args(["--wind", "1,0,1"]).wind == (1.0, 0.0, 1.0)
    for bad in ["1,0", "0,0,0", "a,b,c"]:
        with pytest.raises(SystemExit):
            cli.parse_args(["--wind", bad])


def test_ppm_writer(tmp_path):
    rgba = np.zeros((2, 3, 4), dtype=np.float32)
    rgba[0, 1, 0] = 1.0
    rgba[1, 2, 2] = 0.5
    cli.write_ppm(tmp_path / "m.ppm", rgba)
    data = (tmp_path / "m.ppm").read_bytes()
    head = b"P6\n3 2\n255\n"
    assert data.startswith(head)
    px = np.frombuffer(data[len(head):], dtype=np.uint8).reshape(2, 3, 3)
    assert px[0, 1, 0] == 255 and px[1, 2, 2] == 128 and px.sum() == 255 + 128


@pytest.mark.gpu
@pytest.mark.parametrize("mode,terrain", [("parallel", "bump"), ("ordered", "fbm")])
def test_run_and_export(tmp_path, mode, terrain):
    rc = cli.main(["7", "--size", "64", "--frames", "3", "--every", "2", "--export", str(tmp_path),
                   "--vertices", "--quiet", "--mode", mode, "--terrain", terrain, "--wind", "1,0,1"])
    assert rc == 0
    d = tmp_path / "frame_000001"
    h = np.load(d / "height.npy")
    assert h.shape == (64, 64) and np.isfinite(h).all()
    assert np.load(d / "windmap.npy").shape == (64, 64, 4)
    assert np.load(d / "vertices.npy").shape == (64, 64, 12)
    assert (d / "windmap.ppm").read_bytes().startswith(b"P6\n64 64\n255\n")
    assert not (tmp_path / "frame_000000").exists()
