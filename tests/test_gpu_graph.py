"""A parallel erode cycle captured once into a CUDA graph and replayed: every
replay is one more erode cycle (the random-number cycle counter lives on the
device), bit for bit what direct calls give, in each kernel form (one
cluster, one CTA per SM, all particles at once). The world's first cycle runs
outside the capture, as its buffers are allocated then."""
import numpy as np
import pytest

import simplewinderosion_gb300 as swe
from simplewinderosion_gb300 import terrain
from tests.conftest import WIND_101, bits

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,particles,lanes", [
    (96, 3000, 0),       # 1,024 lanes: one cluster
    (128, 16384, -1),    # 16,384 lanes: one CTA per SM
    (64, 200000, -1),    # all at once beyond that: the colour-phase kernel
])
def test_replayed_graph_equals_direct_cycles(n, particles, lanes):
    torch = pytest.importorskip("torch")
    h = (terrain.normalise(terrain.fbm(n, n, 3, 4.0 / n)) + 0.1).astype(np.float32)
    params = swe.Params(pspeed=WIND_101, frac_bits=16, lanes=lanes)
    direct = swe.World(n, params=params, seed=21)
    graphed = swe.World(n, params=params, seed=21)
    for w in (direct, graphed):
        w.upload(swe.Field.HEIGHT, h)
        w.erode(particles, 1, mode=swe.Mode.PARALLEL)

    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    graphed.set_stream(stream.cuda_stream)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream, capture_error_mode="thread_local"):
        graphed.erode(particles, 1, mode=swe.Mode.PARALLEL, sync=False)
    # capturing runs nothing: the world is still after its first cycle
    for _ in range(3):
        g.replay()
    torch.cuda.synchronize()
    direct.erode(particles, 3, mode=swe.Mode.PARALLEL)
    for f in swe.FIELDS:
        assert np.array_equal(bits(graphed.download(f)), bits(direct.download(f))), f
    assert graphed.status() == 0
    graphed.set_stream(None)
    for w in (direct, graphed):
        w.close()


def test_replayed_batch_graph_equals_direct_cycles():
    """The prepared ensemble (swe_batch_run) captured once and replayed:
    every replay is one more cycle of every world, bit for bit what each
    world's own direct cycles give."""
    torch = pytest.importorskip("torch")
    cases = [(48, 48, 3000, WIND_101, 3), (64, 40, 2500, (0.0, 0.0, -1.0), 4), (96, 96, 9000, (1.0, 0.0, 0.0), 5)]

    def world(n, nz, wind, sd):
        h = (terrain.normalise(terrain.fbm(n, nz, sd, 4.0 / max(n, nz))) + 0.1).astype(np.float32)
        w = swe.World(n, nz, params=swe.Params(pspeed=wind, frac_bits=16), seed=100 + sd)
        w.upload(swe.Field.HEIGHT, h)
        return w

    graphed = [world(n, nz, wind, sd) for n, nz, _, wind, sd in cases]
    direct = [world(n, nz, wind, sd) for n, nz, _, wind, sd in cases]
    particles = [c[2] for c in cases]
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    graphed[0].set_stream(stream.cuda_stream)
    b = swe.Batch(graphed, particles)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream, capture_error_mode="thread_local"):
        b.run(1)
    for _ in range(3):
        g.replay()
    torch.cuda.synchronize()
    for w, p in zip(direct, particles):
        w.erode(p, 3, mode=swe.Mode.PARALLEL)
    for k, (a, c) in enumerate(zip(graphed, direct)):
        for f in swe.FIELDS:
            assert np.array_equal(bits(a.download(f)), bits(c.download(f))), (k, f)
        assert a.status() == 0
    b.close()
    graphed[0].set_stream(None)
    for w in graphed + direct:
        w.close()
