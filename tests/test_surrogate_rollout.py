"""The surrogate rollout's judging, on the host: every `judge_every`-th jump
runs the plain method and compares; a prediction off by more than the bound
rejects the surrogate for good; accepted jumps keep the prediction. The
plain method and the network are stand-ins here (numpy), so the logic is
tested without a GPU."""
import numpy as np

from simplewinderosion_gb300 import surrogate


class FakeWorld:
    """Holds a height map; 'erosion' lowers every cell by 0.01 per cycle."""

    def __init__(self, n):
        self.h = np.linspace(0.0, 1.0, n * n, dtype=np.float32).reshape(n, n)
        self.erode_calls = 0

    @property
    def height(self):
        return self.h.copy()

    def upload(self, field, a):
        self.h = np.asarray(a, np.float32).reshape(self.h.shape).copy()

    def erode(self, particles, cycles, mode=None):
        self.erode_calls += 1
        self.h = self.h - np.float32(0.01 * cycles)

    def close(self):
        pass


class FakeRollout(surrogate.Rollout):
    def __init__(self, error, **kw):
        super().__init__(None, 8, (1.0, 0.0, 0.0), cycles=2, world=FakeWorld(8), **kw)
        self.error = error  # added to the exact change

    def predict_change(self, h):
        return np.full_like(h, -0.02 + self.error)


def test_accurate_surrogate_is_kept_and_judged_every_kth_jump():
    ro = FakeRollout(0.0, judge_every=4, bound=0.01)
    start = ro.world.height
    for _ in range(8):
        ro.step()
    assert ro.world.erode_calls == 2 and len(ro.judged) == 2 and not ro.rejected
    assert max(ro.judged) < 1e-6
    assert np.allclose(ro.world.height, start - 8 * 0.02, atol=1e-5)


def test_inaccurate_surrogate_is_rejected_and_the_plain_method_takes_over():
    ro = FakeRollout(0.05, judge_every=3, bound=0.01)  # 5 % of the range off per jump
    for _ in range(3):
        ro.step()
    assert ro.rejected and len(ro.judged) == 1 and ro.judged[0] > 0.01
    calls = ro.world.erode_calls
    for _ in range(4):
        ro.step()
    assert ro.world.erode_calls == calls + 4  # every later jump is plain
    assert len(ro.judged) == 1  # nothing more to judge
