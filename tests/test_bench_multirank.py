"""The bench's N>1 path on the CPU: two gloo ranks agree on the slowest
rank's time and the whole-job rate, and the reference arm runs on rank 0
alone (the map does not shard, so N GPUs run N independent replicas)."""
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

import bench  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(100.0 + 10.0 * rank)
        rate = bench.whole_job_rate(5, world, t)
        out.put((rank, t, rate))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [110.0, 110.0]
    # 5 cycles on each of 2 replicas in 110 ms
    assert all(abs(r[2] - 10 / 0.110) < 1e-9 for r in res)


def test_single_process_is_unchanged():
    assert bench.max_over_ranks(42.0) == 42.0
    assert bench.whole_job_rate(3, 1, 1500.0) == pytest.approx(2.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setattr("sys.argv", ["bench.py", "--impl", "reference"])
    args = bench.parse_args()
    bench.run_reference(args)
    assert capsys.readouterr().out == ""


def test_step_parts_split_the_kernel_timers():
    """The bench line's per-step split of the bounded-lanes kernel: the
    flights' tag waits and the barrier are parts of the fly slot, the
    refills and absorbs a part of the cascade slot; the all-at-once kernel
    (colour phases) gives none."""
    phases = {"spawn": 300.0, "fly": 1500.0, "unused": 900.0, "colour0": 700.0, "colour1": 150.0,
              "colour2": 0.0, "ema": 0.0}
    parts = bench.step_parts(phases, 2)
    assert parts == {"tag_waits": 150.0, "flights": 150.0, "barrier": 450.0, "refill_absorb": 75.0,
                     "cascades": 275.0}
    assert bench.step_parts({}, 2) is None
    assert bench.step_parts({"fly": 1.0, "colour2": 3.0}, 1) is None
