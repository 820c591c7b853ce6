"""Benchmark: erode cycles/s of the GB300 parallel erosion path at 1024^2.

Workload (the plain-method configuration at 1024^2): a 1024x1024 FP32 height
map of seeded fBm (improved Perlin noise, base frequency 1/256, 8 octaves,
in [0, 0.5]) plus a 0.1 +- 0.02 sediment layer and a square bedrock pyramid
(height 0.4, base 200 cells) at the centre; prevailing wind
normalize(1,0,1); 1,048,576 particles per erode cycle; parallel fixed-point
mode with int32 Q16.16 heights and the default number of particles in flight
(cells/256 = 4,096 lanes at 1024^2, the setting whose height histogram,
spectrum and mean height stay within 2.5x the reference's own seed-to-seed
spread, tests/test_gpu_statistics_1024.py). One bench step = one erode cycle
(World::erode(P), source/world.hpp:36-77). Synthetic seeded data. The same
workload with all particles of a cycle in flight at once (faster, but its
statistics drift from the reference's) is reported beside it.

Timing: W untimed warm-up cycles, then K cycles, each bracketed by CUDA
events on the world's stream; L2 is flushed (256 MiB write) before every
timed cycle, outside the events. Multi-GPU (torchrun): one independent
replica world per rank (the map does not shard), barrier + max over ranks.

Also reported: the roofline of the dominant kernel, a CPU baseline (the
reference's own code compiled here, else the oracle port; bounded sample,
one core), end-to-end cycles/s through the C ABI with pinned host buffers,
and clocks.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "erode cycles/s at 1024^2 (plain GPU method, parallel fixed-point mode)"
UNIT = "cycles/s"
L2_FLUSH_BYTES = 256 << 20
PEAKS_FILE = ROOT / "MEASURED_PEAKS.json"
FALLBACK_HBM_GBS = 6800.0


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--size", type=int, default=1024)
    ap.add_argument("--particles", type=int, default=0, help="particles per cycle (default size^2)")
    ap.add_argument("--frac-bits", type=int, default=16)
    ap.add_argument("--lanes", type=int, default=0,
                    help="particles in flight: 0 = default (cells/256, min 1024), -1 = all at once")
    ap.add_argument("--no-all-at-once", action="store_true")
    ap.add_argument("--no-tc", action="store_true", help="surrogate-step: the warp-level mma.sync convolutions")
    ap.add_argument("--workload", choices=["plain1024", "ensemble", "exact-ensemble", "surrogate", "surrogate-step",
                                           "longrun"],
                    default="plain1024",
                    help="plain1024: the headline; ensemble: 64 terrains in one persistent launch; "
                         "exact-ensemble: independent 256^2 worlds in ORDERED mode, one thread each; "
                         "surrogate: train the learned surrogate at 256^2 and measure it against the plain method; "
                         "longrun: the surrogate-accelerated large map (--long-size, --long-jumps) against plain-only")
    ap.add_argument("--long-size", type=int, default=4096, help="longrun: map side")
    ap.add_argument("--long-jumps", type=int, default=4, help="longrun: 50-cycle jumps (every 4th by the plain method)")
    ap.add_argument("--terrains", type=int, default=64, help="ensemble: number of terrains")
    ap.add_argument("--worlds", type=int, default=8192, help="exact-ensemble: number of worlds")
    ap.add_argument("--pairs", type=int, default=1024, help="surrogate: training pairs")
    ap.add_argument("--train-steps", type=int, default=1000, help="surrogate: timed Adam steps")
    ap.add_argument("--sur-batch", type=int, default=64, help="surrogate: training batch")
    ap.add_argument("--exact-size", type=int, default=256, help="exact-ensemble: map side")
    ap.add_argument("--cpu-sample", type=int, default=196608, help="particles in the CPU baseline sample")
    ap.add_argument("--ref-sample", type=int, default=0,
                    help="particles per reference-arm step (default: a tenth of a cycle)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-surrogate", action="store_true", help="skip the surrogate leg of the plain1024 line")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch form (no autotuning)")
    ap.add_argument("--judge-every", type=int, default=8,
                    help="surrogate leg: every n-th 50-cycle jump is run by the plain method (the judge)")
    return ap.parse_args()


def workload(size: int):
    import simplewinderosion_gb300 as swe
    from simplewinderosion_gb300 import terrain
    h = terrain.config_plain_large(seed=2, n=size)
    wind = swe.wind_direction(1.0, 0.0, 1.0)
    return h, wind


def effective_lanes(lanes: int, size: int, particles: int) -> int:
    """Particles in flight for swe_params.lanes (the library's rule)."""
    if lanes > 0:
        lv = lanes
    elif lanes == 0:
        lv = max(1024, size * size // 256)
    else:
        lv = particles
    return max(1, min(lv, particles))


def kernel_form(lanes: int, sms: int = 152) -> tuple[str, int]:
    """(dominant kernel, its launches per cycle) for `lanes` in flight."""
    if lanes <= 4096:
        return "k_par_lanes (one 16-CTA cluster)", 3
    if lanes <= sms * 256 * 4:
        return "k_par_lanes (one CTA per SM, cooperative)", 3
    return "k_par_cycle (colour phases, cooperative)", 1


def config_dict(args, particles):
    lanes = effective_lanes(args.lanes, args.size, particles)
    return {
        "workload": f"plain method {args.size}^2: fBm(1/256)+sediment+pyramid(0.4, base 200), "
                    f"{particles} particles/cycle, wind normalize(1,0,1), parallel fixed-point "
                    f"int32 Q{32 - args.frac_bits}.{args.frac_bits}",
        "map": f"{args.size}x{args.size}",
        "particles_per_cycle": particles,
        "max_age": 512,
        "frac_bits": args.frac_bits,
        "lanes": lanes,
        "lanes_rule": "cells/256 (min 1024)" if args.lanes == 0 else ("all at once" if args.lanes < 0 else "given"),
        "l2": "flushed (256 MiB write) before every timed cycle",
        "parallelism": f"replicas x{args.gpus}" if args.gpus > 1 else "single GPU",
    }


# ---------------------------------------------------------------- multi-rank
def max_over_ranks(x: float, device="cpu") -> float:
    """The largest of every rank's x (the job's time is its slowest rank's);
    x itself with one process."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, world_size: int, total_ms: float) -> float:
    """Units per second of the whole job: every rank's units over the
    slowest rank's time (replicas: the map does not shard)."""
    return units_per_rank * world_size / (total_ms / 1e3)


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clock / throttle samples while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self._t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self._t = threading.Thread(target=self._read, daemon=True)
        self._t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self._t:
                self._t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- CPU legs
def cpu_cores_desc() -> str:
    core = pinned_core()
    return f"{platform.machine()} x{os.cpu_count()}" + (f", pinned to core {core}" if core is not None else "")


def pinned_core():
    """The host core the single-threaded CPU samples run on: the highest one
    this process may use (None where affinity cannot be set)."""
    try:
        return max(os.sched_getaffinity(0))
    except (AttributeError, OSError, ValueError):
        return None


class _PinnedToOneCore:
    """Runs a block on one host core, then restores the process's affinity."""

    def __enter__(self):
        self.saved = None
        core = pinned_core()
        if core is not None:
            try:
                self.saved = os.sched_getaffinity(0)
                os.sched_setaffinity(0, {core})
            except OSError:
                self.saved = None
        return self

    def __exit__(self, *exc):
        if self.saved is not None:
            os.sched_setaffinity(0, self.saved)
        return False


def cpu_sample(size: int, h, wind, particles: int, total_particles: int, prefer_reference: bool):
    """Time `particles` particles of one World::erode call on the CPU with the
    reference's own code when it is compiled here (oracle/_ref), else the
    oracle port; return (cycles/s, kind, seconds, particle-steps)."""
    from oracle import oracle
    kind = "port"
    if prefer_reference and oracle.reference_available():
        try:
            oracle.build_reference(sizes=(size,))
            kind = "reference"
        except Exception:
            kind = "port"
    if kind == "reference":
        ref = oracle.Reference(size)
        ref.reset(h)
        ref.srand(1)
        calls0 = ref.L.ref_rand_calls()
        with _PinnedToOneCore():
            t0 = time.perf_counter()
            ref.erode(particles, 1, pspeed=wind)
            dt = time.perf_counter() - t0
        # 4 rand() calls per spawn (world.hpp:52-54) and 3 per particle-step
        # (the turbulence draw, wind.hpp:83, made on every step that passes
        # the age and map checks)
        steps = (ref.L.ref_rand_calls() - calls0 - 4 * particles) // 3
    else:
        port = oracle.Port(size, pspeed=wind)
        port.set_field(0, h)
        port.seed(1)
        with _PinnedToOneCore():
            t0 = time.perf_counter()
            port.erode(particles, 1)
            dt = time.perf_counter() - t0
        steps = port.stats()[0]
    cycles_per_s = particles / (dt * total_particles)
    return cycles_per_s, kind, dt, steps


def cpu_work(sample: int, dt: float, steps) -> dict:
    """Per-particle work of a CPU sample, to set beside the GPU cycle's."""
    return {"steps_per_particle": steps / sample, "particle_steps_per_s": steps / dt} if steps else {}


# ---------------------------------------------------------------- reference arm
def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    size = args.size
    particles = args.particles or size * size
    h, wind = workload(size)
    sample = args.ref_sample or max(1, particles // 10)
    vals, secs, steps, kind = [], [], [], "port"
    # every step: the first `sample` particles of the first cycle on the
    # initial terrain (the same work as every timed GPU cycle's start)
    for i in range(args.warmup + args.steps):
        v, kind, dt, st = cpu_sample(size, h, wind, sample, particles, prefer_reference=True)
        if i >= args.warmup:
            vals.append(v)
            secs.append(dt)
            steps.append(st or 0)
    value = statistics.mean(vals)
    step_s = statistics.mean(secs)
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * step_s,
        "cycles_per_step": sample / particles,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": config_dict(args, particles),
        "cpu_baseline": {
            "value": value, "unit": UNIT, "cores": 1, "kind": kind,
            "sample": f"each step: the first {sample} of the {particles} particles ({100 * sample / particles:.0f} %) "
                      f"of one sequential World::erode cycle on the initial terrain, on {cpu_cores_desc()} (the "
                      f"reference loop is single-threaded), scaled to cycles/s",
            **cpu_work(sample * len(secs), sum(secs), sum(steps)),
        },
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- our arm
def run_ours(args):
    import torch
    import torch.distributed as dist

    import simplewinderosion_gb300 as swe

    world_size = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world_size > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)

    size = args.size
    particles = args.particles or size * size
    h, wind = workload(size)
    params = swe.Params(pspeed=wind, frac_bits=args.frac_bits, lanes=args.lanes)
    lanes = effective_lanes(args.lanes, size, particles)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    kernel_name, launches_per_cycle = kernel_form(lanes, sms)
    w = swe.World(size, params=params, seed=1000 + rank)
    w.upload(swe.Field.HEIGHT, h)
    # the autotuner picks the launch form (timed on a scratch copy of the world, before the timed region)
    tuned = w.tune(particles) if not args.no_tune and args.lanes >= 0 else None
    if tuned:
        form = {0: kernel_name, 1: "k_par_lanes (one 16-CTA cluster)",
                2: f"k_par_lanes (cooperative grid of {tuned['ctas']} CTAs)",
                3: f"k_par_lanes (cooperative grid of {tuned['ctas']} CTAs of 128 threads, lanes spread over "
                   f"the warps)"}.get(tuned["kind"], kernel_name)
        kernel_name = form if not (tuned["kind"] == 0) else kernel_name
    stream = torch.cuda.ExternalStream(w.stream(), device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    for _ in range(args.warmup):
        w.upload(swe.Field.HEIGHT, h)
        w.erode(particles, 1, mode=swe.Mode.PARALLEL)
    torch.cuda.synchronize()

    sampler = ClockSampler(local_rank) if rank == 0 else None
    if sampler:
        sampler.start()
    if world_size > 1:
        dist.barrier()
    torch.cuda.synchronize()
    total_ms = 0.0
    fly_ms = cas_ms = 0.0
    psteps = transfers = 0
    phases = {}  # the bounded-lanes kernel's own per-step timers, summed over the timed cycles
    for _ in range(args.steps):
        # every timed cycle is a first cycle on the initial terrain, the work
        # the CPU samples time (uploaded outside the timed region)
        w.upload(swe.Field.HEIGHT, h)
        flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        w.erode(particles, 1, mode=swe.Mode.PARALLEL, sync=False)
        e1.record(stream)
        w.sync()
        total_ms += e0.elapsed_time(e1)
        f, c = w.kernel_times()
        fly_ms += f
        cas_ms += c
        for key, val in w.phase_times().items():
            phases[key] = phases.get(key, 0.0) + val
        s, _, t = w.stats()
        psteps += s
        transfers += t
    torch.cuda.synchronize()
    if world_size > 1:
        dist.barrier()
    total_ms = max_over_ranks(total_ms, dev)
    clocks = sampler.stop() if sampler else None

    value = whole_job_rate(args.steps, world_size, total_ms)
    ms_per_step = total_ms / args.steps

    # Roofline of the dominant kernel. One erode cycle is one launch of the
    # persistent step kernel (with, in the bounded-lanes forms, a map sweep
    # before and after it), so its duration per launch is taken as the
    # event-timed cycle. Algorithmic bytes per particle-step B = 76 + 16 k
    # (3x3 height gather 36, four track read-modify-writes 32, the cell's
    # exchange read-modify-write 8, 16 per cascade transfer), k = transfers
    # per particle-step; bytes per launch = B x particle-steps per cycle.
    k = transfers / max(psteps, 1)
    bytes_per_step = 76.0 + 16.0 * k
    psteps_per_launch = psteps / args.steps
    achieved = bytes_per_step * psteps_per_launch / (ms_per_step / 1e3) / 1e9
    peak, peak_note = FALLBACK_HBM_GBS, "fallback"
    try:
        peak = float(json.loads(PEAKS_FILE.read_text())["hbm_gbs"])
        peak_note = "measured"
    except Exception:
        pass
    traffic = None
    tfile = ROOT / "profiles" / "traffic.json"
    if tfile.exists():
        try:
            tj = json.loads(tfile.read_text())
            if (int(tj.get("size", 0)) == args.size and int(tj.get("particles", 0)) == particles
                    and int(tj.get("lanes", 0)) == lanes):
                traffic = float(tj["dram_bytes_per_launch"])
        except Exception:
            traffic = None

    line = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world_size,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_per_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+i32",
        "data": "synthetic",
        "config": config_dict(args, particles),
        "particle_steps_per_s": whole_job_rate(psteps, world_size, total_ms),
        "kernels": {"cycle_ms": ms_per_step, "fly_phases_ms": fly_ms / args.steps,
                    "cascade_phases_ms": cas_ms / args.steps, "k_transfers_per_step": k,
                    "particle_steps_per_cycle": psteps_per_launch,
                    "steps_per_particle": psteps_per_launch / particles,
                    "step_parts_ms": step_parts(phases, args.steps)},
        "timed_cycles": "each a first cycle on the initial terrain (re-uploaded before it, outside the timing)",
        "roofline": {
            "bound": "hbm",
            "kernel": kernel_name,
            "achieved": achieved,
            "peak": peak,
            "unit": "GB/s",
            "frac": achieved / peak,
            "peak_source": peak_note,
            "bytes_per_particle_step": bytes_per_step,
            "traffic": traffic,
        },
        "gpu_launches": launches_per_cycle * args.steps,
        "launch_form": {"kernel": kernel_name, **(tuned or {"tuned": False})},
        "clocks": clocks,
    }

    if not args.no_e2e:
        line["e2e"] = e2e(w, swe, torch, stream, particles, args, world_size, h)

    if not args.no_surrogate and world_size == 1 and args.size == 1024:
        line["surrogate"] = surrogate_leg(swe, torch, dev, h, wind, args)

    if not args.no_all_at_once and args.lanes >= 0:
        line["lanes_cells_over_64"] = other_lanes(
            swe, torch, dev, h, wind, particles, args, world_size, rank, max(1024, args.size * args.size // 64),
            "cells/64 particles in flight (16,384 at 1024^2): height histogram and spectrum within 2.5x the "
            "reference's seed-to-seed spread, the mean height 8x (tests/statistics_check.py); not the headline")
        line["all_at_once"] = other_lanes(
            swe, torch, dev, h, wind, particles, args, world_size, rank, -1,
            "all particles of a cycle in flight at once: mass conservation exact, but histogram, spectrum and "
            "mean 25-130x the reference's seed-to-seed spread; not the headline")

    if rank == 0 and world_size == 1 and not args.no_cpu_baseline:
        v, kind, dt, steps = cpu_sample(size, h, wind, args.cpu_sample, particles, prefer_reference=True)
        line["cpu_baseline"] = {
            "value": v, "unit": UNIT, "cores": 1, "kind": kind,
            "sample": f"the first {args.cpu_sample} of the {particles} particles of one sequential World::erode "
                      f"cycle on the initial terrain ({dt:.1f} s on {cpu_cores_desc()}, one thread: the reference "
                      f"loop is sequential), scaled to cycles/s",
            **cpu_work(args.cpu_sample, dt, steps),
        }
    if rank == 0:
        print(json.dumps(line), flush=True)
    w.close()
    if world_size > 1:
        dist.destroy_process_group()


def surrogate_leg(swe, torch, dev, h, wind, args):
    """Surrogate-accelerated evolution at the headline configuration: the
    network trained at this density (checkpoint made by
    `python -m simplewinderosion_gb300.train_surrogate`) jumps 50 erode cycles
    of the 1024^2 workload terrain at once; the plain method runs the same 50
    cycles (the judge), and again with other random numbers (its own
    seed-to-seed floor). Height RMSE is relative to the plain result's height
    range. Evolution with the plain method over every `judge_every`-th jump
    runs at judge_every * 50 cycles per ((judge_every - 1) jump + 50 plain
    cycles); both times are measured here with CUDA events."""
    from simplewinderosion_gb300 import surrogate as S
    from simplewinderosion_gb300.train_surrogate import DEFAULT_OUT
    if not DEFAULT_OUT.exists():
        return {"unavailable": f"no checkpoint at {DEFAULT_OUT.name}"}
    with np.load(DEFAULT_OUT) as z:
        state = {k: z[k] for k in z.files}
    meta = json.loads(str(state.pop("meta")))
    model = S.Surrogate(device=dev)
    model.load(state)
    cycles = 50
    n = args.size
    wind_xz = (wind[0], wind[2])

    def plain(seed):
        w = swe.World(n, params=swe.Params(pspeed=wind, frac_bits=16), seed=seed)
        w.upload(swe.Field.HEIGHT, h)
        w.tune(n * n)  # the launch form the headline uses (cached)
        st = torch.cuda.ExternalStream(w.stream(), device=dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        w.erode(n * n, cycles, mode=swe.Mode.PARALLEL, sync=False)
        e1.record(st)
        w.sync()
        out = w.height
        w.close()
        return out, e0.elapsed_time(e1) / 1e3

    h_plain, t_plain = plain(31)
    h_floor, _ = plain(32)
    # the jump: input packing, forward pass, change read-out, on device-resident heights
    hd = torch.from_numpy(np.ascontiguousarray(h[None], np.float32)).to(dev)
    wd = torch.tensor([list(wind_xz)], dtype=torch.float32, device=dev)
    for _ in range(3):
        model.predict(hd, wd)
    torch.cuda.synchronize()
    reps = 10
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        dh = model.predict(hd, wd)
    e1.record()
    torch.cuda.synchronize()
    t_sur = e0.elapsed_time(e1) / 1e3 / reps
    model.ops.status()
    pred = h + dh[0].cpu().numpy()
    pred_tiled = h + S.predict_tiled(model, h, wind_xz)
    rng = max(float(h_plain.max() - h_plain.min()), 1e-12)
    rel = S.rmse(pred, h_plain) / rng
    j = max(1, args.judge_every)
    accel = j * cycles / ((j - 1) * t_sur + t_plain)
    return {
        "metric": f"surrogate-accelerated erode cycles/s at {n}^2 (50-cycle jumps, plain method over every {j}th)",
        "value": accel, "unit": UNIT, "plain_cycles_per_s": cycles / t_plain, "speedup_vs_plain": accel * t_plain / cycles,
        "jump_ms": t_sur * 1e3, "plain_50_cycles_ms": t_plain * 1e3, "judge_every": j, "jump_cycles": cycles,
        "rel_rmse": rel, "rel_rmse_tiled_256_halo32": S.rmse(pred_tiled, h_plain) / rng,
        "no_change_rel_rmse": S.rmse(h, h_plain) / rng, "plain_seed_floor_rel_rmse": S.rmse(h_floor, h_plain) / rng,
        "bound": 0.01, "within_bound": bool(rel <= 0.01),
        "judge": "the plain GPU method (PARALLEL, default lanes, Q16.16) over the same 50 cycles of the workload terrain",
        "checkpoint": {k: meta[k] for k in ("train_runs", "steps", "batch", "crop", "surrogate_rel_rmse",
                                            "no_change_rel_rmse", "plain_seed_floor_rel_rmse") if k in meta},
    }


def step_parts(phases: dict, cycles: int) -> dict | None:
    """The bounded-lanes kernel's per-cycle split (ms, thread 0 of CTA 0's
    clock; swe_world_phase_times): the flights' tag waits, the flights
    themselves, the step's barrier, refills and absorbs, cascades. None for
    the all-at-once kernel, whose slots hold its colour phases."""
    if not phases or cycles < 1:
        return None
    g = {k: v / cycles for k, v in phases.items()}
    if g.get("colour2", 0.0) > 0.0:
        return None
    fly, tags, barrier = g.get("fly", 0.0), g.get("spawn", 0.0), g.get("unused", 0.0)
    casc, absorb = g.get("colour0", 0.0), g.get("colour1", 0.0)
    return {"tag_waits": tags, "flights": fly - tags - barrier, "barrier": barrier, "refill_absorb": absorb,
            "cascades": casc - absorb}


def other_lanes(swe, torch, dev, h, wind, particles, args, world_size, rank, lanes, note):
    """The same workload with another number of particles in flight (more
    lanes: fewer, shorter steps, but the terrain statistics drift further
    from the sequential reference's; `note` says how far). Timed like the
    headline: every cycle a first cycle on the initial terrain, L2 flushed."""
    import torch.distributed as dist
    params = swe.Params(pspeed=wind, frac_bits=args.frac_bits, lanes=lanes)
    w = swe.World(args.size, params=params, seed=1000 + rank)
    stream = torch.cuda.ExternalStream(w.stream(), device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    for _ in range(max(args.warmup, 3)):
        w.upload(swe.Field.HEIGHT, h)
        w.erode(particles, 1, mode=swe.Mode.PARALLEL)
    torch.cuda.synchronize()
    if world_size > 1:
        dist.barrier()
    total = 0.0
    for _ in range(args.steps):
        w.upload(swe.Field.HEIGHT, h)
        flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        w.erode(particles, 1, mode=swe.Mode.PARALLEL, sync=False)
        e1.record(stream)
        w.sync()
        total += e0.elapsed_time(e1)
    total = max_over_ranks(total, dev)
    w.close()
    lv = effective_lanes(lanes, args.size, particles)
    return {"value": whole_job_rate(args.steps, world_size, total), "unit": UNIT, "ms_per_step": total / args.steps,
            "lanes": lv, "kernel": kernel_form(lv)[0], "note": note}


def e2e(w, swe, torch, stream, particles, args, world_size, h):
    """Cycles/s through the C ABI with the height map kept on the host: per
    cycle, upload the height map from pinned memory, erode one cycle, read
    back height and momentum (the fields the reference's app loop reads after
    erode, SimpleWindErosion.cpp:217-230). Every cycle uploads the initial
    terrain, so each is the same first-cycle work the device-timed cycles and
    the CPU samples do; the copies replace the L2 flush."""
    import torch.distributed as dist
    n = w.n
    h_pin = torch.from_numpy(np.ascontiguousarray(h, np.float32).reshape(-1)).pin_memory()
    out_pin = torch.empty(n, dtype=torch.float32).pin_memory()
    moms = [torch.empty(n, dtype=torch.float32).pin_memory() for _ in range(3)]
    mom_fields = [swe.Field.MOMENTUMX, swe.Field.MOMENTUMY, swe.Field.MOMENTUMZ]
    torch.cuda.synchronize()
    if world_size > 1:
        dist.barrier()
    total = 0.0
    for _ in range(args.steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        w.upload_ptr(swe.Field.HEIGHT, h_pin.data_ptr(), n)
        w.erode(particles, 1, mode=swe.Mode.PARALLEL, sync=False)
        w.download_ptr(swe.Field.HEIGHT, out_pin.data_ptr(), n)
        for f, o in zip(mom_fields, moms):
            w.download_ptr(f, o.data_ptr(), n)
        e1.record(stream)
        w.sync()
        total += e0.elapsed_time(e1)
    total = max_over_ranks(total, "cuda")
    return {"value": whole_job_rate(args.steps, world_size, total), "unit": UNIT,
            "h2d_bytes_per_step": 4 * n, "d2h_bytes_per_step": 4 * 4 * n}


def run_ensemble(args):
    """The batched configuration: independent terrains with sides drawn
    log-uniformly from 128 to 1024 (rounded to multiples of 32), each with its
    own seed and a wind direction uniform in [0, 2 pi), side^2/4 particles per
    cycle, eroded together as a prepared batch (swe_batch_create: one
    persistent launch of thread-block clusters per cycle, the launch shape
    chosen by the autotuner unless --no-tune). One step = one cycle of every
    terrain; the metric is aggregate particle-steps/s. Terrains are built on
    the device (fBm of base frequency 4/side, 8 octaves, in [0, 0.5], plus
    0.1 +- 0.02 sediment)."""
    import torch

    import simplewinderosion_gb300 as swe

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    torch.cuda.set_device(0)
    rng = np.random.default_rng(2024)
    sides = np.clip(np.rint(np.exp(rng.uniform(np.log(128), np.log(1024), args.terrains)) / 32) * 32, 128, 1024)
    angles = rng.uniform(0.0, 2.0 * np.pi, args.terrains)
    worlds, particles = [], []
    for k, (side, ang) in enumerate(zip(sides.astype(int), angles)):
        wind = swe.wind_direction(float(np.cos(ang)), 0.0, float(np.sin(ang)))
        w = swe.World(int(side), params=swe.Params(pspeed=wind, frac_bits=args.frac_bits), seed=5000 + k)
        w.terrain(seed=7000 + k, octaves=8, base_freq=4.0 / side, sediment=0.1, sediment_jitter=0.02)
        worlds.append(w)
        particles.append(int(side) * int(side) // 4)
    batch = swe.Batch(worlds, particles, tune=not args.no_tune)
    shape = batch.shape()
    stream = torch.cuda.ExternalStream(worlds[0].stream(), device=torch.device("cuda", 0))
    for _ in range(args.warmup):
        batch.run(1)
    torch.cuda.synchronize()
    sampler = ClockSampler(0)
    sampler.start()
    total_ms, psteps, transfers = 0.0, 0, 0
    for _ in range(args.steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        batch.run(1)
        e1.record(stream)
        torch.cuda.synchronize()
        total_ms += e0.elapsed_time(e1)
        for w in worlds:
            st, _, tr = w.stats()
            psteps += st
            transfers += tr
    clocks = sampler.stop()
    rate = psteps / (total_ms / 1e3)
    k = transfers / max(psteps, 1)
    bps = 76.0 + 16.0 * k
    peak, note = FALLBACK_HBM_GBS, "fallback"
    try:
        peak = float(json.loads(PEAKS_FILE.read_text())["hbm_gbs"])
        note = "measured"
    except Exception:
        pass
    line = {
        "metric": "aggregate particle-steps/s, ensemble of independent terrains (one persistent launch)",
        "value": rate,
        "unit": "particle-steps/s",
        "n_gpus": 1,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+i32",
        "data": "synthetic",
        "config": {"workload": f"{args.terrains} terrains, sides log-uniform 128-1024 (multiples of 32), "
                               f"P = side^2/4, wind angle U[0, 2pi), default lanes, Q{32 - args.frac_bits}."
                               f"{args.frac_bits}",
                   "sides": sides.astype(int).tolist(), "cells": int(sum(int(s) ** 2 for s in sides)),
                   "particles_per_cycle": int(sum(particles))},
        "launch_shape": shape,
        "roofline": {"bound": "hbm", "kernel": "k_par_batch", "achieved": bps * rate / 1e9, "peak": peak,
                     "unit": "GB/s", "frac": bps * rate / 1e9 / peak, "peak_source": note,
                     "bytes_per_particle_step": bps, "traffic": None},
        "gpu_launches": args.steps,
        "clocks": clocks,
    }
    if not args.no_cpu_baseline:
        # the reference loop on one core, on a 256^2 terrain of the ensemble's kind
        from simplewinderosion_gb300 import terrain
        h256 = (terrain.normalise(terrain.fbm(256, 256, 7, 4.0 / 256)) + 0.1).astype(np.float32)
        v, kind, dt, steps = cpu_sample(256, h256, swe.wind_direction(1.0, 0.0, 1.0), 16384, 16384, True)
        if steps:
            line["cpu_baseline"] = {"value": steps / dt, "unit": "particle-steps/s", "cores": 1, "kind": kind,
                                    "sample": f"16384 particles of one sequential World::erode cycle on a 256^2 "
                                              f"terrain ({dt:.1f} s on {cpu_cores_desc()}, one thread)"}
    print(json.dumps(line), flush=True)
    batch.close()
    for w in worlds:
        w.close()


def run_exact_ensemble(args):
    """ORDERED mode at the reference's own small configuration, many times
    over: `--worlds` independent 256^2 worlds (`--exact-size`; fBm of base frequency 1/64, 8
    octaves, in [0, 0.5], plus 0.1 +- 0.02 sediment; wind normalize(1,0,1);
    each world its own terrain and rand() seed), 1000 particles per cycle,
    eroded by swe_batch_erode_ordered: every world bit for bit what the
    reference's World::erode computes from its seed. One step = one cycle of
    every world; the metric is aggregate particle-steps/s. The CPU baseline is
    the oracle port (the same arithmetic) running one world's cycles on one
    host core, the reference loop being single-threaded."""
    import torch

    import simplewinderosion_gb300 as swe
    from oracle import oracle

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    torch.cuda.set_device(0)
    size, particles = args.exact_size, 1000
    wind = swe.wind_direction(1.0, 0.0, 1.0)
    worlds = []
    for k in range(args.worlds):
        w = swe.World(size, params=swe.Params(pspeed=wind), seed=k + 1)
        w.terrain(seed=k + 1, octaves=8, base_freq=1.0 / 64.0, sediment=0.1, sediment_jitter=0.02)
        worlds.append(w)
    h0 = worlds[0].height
    stream = torch.cuda.ExternalStream(worlds[0].stream(), device=torch.device("cuda", 0))
    for _ in range(args.warmup):
        swe.batch_erode(worlds, 1, particles, mode=swe.Mode.ORDERED)
    torch.cuda.synchronize()
    sampler = ClockSampler(0)
    sampler.start()
    total_ms, psteps, transfers = 0.0, 0, 0
    for _ in range(args.steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        swe.batch_erode(worlds, 1, particles, mode=swe.Mode.ORDERED)
        e1.record(stream)
        torch.cuda.synchronize()
        total_ms += e0.elapsed_time(e1)
        st = [w.stats() for w in worlds]
        psteps += sum(x[0] for x in st)
        transfers += sum(x[2] for x in st)
    clocks = sampler.stop()
    value = psteps / (total_ms / 1e3)
    ms_per_step = total_ms / args.steps

    # Algorithmic bytes per particle-step: the 3x3 height gather 36, four
    # track read-modify-writes 32, the cell's height write 4, 4 per cascade
    # transfer.
    k = transfers / max(psteps, 1)
    bytes_per_step = 72.0 + 4.0 * k
    achieved = bytes_per_step * value / 1e9
    peak, peak_note = FALLBACK_HBM_GBS, "fallback"
    try:
        peak = float(json.loads(PEAKS_FILE.read_text())["hbm_gbs"])
        peak_note = "measured"
    except Exception:
        pass

    # e2e: every world's height map kept on the host (pinned), uploaded and
    # read back around each cycle through the C ABI.
    n = size * size
    host = torch.empty((0 if args.no_e2e else args.worlds, n), dtype=torch.float32).pin_memory()
    for i in range(host.shape[0]):
        worlds[i].download_ptr(swe.Field.HEIGHT, host[i].data_ptr(), n)
    e2e_ms, e2e_steps = 0.0, 0
    for _ in range(0 if args.no_e2e else args.steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i, w in enumerate(worlds):
            w.upload_ptr(swe.Field.HEIGHT, host[i].data_ptr(), n)
        swe.batch_erode(worlds, 1, particles, mode=swe.Mode.ORDERED)
        for i, w in enumerate(worlds):
            w.download_ptr(swe.Field.HEIGHT, host[i].data_ptr(), n)
        e1.record(stream)
        torch.cuda.synchronize()
        e2e_ms += e0.elapsed_time(e1)
        e2e_steps += sum(w.stats()[0] for w in worlds)

    # CPU baseline: one whole run of the configuration (100 cycles) on world
    # 0's initial terrain, on one core.
    cpu = None
    if not args.no_cpu_baseline:
        port = oracle.Port(size, pspeed=wind)
        port.set_field(0, h0)
        port.seed(1)
        with _PinnedToOneCore():
            t0 = time.perf_counter()
            port.erode(particles, 100)
            cpu_s = time.perf_counter() - t0
        cpu = {"value": port.stats()[0] / cpu_s, "unit": "particle-steps/s", "cores": 1, "kind": "port",
               "sample": f"one run (100 cycles x 1000 particles) of world 0 on {cpu_cores_desc()}, "
                         f"one thread ({cpu_s:.1f} s)"}

    line = {
        "metric": "aggregate particle-steps/s, ORDERED-mode ensemble (each world bit-identical to the reference)",
        "value": value,
        "unit": "particle-steps/s",
        "n_gpus": 1,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_per_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"{args.worlds} worlds of {size}^2, fBm(1/64)+sediment, wind normalize(1,0,1), "
                               f"1000 particles per cycle, ORDERED mode",
                   "worlds": args.worlds, "particles_per_cycle": particles,
                   "l2": f"working set {args.worlds * 9 * n * 4 / 2**30:.1f} GiB, larger than L2",
                   "reference_runs_per_s": args.worlds / (ms_per_step / 1e3) / 100.0},
        "roofline": {"bound": "hbm", "kernel": "k_ordered_batch (one thread per world)", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_note,
                     "bytes_per_particle_step": bytes_per_step, "traffic": None},
        "gpu_launches": 3 * args.steps,
        "clocks": clocks,
    }
    if not args.no_e2e:
        line["e2e"] = {"value": e2e_steps / (e2e_ms / 1e3), "unit": "particle-steps/s",
                       "h2d_bytes_per_step": 4 * n * args.worlds, "d2h_bytes_per_step": 4 * n * args.worlds}
    if cpu is not None:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)
    for w in worlds:
        w.close()


def run_surrogate_step(args):
    """One training step of the learned surrogate at batch `--sur-batch` and
    256^2 on seeded random terrains and targets (the kernels' speed does not
    depend on the values): `--warmup` untimed then `--steps` timed Adam steps
    (forward, backward, update) with CUDA events; tensor-core convolutions
    unless `--no-tc`. Reports ms per step and convolution TFLOP/s against
    the measured sustained bf16 peak. Small enough to run under ncu."""
    import torch

    from simplewinderosion_gb300 import surrogate as S

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    size, batch = 256, args.sur_batch
    rs = np.random.RandomState(5)
    h = torch.from_numpy(rs.uniform(0.1, 0.6, (batch, size, size)).astype(np.float32)).to(dev)
    wxz = torch.from_numpy(rs.standard_normal((batch, 2)).astype(np.float32)).to(dev)
    dh = torch.from_numpy((rs.standard_normal((batch, size, size)) * 0.01).astype(np.float32)).to(dev)
    model = S.Surrogate(device=dev, seed=1, use_tc=not args.no_tc)
    for _ in range(max(args.warmup, 3)):
        model.train_step(h, wxz, dh)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        model.train_step(h, wxz, dh)
    e1.record()
    torch.cuda.synchronize()
    model.ops.status()
    ms = e0.elapsed_time(e1) / args.steps
    flops = S.conv_flops(batch, size, size, backward=True)
    peak, note = 1700.0, "fallback"
    try:
        peak = float(json.loads(PEAKS_FILE.read_text())["bf16_tflops_sustained"])
        note = "measured sustained"
    except Exception:
        pass
    tf = flops / (ms / 1e3) / 1e12
    print(json.dumps({"metric": "surrogate training step (batch %d, 256^2)" % batch, "value": ms, "unit": "ms",
                      "higher_is_better": False, "steps": args.steps, "warmup": args.warmup,
                      "tensor_cores": "tcgen05" if not args.no_tc else "mma.sync",
                      "conv_tflops": tf, "roofline": {"bound": "tensor", "achieved": tf, "peak": peak,
                                                      "unit": "TFLOP/s", "frac": tf / peak, "peak_source": note}}),
          flush=True)


def run_surrogate(args):
    """The learned surrogate at 256^2: training pairs of 50 cycles x 1000
    particles made by the plain GPU method (PARALLEL, seeded fBm terrains of
    persistence U[0.4, 0.6], random wind angles), `--train-steps` timed Adam
    steps of batch 64 (lr 1e-3) after `--warmup` untimed ones, then on 64
    held-out pairs: the network's RMSE of the change, the no-change RMSE and
    the noise floor (the same held-out terrains eroded with other random
    numbers); the time of one 50-cycle jump by the network and by the plain
    method; and a judged rollout (8 jumps, the plain method every 4th). The
    metric is the jump speed-up; the line carries the accuracy beside it."""
    import torch

    import simplewinderosion_gb300 as swe
    from simplewinderosion_gb300 import surrogate as S

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    size, cycles, particles, batch = 256, 50, 1000, args.sur_batch
    t0 = time.perf_counter()
    h_tr, w_tr, d_tr = S.make_pairs(args.pairs, size, cycles, particles, seed=21)
    h_te, w_te, d_te = S.make_pairs(64, size, cycles, particles, seed=22)
    _, _, d_te2 = S.make_pairs(64, size, cycles, particles, seed=22, erosion_seed=1)
    gen_s = time.perf_counter() - t0

    model = S.Surrogate(seed=1, scale=1.0 / max(float(d_tr.std()), 1e-9))
    hd, wd, td = (torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (h_tr, w_tr, d_tr))
    rs = np.random.RandomState(3)

    def step():
        idx = torch.from_numpy(rs.randint(0, args.pairs, batch)).to(dev)
        return model.train_step(hd[idx].contiguous(), wd[idx].contiguous(), td[idx].contiguous(), lr=1e-3)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    losses = []
    e0.record(stream)
    for _ in range(args.train_steps):
        losses.append(step())
    e1.record(stream)
    torch.cuda.synchronize()
    train_ms = e0.elapsed_time(e1) / args.train_steps
    flops = S.conv_flops(batch, size, size, backward=True)
    tflops = flops / (train_ms / 1e3) / 1e12

    # accuracy on held-out pairs
    ht, wt = torch.from_numpy(h_te).to(dev), torch.from_numpy(w_te).to(dev)
    pred = model.predict(ht, wt).cpu().numpy()
    rng = float(np.mean([(h + d).max() - (h + d).min() for h, d in zip(h_te, d_te)]))
    err_net, err_none, err_floor = S.rmse(pred, d_te), S.rmse(0 * d_te, d_te), S.rmse(d_te2, d_te)

    # one 50-cycle jump of one terrain: network vs plain method
    def timed(fn, reps=5):
        fn()
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            best = min(best, a.elapsed_time(b))
        return best

    one_h, one_w = ht[:1].contiguous(), wt[:1].contiguous()
    sur_ms = timed(lambda: model.predict(one_h, one_w))
    sur_batch_ms = timed(lambda: model.predict(ht, wt)) / 64
    wind = (float(w_te[0, 0]), 0.0, float(w_te[0, 1]))
    world = swe.World(size, params=swe.Params(pspeed=wind), seed=5)
    world.upload(swe.Field.HEIGHT, h_te[0])
    wstream = torch.cuda.ExternalStream(world.stream(), device=dev)
    world.erode(particles, cycles, mode=swe.Mode.PARALLEL)
    world.sync()
    plain_ms = float("inf")
    for _ in range(3):
        world.upload(swe.Field.HEIGHT, h_te[0])
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(wstream)
        world.erode(particles, cycles, mode=swe.Mode.PARALLEL, sync=False)
        b.record(wstream)
        world.sync()
        plain_ms = min(plain_ms, a.elapsed_time(b))
    world.close()

    # judged rollout: 8 jumps, the plain method over every 4th
    ro = S.Rollout(model, size, wind, cycles=cycles, particles=particles, seed=9, judge_every=4, bound=0.01)
    ro.start(h_te[0])
    t1 = time.perf_counter()
    for _ in range(8):
        ro.step()
    roll_s = time.perf_counter() - t1
    judged, rejected = ro.judged, ro.rejected
    ro.close()

    peak, peak_note = 1900.0, "fallback"
    try:
        peak = float(json.loads(PEAKS_FILE.read_text())["bf16_tflops_sustained"])
        peak_note = "measured (sustained)"
    except Exception:
        pass
    line = {
        "metric": "surrogate speed-up over plain GPU erosion, one 50-cycle jump of a 256^2 terrain",
        "value": plain_ms / sur_ms,
        "unit": "x",
        "n_gpus": 1,
        "steps": args.train_steps,
        "warmup": max(args.warmup, 3),
        "ms_per_step": train_ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "bf16 (fp32 accumulate)",
        "data": "synthetic",
        "config": {"workload": f"U-Net 32/64/96/128 at 256^2, {args.pairs} training pairs of 50 cycles x 1000 "
                               f"particles (PARALLEL plain method), batch {batch}, Adam lr 1e-3, "
                               f"{args.train_steps} timed steps",
                   "pairs": args.pairs, "pair_generation_s": gen_s, "l2": "activations of a batch exceed L2"},
        "surrogate": {"jump_ms": sur_ms, "jump_ms_per_terrain_batch64": sur_batch_ms, "plain_jump_ms": plain_ms,
                      "speedup_batch64": plain_ms / sur_batch_ms,
                      "heldout_rmse_change": {"network": err_net, "no_change": err_none, "noise_floor": err_floor},
                      "heldout_rel_rmse": {"network": err_net / rng, "no_change": err_none / rng,
                                           "noise_floor": err_floor / rng},
                      "gain_over_no_change": 1.0 - err_net / err_none,
                      "loss_first_last": [float(np.mean(losses[:10])), float(np.mean(losses[-10:]))],
                      "rollout": {"jumps": 8, "judge_every": 4, "judged_rel_rmse": judged, "rejected": rejected,
                                  "seconds": roll_s}},
        "roofline": {"bound": "tensor", "kernel": "k_conv3x3 + k_conv_wgrad (warp-level mma.sync m16n8k16)",
                     "achieved": tflops, "peak": peak, "unit": "TFLOP/s", "frac": tflops / peak,
                     "peak_source": peak_note, "flops_per_step": flops, "traffic": None},
        "gpu_launches": 126 * args.train_steps,
    }
    print(json.dumps(line), flush=True)


def run_longrun(args):
    """The large-domain long run (simplewinderosion_gb300/longrun.py) with the
    committed checkpoint: `--long-jumps` 50-cycle jumps of a `--long-size`^2
    map, surrogate jumps in 256^2 tiles with 32-cell halos, every 4th jump by
    the plain method at one particle per cell per cycle, beside a plain-only
    run of the same terrain and wind. One JSON line: cycles/s of the
    accelerated run (host copies of the tiled prediction included) and of
    the plain-only run, and the comparison after the last judged jump."""
    import torch

    from simplewinderosion_gb300.longrun import long_run
    from simplewinderosion_gb300.surrogate import Surrogate
    from simplewinderosion_gb300.train_surrogate import DEFAULT_OUT

    torch.cuda.set_device(0)
    with np.load(DEFAULT_OUT) as z:
        state = {k: z[k] for k in z.files if k != "meta"}
    model = Surrogate()
    model.load(state)
    rec = long_run(model, args.long_size, args.long_jumps, 4, log=lambda *_: None)
    cycles = rec["jump_cycles"] * rec["jumps"]
    acc_s, plain_s = rec["seconds"]["accelerated"], rec["seconds"]["plain_only"]
    judged = [st for st in rec["steps"] if "rel_rmse" in st]
    line = {
        "metric": f"surrogate-accelerated erode cycles/s at {args.long_size}^2 (50-cycle jumps, plain method over "
                  f"every 4th)",
        "value": cycles / acc_s if acc_s > 0 else None,
        "unit": "cycles/s",
        "higher_is_better": True,
        "plain_only_cycles_per_s": cycles / plain_s if plain_s > 0 else None,
        "speedup_vs_plain_only": rec["speedup_vs_plain_only"],
        "jumps": rec["jumps"],
        "particles_per_cycle": rec["particles_per_cycle"],
        "tile": rec["tile"],
        "halo": rec["halo"],
        "last_comparison": judged[-1] if judged else None,
        "data": "synthetic",
        "steps": rec["steps"],
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "ensemble":
        run_ensemble(args)
    elif args.workload == "exact-ensemble":
        run_exact_ensemble(args)
    elif args.workload == "surrogate":
        run_surrogate(args)
    elif args.workload == "surrogate-step":
        run_surrogate_step(args)
    elif args.workload == "longrun":
        run_longrun(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
