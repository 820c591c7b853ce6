"""The large-domain long run: a 4096^2 terrain evolved by surrogate jumps
applied in 256^2 tiles with 32-cell halos, with every `judge_every`-th jump
replaced by 50 plain-method cycles at one particle per cell per cycle
(16,777,216 at 4096^2) as correction and judge, compared after every judged
jump with a plain-only run of the same terrain and wind on height RMSE and
the radially averaged power spectrum (dune wavelengths).

    python -m simplewinderosion_gb300.longrun [--size N] [--jumps J] [--judge-every K] [--out PATH]

The reference erodes one fixed 512^2 tile (source/cellpool.h:186-195); this
is the same World::erode loop (source/world.hpp:36-77) at 64x the area, with
the learned jumps in between. The terrain: fBm of base frequency
1/1024 (scaled with the side) in [0, 0.5], 0.1 +- 0.02 sediment, 16 bedrock
pyramids of height 0.2-0.5 and base 100-400 cells (scaled with the side) at
seeded random places.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import Field, Mode, Params, World, wind_direction
from .surrogate import Surrogate, predict_tiled, rmse

JUMP_CYCLES = 50


def terrain_settings(size: int, seed: int) -> dict:
    rs = np.random.RandomState(seed)
    pyr = [(rs.uniform(0.05, 0.95) * size, rs.uniform(0.05, 0.95) * size, rs.uniform(0.2, 0.5),
            rs.uniform(100, 400) * size / 4096) for _ in range(16)]
    return {"seed": seed, "octaves": 8, "base_freq": 4.0 / size, "persistence": 0.5, "sediment": 0.1,
            "sediment_jitter": 0.02, "pyramids": pyr}


def log_radial_spectrum(h, bins: int = 48) -> np.ndarray:
    """log10 of the radially averaged power spectrum of the mean-free map."""
    h = np.asarray(h, np.float64)
    f = np.abs(np.fft.rfft2(h - h.mean())) ** 2
    k = np.sqrt(np.fft.fftfreq(h.shape[0])[:, None] ** 2 + np.fft.rfftfreq(h.shape[1])[None, :] ** 2)
    idx = np.minimum((k / 0.5 * bins).astype(np.int64), bins)
    s = np.bincount(idx.ravel(), weights=f.ravel(), minlength=bins + 1)[:bins]
    c = np.bincount(idx.ravel(), minlength=bins + 1)[:bins]
    return np.log10(s / np.maximum(c, 1) + 1e-30)


def compare(h, ref) -> dict:
    rng = max(float(ref.max() - ref.min()), 1e-12)
    return {"rel_rmse": rmse(h, ref) / rng,
            "spectrum_rms_log10": float(np.sqrt(np.mean((log_radial_spectrum(h) - log_radial_spectrum(ref)) ** 2))),
            "mean_diff": float(np.mean(h, dtype=np.float64) - np.mean(ref, dtype=np.float64))}


def long_run(model: Surrogate, size: int = 4096, jumps: int = 8, judge_every: int = 4, seed: int = 5,
             wind_angle: float = 0.7, tile: int = 256, halo: int = 32, log=print) -> dict:
    """Runs the surrogate-accelerated evolution and the plain-only run side by
    side (the plain-only world advances 50 cycles per jump); returns per-jump
    timings and, after every judged jump, the comparison of the two maps."""
    wx, wy, wz = wind_direction(float(np.cos(wind_angle)), 0.0, float(np.sin(wind_angle)))
    params = Params(pspeed=(wx, wy, wz), frac_bits=16)
    t = terrain_settings(size, seed)
    acc = World(size, params=params, seed=seed * 1000 + 1)
    acc.terrain(**t)
    plain = World(size, params=params, seed=seed * 1000 + 1)
    plain.terrain(**t)
    particles = size * size
    acc.tune(particles)  # the fastest launch form for this size (timed on a scratch copy)
    plain.tune(particles)
    rec = {"size": size, "jumps": jumps, "judge_every": judge_every, "tile": tile, "halo": halo,
           "particles_per_cycle": particles, "jump_cycles": JUMP_CYCLES, "steps": []}
    t_sur = t_judge = t_plain = 0.0
    for j in range(1, jumps + 1):
        judged = j % judge_every == 0
        t0 = time.time()
        if judged:
            acc.erode(particles, JUMP_CYCLES, mode=Mode.PARALLEL)
            dt = time.time() - t0
            t_judge += dt
        else:
            h = acc.height
            acc.upload(Field.HEIGHT, (h + predict_tiled(model, h, (wx, wz), tile, halo)).astype(np.float32))
            dt = time.time() - t0
            t_sur += dt
        t1 = time.time()
        plain.erode(particles, JUMP_CYCLES, mode=Mode.PARALLEL)
        t_plain += time.time() - t1
        step = {"jump": j, "by": "plain" if judged else "surrogate", "seconds": dt}
        if judged or j == jumps:
            step.update(compare(acc.height, plain.height))
        rec["steps"].append(step)
        log(json.dumps(step))
    rec["seconds"] = {"accelerated": t_sur + t_judge, "surrogate_jumps": t_sur, "judged_jumps": t_judge,
                      "plain_only": t_plain}
    rec["speedup_vs_plain_only"] = t_plain / max(t_sur + t_judge, 1e-12)
    acc.close()
    plain.close()
    return rec


def main(argv=None):
    from .train_surrogate import DEFAULT_OUT
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=4096)
    ap.add_argument("--jumps", type=int, default=40, help="50-cycle jumps (40: 2000 cycles)")
    ap.add_argument("--judge-every", type=int, default=4)
    ap.add_argument("--seed", type=int, default=5)
    ap.add_argument("--checkpoint", default=str(DEFAULT_OUT))
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    with np.load(a.checkpoint) as z:
        state = {k: z[k] for k in z.files if k != "meta"}
    model = Surrogate()
    model.load(state)
    rec = long_run(model, a.size, a.jumps, a.judge_every, a.seed)
    print(json.dumps(rec))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(rec, f)


if __name__ == "__main__":
    main()
