"""Training and evaluation of the learned surrogate at the density the
headline metric is quoted on: 1024^2 maps with 1,048,576 particles per
erode cycle (one per cell), jumps of 50 cycles.

    python -m simplewinderosion_gb300.train_surrogate [--runs R] [--eval-runs E] [--steps S] [--out PATH]

1. Data: R + E plain-method runs (PARALLEL mode, Q16.16) of 50 cycles x
   size^2 particles (the training runs with cells/64 particles in flight,
   four times faster than the default cells/256 and statistically close to
   it; the held-out runs with the default) on seeded device terrains (fBm of
   base frequency 1/256 with persistence U[0.4, 0.6] in [0, 0.5], 0.1 +-
   0.02 sediment, 0-3 bedrock pyramids of height 0.2-0.5 and base 100-300
   cells) with random wind angles. Each run gives the pair (initial heights,
   change after 50 cycles).
2. Training: Adam on random 256^2 crops of the R training pairs with the
   eight symmetries of the square applied to map and wind together (the
   erosion rules treat the grid's axes alike), batch 32, the change scaled
   to unit variance.
3. Evaluation on the E held-out runs, whole 1024^2 maps: height RMSE of the
   surrogate's jump against the plain method, relative to the plain
   result's height range; the same for "no change"; and the plain method's
   own seed-to-seed spread (each held-out start eroded again with other
   random numbers): no predictor of a stochastic result can beat that floor.

The checkpoint (weights, scale, and these numbers) goes to --out as .npz.
"""
from __future__ import annotations

import argparse
import json
import time
from pathlib import Path

import numpy as np

from . import Field, Mode, Params, World, wind_direction
from .surrogate import Surrogate, rmse

DEFAULT_OUT = Path(__file__).resolve().parent / "data" / "surrogate_1024.npz"


def run_terrain(rs: np.random.RandomState, size: int):
    """Random terrain settings for one run (device generator arguments)."""
    npyr = int(rs.randint(0, 4))
    pyr = []
    for _ in range(npyr):
        pyr.append((rs.uniform(0.15, 0.85) * size, rs.uniform(0.15, 0.85) * size, rs.uniform(0.2, 0.5),
                    rs.uniform(100, 300) * size / 1024))
    return {"seed": int(rs.randint(1, 2 ** 31)), "octaves": 8, "base_freq": 1.0 / 256.0 * 1024 / size,
            "persistence": float(rs.uniform(0.4, 0.6)), "sediment": 0.1, "sediment_jitter": 0.02, "pyramids": pyr}


def plain_runs(count: int, size: int = 1024, cycles: int = 50, seed: int = 0, erosion_seeds=(1,), lanes: int = 0,
               log=print):
    """`count` plain-method runs with `lanes` particles in flight (0: the
    library's default): returns h0 [count,size,size], wind_xz [count,2] and,
    per erosion seed, h_after [count,size,size] (float32)."""
    rs = np.random.RandomState(seed)
    h0 = np.empty((count, size, size), np.float32)
    wind = np.empty((count, 2), np.float32)
    after = {e: np.empty((count, size, size), np.float32) for e in erosion_seeds}
    for i in range(count):
        ang = rs.uniform(0.0, 2.0 * np.pi)
        wx, wy, wz = wind_direction(float(np.cos(ang)), 0.0, float(np.sin(ang)))
        wind[i] = (wx, wz)
        t = run_terrain(rs, size)
        for e in erosion_seeds:
            t0 = time.time()
            w = World(size, params=Params(pspeed=(wx, wy, wz), frac_bits=16, lanes=lanes),
                      seed=int(seed * 100003 + i * 131 + e))
            w.terrain(**t)
            if e == erosion_seeds[0]:
                h0[i] = w.height
            w.erode(size * size, cycles, mode=Mode.PARALLEL)
            after[e][i] = w.height
            w.close()
            log(f"run {i + 1}/{count} erosion seed {e}: {time.time() - t0:.1f} s")
    return h0, wind, after


_SYMS = [(t, fx, fz) for t in (False, True) for fx in (False, True) for fz in (False, True)]


def transform(a: np.ndarray, wind_xz, sym):
    """One of the eight symmetries of the square on a map [..., x, z] and its
    wind (x, z): optional transpose, then flips of x and z."""
    t, fx, fz = sym
    wx, wz = float(wind_xz[0]), float(wind_xz[1])
    if t:
        a = np.swapaxes(a, -1, -2)
        wx, wz = wz, wx
    if fx:
        a = a[..., ::-1, :]
        wx = -wx
    if fz:
        a = a[..., :, ::-1]
        wz = -wz
    return a, (wx, wz)


def train(model: Surrogate, h0, wind, dh, steps: int, batch: int = 32, crop: int = 256, lr: float = 1e-3,
          seed: int = 0, log=print):
    torch = model.torch
    rs = np.random.RandomState(seed)
    n, size, _ = h0.shape
    losses = []
    t0 = time.time()
    for step in range(steps):
        hb = np.empty((batch, crop, crop), np.float32)
        db = np.empty((batch, crop, crop), np.float32)
        wb = np.empty((batch, 2), np.float32)
        for b in range(batch):
            i = rs.randint(n)
            x0, z0 = rs.randint(0, size - crop + 1, size=2)
            sym = _SYMS[rs.randint(8)]
            pair = np.stack([h0[i, x0:x0 + crop, z0:z0 + crop], dh[i, x0:x0 + crop, z0:z0 + crop]])
            pair, wxz = transform(pair, wind[i], sym)
            hb[b], db[b] = pair[0], pair[1]
            wb[b] = wxz
        dev = model.device
        lr_t = lr * (0.5 * (1.0 + np.cos(np.pi * step / steps)) * 0.9 + 0.1)
        loss = model.train_step(torch.from_numpy(hb).to(dev), torch.from_numpy(wb).to(dev),
                                torch.from_numpy(db).to(dev), lr=float(lr_t))
        losses.append(loss)
        if step % 200 == 0 or step == steps - 1:
            log(f"step {step}: loss {np.mean(losses[-50:]):.5f} ({time.time() - t0:.0f} s)")
    model.ops.status()
    return losses


def predict_map(model: Surrogate, h, wind_xz):
    """The surrogate's height change over one jump for one whole map."""
    torch = model.torch
    hd = torch.from_numpy(np.ascontiguousarray(h[None], np.float32)).to(model.device)
    wd = torch.tensor([list(wind_xz)], dtype=torch.float32, device=model.device)
    return model.predict(hd, wd)[0].cpu().numpy()


def evaluate(model: Surrogate, h0, wind, after_a, after_b) -> dict:
    """Relative height RMSE (RMSE / the plain result's height range) of the
    surrogate, of no change, and of a second plain run, per held-out run."""
    sur, none, floor = [], [], []
    for i in range(h0.shape[0]):
        plain = after_a[i]
        rng = max(float(plain.max() - plain.min()), 1e-12)
        pred = h0[i] + predict_map(model, h0[i], wind[i])
        sur.append(rmse(pred, plain) / rng)
        none.append(rmse(h0[i], plain) / rng)
        floor.append(rmse(after_b[i], plain) / rng)
    return {"surrogate_rel_rmse": float(np.mean(sur)), "no_change_rel_rmse": float(np.mean(none)),
            "plain_seed_floor_rel_rmse": float(np.mean(floor)), "per_run": {"surrogate": sur, "no_change": none,
                                                                              "floor": floor}}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--runs", type=int, default=16)
    ap.add_argument("--eval-runs", type=int, default=2)
    ap.add_argument("--size", type=int, default=1024)
    ap.add_argument("--cycles", type=int, default=50)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--data-lanes", type=int, default=-64,
                    help="particles in flight of the training runs (-64: cells/64, four times the default's, "
                         "faster; 0: the default); the held-out runs always use the default")
    ap.add_argument("--out", default=str(DEFAULT_OUT))
    a = ap.parse_args(argv)
    t0 = time.time()
    data_lanes = a.size * a.size // 64 if a.data_lanes == -64 else a.data_lanes
    h0, wind, after = plain_runs(a.runs, a.size, a.cycles, seed=a.seed + 1, lanes=data_lanes)
    dh = after[1] - h0
    e0, ewind, eafter = plain_runs(a.eval_runs, a.size, a.cycles, seed=a.seed + 1000, erosion_seeds=(1, 2))
    data_s = time.time() - t0
    scale = float(1.0 / max(float(dh.std()), 1e-6))
    model = Surrogate(seed=a.seed, scale=scale)
    t1 = time.time()
    train(model, h0, wind, dh, a.steps, batch=a.batch, seed=a.seed)
    train_s = time.time() - t1
    ev = evaluate(model, e0, ewind, eafter[1], eafter[2])
    meta = {"size": a.size, "cycles": a.cycles, "particles_per_cycle": a.size * a.size, "train_runs": a.runs,
            "train_lanes": data_lanes, "eval_lanes": "default",
            "eval_runs": a.eval_runs, "steps": a.steps, "batch": a.batch, "crop": 256, "data_s": data_s,
            "train_s": train_s, "height_ref": model.height_ref,
            **{k: v for k, v in ev.items() if k != "per_run"}}
    print(json.dumps(meta))
    out = Path(a.out)
    out.parent.mkdir(parents=True, exist_ok=True)
    st = model.state()
    np.savez_compressed(out, meta=json.dumps(meta), **st)
    print(f"wrote {out}")


if __name__ == "__main__":
    main()
