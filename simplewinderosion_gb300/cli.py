"""Headless command line version of the reference's app loop.

SimpleWindErosion.cpp seeds the world from its first argument (or the clock),
builds the map (map::init's Gaussian bump) and then, every frame it is not
paused, calls world.erode(8 * tilesize), refreshes the vertex pool from the
heights (updatenode) and rebuilds the wind map from the momentum fields,
printing a frame counter (SimpleWindErosion.cpp:27-34, 211-231). This runs
the same cadence on the GPU with no window: frames are counted instead of
rendered, and every --every frames the observables are written to --export:
height.npy, massflow.npy, windmap.npy (RGBA floats), windmap.ppm (8-bit RGB)
and, with --vertices, vertices.npy (updatenode's per-cell position, normal
and edges).

    python -m simplewinderosion_gb300.cli [SEED] [--size 512] [--frames 10]
        [--mode parallel|ordered] [--terrain bump|fbm] [--wind X,Y,Z]
        [--export DIR] [--every 1]
"""
from __future__ import annotations

import argparse
import sys
import time
from pathlib import Path

import numpy as np


def parse_args(argv=None):
    ap = argparse.ArgumentParser(prog="winderosion", description=__doc__.split("\n\n")[0])
    ap.add_argument("seed", nargs="?", type=int, default=None, help="world seed (default: the clock, as the app)")
    ap.add_argument("--size", type=int, default=512, help="map side (the reference's tilesize, 512)")
    ap.add_argument("--particles", type=int, default=0, help="particles per frame (default 8 * size)")
    ap.add_argument("--frames", type=int, default=10, help="frames to run")
    ap.add_argument("--mode", choices=["parallel", "ordered"], default="parallel")
    ap.add_argument("--lanes", type=int, default=0, help="parallel mode: particles in flight (0: default)")
    ap.add_argument("--wind", type=str, default=None,
                    help="prevailing wind X,Y,Z, normalised (default: the reference's Wind::pspeed, 1,0,0)")
    ap.add_argument("--terrain", choices=["bump", "fbm"], default="bump",
                    help="bump: the reference's map::init terrain; fbm: seeded fBm plus a sediment layer")
    ap.add_argument("--export", type=Path, default=None, help="directory for the observables")
    ap.add_argument("--every", type=int, default=1, help="export every N frames")
    ap.add_argument("--vertices", action="store_true", help="also export updatenode's vertices")
    ap.add_argument("--quiet", action="store_true", help="no frame counter")
    args = ap.parse_args(argv)
    if args.size < 1 or args.frames < 0 or args.every < 1:
        ap.error("size >= 1, frames >= 0 and every >= 1 are required")
    if args.wind is not None:
        try:
            w = [float(v) for v in args.wind.split(",")]
        except ValueError:
            w = []
        if len(w) != 3 or not any(w):
            ap.error("--wind takes three numbers X,Y,Z, not all zero")
        args.wind = tuple(w)
    return args


def write_ppm(path: Path, rgba: np.ndarray) -> None:
    """8-bit binary PPM of the RGB channels (values in [0, 1])."""
    nx, nz, _ = rgba.shape
    rgb = np.clip(np.rint(rgba[..., :3] * 255.0), 0, 255).astype(np.uint8)
    with open(path, "wb") as f:
        f.write(f"P6\n{nz} {nx}\n255\n".encode())
        f.write(rgb.tobytes())


def export(world, out: Path, frame: int, vertices: bool) -> None:
    import simplewinderosion_gb300 as swe
    d = out / f"frame_{frame:06d}"
    d.mkdir(parents=True, exist_ok=True)
    np.save(d / "height.npy", world.height)
    np.save(d / "massflow.npy", world.download(swe.Field.MASSFLOW))
    wm = world.windmap()
    np.save(d / "windmap.npy", wm)
    write_ppm(d / "windmap.ppm", wm)
    if vertices:
        np.save(d / "vertices.npy", world.vertices())


def main(argv=None) -> int:
    args = parse_args(argv)
    import simplewinderosion_gb300 as swe

    seed = args.seed if args.seed is not None else int(time.time())
    particles = args.particles or 8 * args.size
    mode = swe.Mode.PARALLEL if args.mode == "parallel" else swe.Mode.ORDERED
    params = swe.Params(lanes=args.lanes)
    if args.wind is not None:
        params = swe.Params(lanes=args.lanes, pspeed=swe.wind_direction(*args.wind))
    world = swe.World(args.size, params=params, seed=seed)
    try:
        if args.terrain == "bump":
            world.terrain()
        else:
            world.terrain(seed=seed, octaves=8, base_freq=4.0 / args.size, sediment=0.1, sediment_jitter=0.02)
        if not args.quiet:
            print(f"Seed: {seed}", flush=True)
        for frame in range(args.frames):
            world.erode(particles, 1, mode=mode)
            if not args.quiet:
                print(frame, flush=True)
            if args.export is not None and (frame + 1) % args.every == 0:
                export(world, args.export, frame, args.vertices)
        world.sync()
    except swe.SweError as e:
        print(f"winderosion: {e}", file=sys.stderr)
        return 1
    finally:
        world.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
