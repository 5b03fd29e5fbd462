"""Autotuner of the launch shapes of the GB300 path.

Tunable without recompiling (eqd_options):
  tile_shape   the brick of 128 elements behind each binary32 tile (bx, by, bz): it sets the number
               of distinct nodes a tile gathers and the locality of those gathers;
  block_node   node-update block size;
  block_fault  fault-kernel block size.

The search is coordinate descent (tile shape, then node block, then fault block) on a scaled copy
of a configuration (same shapes, fewer elements), timing each candidate with CUDA events over a
few steps after a warm-up; each candidate is a fresh context.  The result is written as JSON under
eqdyna_gb300/tuning/ keyed by GPU name and configuration, and `tuned_options` reads it back.

    python -m eqdyna_gb300.autotune --config C1 --scale 2
"""
import argparse
import json
import os
import shutil
import subprocess
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
TUNING_DIR = os.path.join(HERE, "tuning")

TILE_SHAPES = [(4, 8, 4), (4, 4, 8), (8, 4, 4), (2, 8, 8), (8, 8, 2), (8, 2, 8), (2, 16, 4), (4, 16, 2)]
BLOCK_NODE = [128, 256, 512]
BLOCK_FAULT = [32, 64, 128]


def pack_tile(shape):
    bx, by, bz = shape
    return bx | by << 8 | bz << 16


def gpu_name(device=0):
    try:
        out = subprocess.run(["nvidia-smi", "-i", str(device), "--query-gpu=name", "--format=csv,noheader"],
                             stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True, timeout=30)
        name = out.stdout.strip().splitlines()[0] if out.stdout.strip() else "unknown"
    except (OSError, subprocess.SubprocessError):
        name = "unknown"
    return name


def _slug(s):
    return "".join(ch if ch.isalnum() else "_" for ch in s).strip("_").lower()


def tuning_path(config, gpu):
    return os.path.join(TUNING_DIR, f"{_slug(gpu)}_{config}.json")


def measure(case, precision, options, steps=16, warmup=3, device=0):
    """Device time per step (ms, the production path: graphs and the overlapped fault phase) and
    per-kernel shares (per-launch events, the reference's order) of a fresh context."""
    from .solver import GpuSolver
    with GpuSolver(case.clone(), precision=precision, device=device, **options) as s:
        s.step(warmup)
        s.profile(True, reset=True)
        s.step(steps)
        s.profile(False)
        kt = s.kernel_times()
        s.profile(True, reset=True, calls_only=True)
        s.step(steps)
        s.profile(False)
        total = s.kernel_times()["step"][0]
    seq = kt["step"][0]
    return total / steps, {k: round(v[0] / seq, 4) for k, v in kt.items() if k != "step"}


def tune(case, precision="fp32", steps=16, warmup=3, device=0, log=print):
    best = {"tile_shape": pack_tile(TILE_SHAPES[0]), "block_node": 256, "block_fault": 128}
    trials = []

    def run(opts):
        ms, share = measure(case, precision, opts, steps, warmup, device)
        trials.append({"options": dict(opts), "ms_per_step": ms, "share": share})
        log(f"  {opts} -> {ms:.4f} ms/step")
        return ms

    best_ms = run(best)
    for key, values in (("tile_shape", [pack_tile(t) for t in TILE_SHAPES]), ("block_node", BLOCK_NODE),
                        ("block_fault", BLOCK_FAULT)):
        for v in values:
            if v == best[key]:
                continue
            cand = dict(best, **{key: v})
            ms = run(cand)
            if ms < best_ms:
                best, best_ms = cand, ms
    return best, best_ms, trials


def tuned_options(config, device=0):
    """The tuned launch options for this GPU and configuration, or {} when none were recorded."""
    path = tuning_path(config, gpu_name(device))
    if not os.path.exists(path):
        return {}
    with open(path) as f:
        return dict(json.load(f)["best"])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="C1")
    ap.add_argument("--scale", type=float, default=2.0, help="coarsening of the tuning proxy")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--steps", type=int, default=16)
    ap.add_argument("--device", type=int, default=0)
    args = ap.parse_args()
    from . import configs
    from .case import Case
    tmp = tempfile.mkdtemp(prefix="eqd_tune_")
    configs.CONFIGS[args.config](tmp, scale=args.scale, nsteps=args.steps + 8)
    case = Case.from_dir(tmp)
    shutil.rmtree(tmp, ignore_errors=True)
    t0 = time.perf_counter()
    best, best_ms, trials = tune(case, args.precision, steps=args.steps, device=args.device)
    gpu = gpu_name(args.device)
    os.makedirs(TUNING_DIR, exist_ok=True)
    out = {"gpu": gpu, "config": args.config, "proxy_scale": args.scale, "precision": args.precision,
           "elements": case.sizes["nelem"], "best": best, "best_ms_per_step": best_ms,
           "tile_shape_xyz": [best["tile_shape"] & 255, (best["tile_shape"] >> 8) & 255,
                              (best["tile_shape"] >> 16) & 255],
           "trials": trials, "tuning_s": round(time.perf_counter() - t0, 1)}
    with open(tuning_path(args.config, gpu), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps({k: out[k] for k in ("gpu", "config", "best", "best_ms_per_step", "tuning_s")}))


if __name__ == "__main__":
    main()
