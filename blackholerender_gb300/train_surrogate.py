"""Trains the orbit surrogate on the GPU and writes a checkpoint.

    python -m blackholerender_gb300.train_surrogate [--orbits 1e7] [--steps 20000] [--out PATH]

Training data: orbits integrated by the library's FP64 RK4 kernel in the orbital plane, r_cam
log-uniform in [6, 200], b uniform in [0, 60] mixed with b dense near sqrt(27) (uniform in the
input transform), several samples along each orbit. Prints one JSON line (timings, losses).
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--orbits", type=float, default=1e7)
    ap.add_argument("--per-orbit", type=int, default=4)
    ap.add_argument("--steps", type=int, default=200000)
    ap.add_argument("--batch", type=int, default=16384)
    ap.add_argument("--lr-max", type=float, default=2e-3)
    ap.add_argument("--lr-min", type=float, default=1e-6)
    ap.add_argument("--w-capture", type=float, default=0.01)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    import torch

    from .surrogate import DEFAULT_CHECKPOINT, Surrogate

    out = a.out or str(DEFAULT_CHECKPOINT)
    s = Surrogate(seed=a.seed)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    counts = s.generate(int(a.orbits), per_orbit=a.per_orbit, seed=a.seed * 7919 + 1)
    t1 = time.perf_counter()
    hist = s.train(a.steps, batch=a.batch, lr_max=a.lr_max, lr_min=a.lr_min, w_c=a.w_capture, seed=a.seed)
    t2 = time.perf_counter()
    from pathlib import Path

    Path(out).parent.mkdir(parents=True, exist_ok=True)
    s.save(out)
    k = max(1, a.steps // 20)
    print(json.dumps({
        "orbits": int(a.orbits), "escaped": counts[0], "captured": counts[1], "unusable": counts[2],
        "generate_s": t1 - t0, "train_s": t2 - t1, "steps": a.steps, "batch": a.batch,
        "mse_first": float(hist[:k, 0].mean()), "mse_last": float(hist[-k:, 0].mean()),
        "rms_residual_rad_last": float(np.sqrt(hist[-k:, 0].mean()) * s.cfg.y_scale),
        "bce_last": float(hist[-k:, 1].mean()), "checkpoint": out,
    }), flush=True)


if __name__ == "__main__":
    main()
