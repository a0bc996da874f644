#!/usr/bin/env python3
"""Throughput of the per-pixel Schwarzschild tracer on GB300 (one JSON line on stdout).

Workload (one "step"): the 16 camera poses of the 1080p configuration (seed 0; r ~ U[15,60],
inclination ~ U[60,90] deg, azimuth ~ U[0,2 pi)), 1920x1080 each, FOV 60, 450-step budget
(High preset: step 0.05 r, disk step 0.18), thin disk r in [6,20], escape at r > 1000,
capture at r < 2.0001 -- 33.2 M rays per step. Inputs are camera views (no dataset exists);
outputs are 64-byte hit records (2.1 GB per step, larger than L2, and L2 is also flushed
between timed steps).

  value  Mrays/s of the traced rays, device-timed with CUDA events on the launch stream
  e2e    the same through bhr_trace_host: host views in, records in pinned host memory out,
         device->host copies inside the timed region
  roofline  the march kernel's FP32 FLOP rate (160 FLOP per executed step + 60 per ray)
         against a measured FP32 peak (cuBLAS SGEMM, TF32 off) -- the path is FP32-pipe bound
  cpu_baseline  the CPU restatement of the same march (oracle/, FP64) on all host cores,
         on a bounded sample of the same workload

--impl reference times that CPU march alone, on all host threads, as the reference arm.
Multi-GPU (torchrun): every rank traces its own copy of the 16 views (weak scaling, no
collective on the data path); rank 0 prints the max-over-ranks timing.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = json.loads((ROOT / "BASELINE.json").read_text())["metric"] if (ROOT / "BASELINE.json").exists() else \
    "Mrays/s at 1080p x 450 steps"
UNIT = "Mrays/s"
F_STEP = 160  # FP32 FLOP per executed march step (FMA = 2)
F_SETUP = 60  # FP32 FLOP per ray (ray generation, initial velocity, constants)
WORKLOAD = ("16 poses (seed 0) x 1920x1080, FOV 60, 450 steps (High preset), thin disk [6,20], "
            "escape r>1000, capture r<2.0001")


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------------------- CPU march
def _oracle():
    lib = ROOT / "oracle" / "_build" / "liboracle.so"
    if not lib.exists():
        subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "all"], check=True)
    return ctypes.CDLL(str(lib))


def cpu_march_sample(views, seconds: float, seed: int = 0, chunk: int = 32768):
    """The CPU march (FP64 restatement, all host threads) on random pixels of the views until
    `seconds` elapse; returns (Mrays/s, rays, threads, steps/ray)."""
    from blackholerender_gb300 import HIT_DTYPE

    L = _oracle()
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(seed)
    rays = 0
    steps = 0
    t0 = time.perf_counter()
    k = 0
    while True:
        v = views[k % len(views)]
        idx = np.ascontiguousarray(rng.choice(v.rays, chunk, replace=False), dtype=np.int64)
        out = np.zeros(chunk, dtype=HIT_DTYPE)
        rc = L.oracle_trace_pixels(ctypes.byref(v), ctypes.c_void_p(idx.ctypes.data), ctypes.c_int64(chunk),
                                   ctypes.c_void_p(out.ctypes.data), threads, 1)
        assert rc == 0
        rays += chunk
        steps += int(out["steps"].sum())
        k += 1
        dt = time.perf_counter() - t0
        if dt >= seconds:
            return rays / dt / 1e6, rays, threads, steps / rays


def cpu_model() -> str:
    try:
        for ln in Path("/proc/cpuinfo").read_text().splitlines():
            if ln.lower().startswith(("model name", "cpu part")):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


# ----------------------------------------------------------------------------- reference arm
def run_reference(args):
    from blackholerender_gb300 import TERM_CONFIG, workloads

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    views = workloads.c2_views(TERM_CONFIG)
    per_step_s = 4.0
    for _ in range(args.warmup):
        cpu_march_sample(views, 0.5, seed=99)
    vals = []
    rays_total = 0
    t0 = time.perf_counter()
    for s in range(args.steps):
        v, rays, threads, spr = cpu_march_sample(views, per_step_s, seed=s)
        vals.append(v)
        rays_total += rays
    wall = time.perf_counter() - t0
    value = rays_total / wall / 1e6
    sample = (f"random pixels of the 16 poses, {per_step_s:.0f} s of CPU march per step "
              f"({rays_total / max(args.steps, 1):.0f} rays/step), FP64 restatement of the shader march")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall * 1e3 / max(args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "path": "CPU march, oracle/ restatement (reference's CPU integrator "
                   "rule set; the shader itself cannot run here)", "cpu": cpu_model()},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- GPU arm
def fp32_peak_tflops(dev) -> float:
    import torch

    torch.backends.cuda.matmul.allow_tf32 = False
    n = 8192
    a = torch.randn(n, n, device=dev)
    b = torch.randn(n, n, device=dev)
    for _ in range(2):
        a @ b
    torch.cuda.synchronize(dev)
    best = 1e30
    for _ in range(5):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        a @ b
        e1.record()
        torch.cuda.synchronize(dev)
        best = min(best, e0.elapsed_time(e1))
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def run_gpu(args):
    import torch

    from blackholerender_gb300 import HIT_BYTES, PREC_FP32, TERM_CONFIG, Tracer, workloads

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    views = workloads.c2_views(TERM_CONFIG)
    rays = sum(v.rays for v in views)
    tr = Tracer(local, block_size=args.block, chunk=args.chunk, refill=args.refill)
    outs = [torch.empty(v.rays * HIT_BYTES, dtype=torch.uint8, device=dev) for v in views]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step():
        if args.launch == "multi":
            tr.trace(views, outs, PREC_FP32, stream=stream)
            return 1
        for v, o in zip(views, outs):
            tr.trace([v], [o], PREC_FP32, stream=stream)
        return len(views)

    for _ in range(max(args.warmup, 0)):
        step()
    torch.cuda.synchronize(dev)
    # executed steps of one pass (identical every pass: the march is deterministic)
    if args.launch == "multi":
        tr.trace(views, outs, PREC_FP32, stream=stream)
        steps_exec = tr.stats().steps
    else:
        steps_exec = 0
        for v, o in zip(views, outs):
            tr.trace([v], [o], PREC_FP32, stream=stream)
            steps_exec += tr.stats().steps
    torch.cuda.synchronize(dev)

    if dist:
        dist.barrier()
    torch.cuda.synchronize(dev)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    launches = 0
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            flush.zero_()  # evict L2 between timed steps (outside the timed events)
            ev[k][0].record(stream)
            launches += step()
            ev[k][1].record(stream)
        torch.cuda.synchronize(dev)
    if dist:
        dist.barrier()
    per_step = [a.elapsed_time(b) for a, b in ev]
    total_ms = sum(per_step)
    if dist:
        t = torch.tensor([total_ms], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_per_step = total_ms / args.steps
    value = rays * world / (ms_per_step * 1e-3) / 1e6

    # ---- end to end through the host-buffer entry point
    host = [torch.empty(v.rays * HIT_BYTES, dtype=torch.uint8, pin_memory=True) for v in views]
    host_np = [h.numpy() for h in host]
    tr.trace_host(views, host_np, PREC_FP32)
    e2e_steps = max(2, min(args.steps, 5))
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        tr.trace_host(views, host_np, PREC_FP32)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    if dist:
        t = torch.tensor([e2e_s], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = {"value": rays * world / e2e_s / 1e6, "unit": UNIT,
           "h2d_bytes_per_step": len(views) * 160, "d2h_bytes_per_step": rays * HIT_BYTES,
           "ms_per_step": e2e_s * 1e3, "api": "bhr_trace_host (pinned host records)"}

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    # ---- roofline of the march kernel
    flop = steps_exec * F_STEP + rays * F_SETUP
    ms_per_launch = ms_per_step * (1 if args.launch == "multi" else 1.0 / len(views))
    flop_per_launch = flop if args.launch == "multi" else flop / len(views)
    achieved = flop_per_launch / (ms_per_launch * 1e-3) / 1e12
    peak_meas = fp32_peak_tflops(dev)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    nominal = sms * 128 * 2 * 2.07e9 / 1e12
    traffic = None
    tfile = ROOT / "profiles" / "traffic.json"
    if tfile.exists():
        try:
            traffic = json.loads(tfile.read_text()).get(f"k_march_{args.launch}")
        except Exception:
            traffic = None
    roof = {"bound": "fp32", "achieved": achieved, "peak": peak_meas, "unit": "TFLOP/s",
            "frac": achieved / peak_meas, "traffic": traffic,
            "peak_source": "measured in this run: cuBLAS SGEMM 8192^3, TF32 off (FP32 FMA pipe)",
            "nominal_peak": nominal, "frac_of_nominal": achieved / nominal,
            "flop_per_launch": flop_per_launch, "ms_per_launch": ms_per_launch,
            "algorithm": f"{F_STEP} FLOP per executed step + {F_SETUP} per ray; {steps_exec / rays:.2f} steps/ray"}

    cpu = None
    if not args.no_cpu and world == 1:
        v_cpu, n_cpu, thr, spr = cpu_march_sample(views, args.cpu_seconds)
        cpu = {"value": v_cpu, "unit": UNIT, "cores": thr, "kind": "port",
               "sample": f"{n_cpu} random pixels of the 16 poses ({args.cpu_seconds:.0f} s), FP64 CPU restatement "
                         f"of the march, {spr:.1f} steps/ray, {cpu_model()}"}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "views": len(views), "rays_per_step": rays, "method": "plain",
                   "launch": args.launch, "l2": "inputs are camera views; 2.1 GB of records per step and a "
                   "256 MiB L2 flush between timed steps", "parallelism": f"replicas x{world}"},
        "e2e": e2e,
        "gpu_launches": launches,
        "roofline": roof,
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "steps_per_ray": steps_exec / rays,
        "per_step_ms": per_step,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--launch", default="multi", choices=["multi", "one"])
    ap.add_argument("--block", type=int, default=0)
    ap.add_argument("--chunk", type=int, default=0)
    ap.add_argument("--refill", type=int, default=0)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        log("note: fewer than 3 warm-up steps")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
