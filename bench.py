#!/usr/bin/env python3
"""Throughput of the per-pixel Schwarzschild tracer on GB300 (one JSON line on stdout).

Workload (one "step"): the 16 camera poses of the 1080p configuration (seed 0; r ~ U[15,60],
inclination ~ U[60,90] deg, azimuth ~ U[0,2 pi)), 1920x1080 each, FOV 60, 450-step budget
(High preset: step 0.05 r, disk step 0.18), thin disk r in [6,20], escape at r > 1000,
capture at r < 2.0001 -- 33.2 M rays per step. Inputs are camera views (no dataset exists);
outputs are 64-byte hit records (2.1 GB per step, larger than L2, and L2 is also flushed
between timed steps).

  value  Mrays/s of the learned-surrogate path (network + closed-form orbit, with the plain
         integrator as fallback for near-critical, outgoing and out-of-range rays), device-timed
         with CUDA events on the launch stream; the plain FP32 integrator on the same 16 views is
         timed right after it, into its own records (paths.plain_mrays_s)
  e2e    the same through bhr_surrogate_trace_host: host views in, records in pinned host memory
         out, device->host copies inside the timed region
  roofline  the surrogate pass against the measured HBM bandwidth (its algorithmic work is the 64-B
         hit record per ray; the network runs only in the views' tables, whose BF16 figures ride
         along in roofline.tensor);
         roofline_plain: the plain march against a measured FP32 peak (160 FLOP per executed step
         + 60 per ray, cuBLAS SGEMM with TF32 off as the FP32 denominator)
  cpu_baseline  the CPU restatement of the same march (oracle/, FP64) on all host cores,
         over every ray of the step (about 9 s on 16 cores)
  accuracy  that CPU march then checks both GPU paths' records ray by ray: classification
         mismatches over the whole step (class_mismatch_full), and, on every ray where the two
         paths' directions differ by more than 5e-5 rad, both against the converged FP64 orbit
         (surrogate_worst_vs_converged_rad)

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
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mrays/s at 1080p×450 steps: surrogate vs plain kernel, GB300, ≤1e-4 rad err"
UNIT = "Mrays/s"
F_STEP = 160  # FP32 FLOP per executed march step (FMA = 2)
F_SETUP = 60  # FP32 FLOP per ray (ray generation, initial velocity, constants)
F_MLP = 2 * (3 * 64 + 64 * 64 + 64 * 64 + 64 * 2)  # BF16-equivalent FLOP per network query
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
        self.lines = []
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "50",
                 "-i", str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True, bufsize=1)
        except OSError:
            self.proc = None
            return self
        self.reader = threading.Thread(target=self._read, daemon=True)
        self.reader.start()
        return self

    def _read(self):
        for ln in self.proc.stdout:
            if ln.strip():
                self.lines.append(ln)

    def samples(self) -> int:
        return len(self.lines)

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.proc.wait()
            self.reader.join(timeout=5)

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


SQRT27 = 27.0 ** 0.5


def _near_edge(h, r_in: float, r_out: float, rel: float) -> np.ndarray:
    near = np.zeros(len(h), dtype=bool)
    for k in range(3):
        r = h["cross_r"][:, k].astype(np.float64)
        near |= (k < h["ncross"]) & ((np.abs(r - r_in) < rel * r_in) | (np.abs(r - r_out) < rel * r_out))
    return near


def class_mismatches(gpu, ref, view, band: float, edge_rel: float):
    """(mismatches, compared): rays whose classification (status, and disk yes/no) differs from
    the oracle's, among the rays outside the ill-conditioned sets: |b - sqrt 27| < band, the
    oracle's ray ending within 2 steps of the budget, a crossing within edge_rel of a disk edge."""
    amb = np.abs(ref["b"].astype(np.float64) - SQRT27) < band
    amb |= np.abs(ref["steps"].astype(np.int64) - view.max_steps) <= 2
    amb |= _near_edge(ref, view.disk_inner, view.disk_outer, edge_rel)
    amb |= _near_edge(gpu, view.disk_inner, view.disk_outer, edge_rel)
    same = (gpu["status"] == ref["status"]) & ((gpu["ncross"] > 0) == (ref["ncross"] > 0))
    return int((~amb & ~same).sum()), int((~amb).sum())


def _angle(a, b) -> np.ndarray:
    a = a.astype(np.float64)
    b = b.astype(np.float64)
    return np.arctan2(np.linalg.norm(np.cross(a, b), axis=1), np.sum(a * b, axis=1))


def cpu_baseline_and_check(views, outs_s, outs_p, outs_c, disagree_rad: float = 5e-5, sample: int = 2000):
    """The cpu_baseline leg over the whole step: the FP64 CPU restatement of the march on every
    ray of the 16 views, on all host threads (timed: the CPU baseline), used afterwards as the
    checker of both GPU paths' records (the surrogate path's in outs_s, the plain FP32 path's in
    outs_p): classification of every ray, and the converged FP64 orbit (step scale 0.002, no slab
    clamp) on every ray where the two GPU paths' escape directions differ by more than
    disagree_rad. The non-learned comparator's records (outs_c) get the same classification check,
    and both surrogate variants are compared with the converged orbit on `sample` random rays
    per view. Returns (cpu_baseline, accuracy)."""
    from blackholerender_gb300 import FLAG_SURROGATE, HIT_DTYPE, hits_numpy

    L = _oracle()
    threads = os.cpu_count() or 1
    t_cpu, t_conv, rays, steps = 0.0, 0.0, 0, 0
    acc = {"class_mismatch_full": 0, "class_mismatch_full_plain": 0, "rays_compared": 0, "rays_compared_plain": 0,
           "disagreeing_rays": 0, "converged_checked": 0, "surrogate_worst_vs_converged_rad": 0.0,
           "plain_worst_vs_converged_rad": 0.0, "class_mismatch_full_closed_form": 0}
    agree, samp_s, samp_c = [], [], []
    rng = np.random.default_rng(0)
    for v, so, po, co in zip(views, outs_s, outs_p, outs_c):
        ref = np.zeros(v.rays, dtype=HIT_DTYPE)
        t0 = time.perf_counter()
        rc = L.oracle_trace_view(ctypes.byref(v), ctypes.c_void_p(ref.ctypes.data), threads, 1)
        t_cpu += time.perf_counter() - t0
        assert rc == 0
        rays += v.rays
        steps += int(ref["steps"].astype(np.int64).sum())
        gs = hits_numpy(so.cpu())
        gp = hits_numpy(po.cpu())
        m, n = class_mismatches(gs, ref, v, 2e-3, 1e-3)
        acc["class_mismatch_full"] += m
        acc["rays_compared"] += n
        m, n = class_mismatches(gp, ref, v, 1e-2, 1e-4)
        acc["class_mismatch_full_plain"] += m
        acc["rays_compared_plain"] += n
        gc = hits_numpy(co.cpu())
        acc["class_mismatch_full_closed_form"] += class_mismatches(gc, ref, v, 2e-3, 1e-3)[0]
        fine = v.copy()
        fine.step_scale, fine.ds_floor, fine.max_steps, fine.disk_mode = 0.002, 1e-4, 200000, 0
        idx = np.ascontiguousarray(np.sort(rng.choice(v.rays, sample, replace=False)), dtype=np.int64)
        conv = np.zeros(len(idx), dtype=HIT_DTYPE)
        rc = L.oracle_trace_pixels(ctypes.byref(fine), ctypes.c_void_p(idx.ctypes.data), ctypes.c_int64(len(idx)),
                                   ctypes.c_void_p(conv.ctypes.data), threads, 1)
        assert rc == 0
        ok = (conv["status"] == 1) & ((gs["flags"][idx] & FLAG_SURROGATE) != 0) & ((gc["flags"][idx] & FLAG_SURROGATE) != 0)
        samp_s.append(_angle(gs["dir"][idx][ok], conv["dir"][ok]))
        samp_c.append(_angle(gc["dir"][idx][ok], conv["dir"][ok]))
        both = np.nonzero(((gs["flags"] & FLAG_SURROGATE) != 0) & (gs["status"] == 1) & (gp["status"] == 1))[0]
        a = _angle(gs["dir"][both], gp["dir"][both])
        agree.append(a)
        idx = np.ascontiguousarray(both[a > disagree_rad], dtype=np.int64)
        acc["disagreeing_rays"] += len(idx)
        if len(idx):
            fine = v.copy()
            fine.step_scale, fine.ds_floor, fine.max_steps, fine.disk_mode = 0.002, 1e-4, 200000, 0
            conv = np.zeros(len(idx), dtype=HIT_DTYPE)
            t0 = time.perf_counter()
            rc = L.oracle_trace_pixels(ctypes.byref(fine), ctypes.c_void_p(idx.ctypes.data), ctypes.c_int64(len(idx)),
                                       ctypes.c_void_p(conv.ctypes.data), threads, 1)
            t_conv += time.perf_counter() - t0
            assert rc == 0
            ok = conv["status"] == 1
            acc["converged_checked"] += int(ok.sum())
            es = _angle(gs["dir"][idx][ok], conv["dir"][ok])
            ep = _angle(gp["dir"][idx][ok], conv["dir"][ok])
            acc["surrogate_worst_vs_converged_rad"] = max(acc["surrogate_worst_vs_converged_rad"],
                                                          float(es.max(initial=0.0)))
            acc["plain_worst_vs_converged_rad"] = max(acc["plain_worst_vs_converged_rad"], float(ep.max(initial=0.0)))
    agree = np.concatenate(agree)
    samp_s, samp_c = np.concatenate(samp_s), np.concatenate(samp_c)
    acc["sample_vs_converged_rad"] = {
        "rays": int(len(samp_s)),
        "learned": {"p50": float(np.percentile(samp_s, 50)), "p99": float(np.percentile(samp_s, 99)),
                    "max": float(samp_s.max())},
        "closed_form": {"p50": float(np.percentile(samp_c, 50)), "p99": float(np.percentile(samp_c, 99)),
                        "max": float(samp_c.max())}}
    acc["agreement_vs_plain_fp32_rad"] = {"p50": float(np.percentile(agree, 50)), "p99": float(np.percentile(agree, 99)),
                                          "max": float(agree.max()), "rays": int(len(agree))}
    acc["converged_s"] = t_conv
    acc["note"] = ("every ray of the step against the FP64 oracle of the same rule: classification outside the "
                   "photon-sphere band (2e-3 surrogate path, 1e-2 plain), the budget's last 2 steps and disk-edge "
                   "crossings; on the rays where the two GPU paths differ by more than 5e-5 rad, both against the "
                   "converged FP64 orbit (step scale 0.002)")
    cpu = {"value": rays / t_cpu / 1e6, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"every ray of the step ({rays} rays, {t_cpu:.1f} s), FP64 CPU restatement of the march, "
                     f"{steps / rays:.1f} steps/ray, {cpu_model()}"}
    return cpu, acc


def cpu_model() -> str:
    try:
        for ln in Path("/proc/cpuinfo").read_text().splitlines():
            if ln.lower().startswith(("model name", "cpu part")):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def oracle_c2_views(term_mode: int):
    """The 16 poses' views built by the oracle (no product library mapped); byte-equal to the
    library's views (tests/test_cpu_host.py)."""
    from blackholerender_gb300 import View, workloads

    L = _oracle()
    L.oracle_orbit_view.argtypes = [ctypes.POINTER(View), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_float, ctypes.c_double, ctypes.c_double, ctypes.c_double]
    out = []
    for r, inc, az in workloads.c2_poses():
        v = View()
        assert L.oracle_orbit_view(ctypes.byref(v), term_mode, 2, 1920, 1080, 60.0, r, inc, az) == 0
        out.append(v)
    return out


def step_config(views) -> dict:
    """The `config` both arms print: the workload of one step."""
    rays = sum(v.rays for v in views)
    return {"workload": WORKLOAD if len(views) == 16 else f"first {len(views)} of: {WORKLOAD}",
            "views": len(views), "rays_per_step": rays,
            "l2": "inputs are camera views; 2.1 GB of records per step and a 256 MiB L2 flush between timed steps"}


# ----------------------------------------------------------------------------- reference arm
def run_reference(args):
    from blackholerender_gb300 import TERM_CONFIG

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    views = oracle_c2_views(TERM_CONFIG)[:args.views]
    # a bounded sample per step: 4 s of CPU march, less when many steps are asked for, so that the
    # whole run stays within about three minutes
    per_step_s = max(0.25, min(4.0, 180.0 / max(args.steps, 1)))
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
    sample = (f"random pixels of the 16 poses, {per_step_s:.2f} s of CPU march per step "
              f"({rays_total / max(args.steps, 1):.0f} rays/step), FP64 restatement of the shader march")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall * 1e3 / max(args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": step_config(views),
        "path": "CPU march, oracle/ restatement of the shader march (FP64; the shader itself cannot run here); "
                "views built by the oracle, no product library loaded",
        "cpu": cpu_model(),
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
    from blackholerender_gb300.surrogate import DEFAULT_CHECKPOINT, Surrogate

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
    views = workloads.c2_views(TERM_CONFIG)[:args.views]
    rays = sum(v.rays for v in views)
    tr = Tracer(local, block_size=args.block, chunk=args.chunk, refill=args.refill)
    sur = Surrogate(device=local, seed=2)
    trained_here = None
    if DEFAULT_CHECKPOINT.exists() and not args.retrain:
        sur.load(DEFAULT_CHECKPOINT)
    else:  # train on this GPU with the library's own kernels (about 30 s)
        t0 = time.perf_counter()
        sur.generate(10_000_000, per_orbit=4, seed=7920)
        sur.train(200_000, batch=16384, lr_max=2e-3, lr_min=1e-6)
        trained_here = time.perf_counter() - t0
    outs = [torch.empty(v.rays * HIT_BYTES, dtype=torch.uint8, device=dev) for v in views]
    outs_p = [torch.empty(v.rays * HIT_BYTES, dtype=torch.uint8, device=dev) for v in views]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    # both paths as the library's CUDA-graph plans (one graph launch per step), each into its own
    # records; the plain path with the launch shape its autotuner picks for these views
    sur.trace_ptrs(views, outs, stream)
    torch.cuda.synchronize(dev)
    plan_s = sur.plan(views, outs)
    plan_p = tr.plan(views, outs_p, PREC_FP32, autotune=True)
    plain_shape = plan_p.launch_shape.as_dict()

    def step_surrogate():
        plan_s.launch(stream)
        # one table launch per 64 views (every view's exit and crossing tables), one pass per
        # view, one fallback march for all views, and the band search and band march (one launch
        # each for up to 64 views that share one rule, as these do)
        return (len(views) + 63) // 64 + len(views) + 1 + (2 if len(views) <= 64 else 0)

    def step_plain():
        plan_p.launch(stream)
        return 1

    for _ in range(max(args.warmup, 0)):
        step_plain()
        step_surrogate()
    torch.cuda.synchronize(dev)

    step_surrogate()
    torch.cuda.synchronize(dev)
    st = sur.trace_stats()
    # phase times of one (eager) surrogate trace (dominant kernel: the surrogate pass)
    sur.trace_ptrs(views, outs, stream)
    t_pass, t_fb = sur.trace_times_ms()

    def timed(step, k_steps):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k_steps)]
        launches = 0
        for k in range(k_steps):
            flush.zero_()  # evict L2 between timed steps (outside the timed events)
            ev[k][0].record(stream)
            launches += step()
            ev[k][1].record(stream)
        torch.cuda.synchronize(dev)
        return [a.elapsed_time(b) for a, b in ev], launches

    if dist:
        dist.barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clk:
        t_wait = time.perf_counter()  # keep the GPU loaded until the sampler reports (<= 3 s, untimed)
        while clk.samples() < 2 and time.perf_counter() - t_wait < 3.0:
            step_surrogate()
            torch.cuda.synchronize(dev)
        per_step, launches = timed(step_surrogate, args.steps)
    if dist:
        dist.barrier()
    total_ms = sum(per_step)
    per_plain, _ = timed(step_plain, args.steps)
    plain_ms = sum(per_plain) / args.steps
    if dist:
        t = torch.tensor([total_ms, plain_ms], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms, plain_ms = float(t[0].item()), float(t[1].item())
    ms_per_step = total_ms / args.steps
    value = rays * world / (ms_per_step * 1e-3) / 1e6
    plain_value = rays * world / (plain_ms * 1e-3) / 1e6

    # the non-learned comparator: the same pass with its views' tables built from the converged
    # closed form (bhr_surrogate_use_network(0)), no network, the same fallback; its own records
    outs_c = [torch.empty(v.rays * HIT_BYTES, dtype=torch.uint8, device=dev) for v in views]
    sur.use_network(False)
    plan_c = sur.plan(views, outs_c)
    sur.use_network(True)
    for _ in range(max(args.warmup, 0)):
        plan_c.launch(stream)
    per_cf, _ = timed(lambda: (plan_c.launch(stream), 0)[1], args.steps)
    cf_ms = sum(per_cf) / args.steps
    if dist:
        t = torch.tensor([cf_ms], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        cf_ms = float(t.item())
    cf_value = rays * world / (cf_ms * 1e-3) / 1e6

    # ---- end to end through the host-buffer entry point (records in pinned host memory)
    host = [torch.empty(v.rays * HIT_BYTES, dtype=torch.uint8, pin_memory=True) for v in views]
    host_np = [h.numpy() for h in host]
    for _ in range(max(args.warmup, 3)):  # warm-up steps, as for the device-timed paths
        sur.trace_host(views, host_np)
    e2e_steps = max(3, min(args.steps, 10))
    if dist:
        dist.barrier()
    e2e_each = []
    for _ in range(e2e_steps):
        t0 = time.perf_counter()
        sur.trace_host(views, host_np)
        e2e_each.append(time.perf_counter() - t0)
    # the median step: single steps on a GB300 host have been seen stalled for tens of ms
    # (8 of 10 steps at 11.3 ms, one at 96 ms); the mean and every step are reported beside it
    e2e_s = statistics.median(e2e_each)
    e2e_mean = sum(e2e_each) / e2e_steps
    if dist:
        t = torch.tensor([e2e_s, e2e_mean], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s, e2e_mean = float(t[0].item()), float(t[1].item())
    e2e = {"value": rays * world / e2e_s / 1e6, "unit": UNIT,
           "h2d_bytes_per_step": len(views) * 160, "d2h_bytes_per_step": rays * HIT_BYTES,
           "ms_per_step": e2e_s * 1e3, "statistic": f"median of {e2e_steps} steps",
           "mean_value": rays * world / e2e_mean / 1e6, "per_step_ms": [round(t * 1e3, 3) for t in e2e_each],
           "api": "bhr_surrogate_trace_host (pinned host records)"}

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    # ---- roofline of the dominant kernel (the surrogate pass). Its algorithmic work is the hit
    # records it writes (64 B per ray): the network runs only in the views' tables, so the HBM
    # roofline is the one it is measured against; the tensor figures ride along.
    peaks = {}
    pfile = ROOT / "MEASURED_PEAKS.json"
    if pfile.exists():
        try:
            peaks = json.loads(pfile.read_text())
        except Exception:
            peaks = {}
    bf16_peak = peaks.get("bf16_tflops")
    bf16_src = "MEASURED_PEAKS.json bf16_tflops (burst, cuBLAS)" if bf16_peak else "fallback 1900 TFLOP/s"
    bf16_peak = bf16_peak or 1900.0
    hbm_peak = peaks.get("hbm_gbs")
    hbm_src = "MEASURED_PEAKS.json hbm_gbs (copy)" if hbm_peak else "fallback 6800 GB/s"
    hbm_peak = hbm_peak or 6800.0
    mlp_flop = st["mlp_queries"] * F_MLP
    tensor_achieved = mlp_flop / (t_pass * 1e-3) / 1e12
    rec_bytes = rays * HIT_BYTES
    achieved = rec_bytes / (t_pass * 1e-3) / 1e9
    fp32_peak = fp32_peak_tflops(dev)
    traffic = None
    tfile = ROOT / "profiles" / "traffic.json"
    if tfile.exists():
        try:  # DRAM bytes of one k_surrogate launch (one view) from the committed ncu capture
            traffic = json.loads(tfile.read_text())["k_surrogate"]["dram_bytes_per_launch"]
        except (KeyError, ValueError):
            traffic = None
    roof = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
            "traffic": traffic,
            "traffic_note": "dram read+write bytes per k_surrogate launch (one view, ncu); the algorithmic writes "
                            "are 64 B x 2.07 M rays = 133 MB per view, part of the dirty lines still in L2 when "
                            "the kernel ends",
            "peak_source": hbm_src,
            "kernel": "k_surrogate (one launch per view), after k_tables (every view's exit and crossing tables) "
                      "and k_band_list (every view's band rays), one launch each; pass_ms runs from the step's start "
                      "to the end of the 16 passes, beside which the band march runs",
            "algorithm": f"{HIT_BYTES} B written per ray (the hit record), {rays} rays per step",
            "pass_ms": t_pass, "fallback_ms": t_fb,
            "tensor": {"achieved": tensor_achieved, "peak": bf16_peak, "unit": "TFLOP/s",
                       "frac": tensor_achieved / bf16_peak, "peak_source": bf16_src,
                       "algorithm": f"{F_MLP} BF16 FLOP per network row; {st['mlp_queries']} rows "
                                    f"({st['mlp_queries'] / max(st['surrogate'], 1):.3f} per surrogate ray: the views' "
                                    f"exit and crossing tables, {st['mlp_queries'] // max(len(views), 1)} rows per "
                                    f"view, which the rays interpolate)"},
            "note": "the pass is issue- and latency-bound on the CUDA cores (ray setup, closed-form orbit, the "
                    "tables' loads, the records); neither HBM nor the tensor pipe is its limit"}
    plan_p.launch(stream)
    steps_plain = plan_p.stats().steps
    plain_flop = steps_plain * F_STEP + rays * F_SETUP
    roof_plain = {"bound": "fp32", "achieved": plain_flop / (plain_ms * 1e-3) / 1e12, "peak": fp32_peak,
                  "unit": "TFLOP/s", "frac": plain_flop / (plain_ms * 1e-3) / 1e12 / fp32_peak,
                  "peak_source": "measured in this run: cuBLAS SGEMM 8192^3, TF32 off",
                  "algorithm": f"{F_STEP} FLOP per executed step + {F_SETUP} per ray; "
                               f"{steps_plain / rays:.2f} steps/ray"}

    cpu, accuracy = None, None
    if not args.no_cpu and world == 1:
        cpu, accuracy = cpu_baseline_and_check(views, outs, outs_p, outs_c)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+bf16", "data": "synthetic",
        "config": step_config(views),
        "paths": {"method": "learned surrogate + plain FP32 integrator fallback",
                  "plain_mrays_s": plain_value, "plain_ms_per_step": plain_ms,
                  "plain_launch_shape": plain_shape, "graph_plans": True,
                  "speedup_vs_plain": value / plain_value,
                  "closed_form_mrays_s": cf_value, "closed_form_ms_per_step": cf_ms,
                  "closed_form": "the same pass and fallback with the views' tables from the converged closed form "
                                 "(Carlson R_F, three duplication steps), no network: the non-learned comparator",
                  "surrogate_fraction": st["surrogate"] / rays, "fallback_rays": st["fallback"],
                  "capture_flag_disagreements": st["capture_disagree"],
                  "checkpoint": "trained in this run" if trained_here else str(DEFAULT_CHECKPOINT.relative_to(ROOT)),
                  "train_s": trained_here, "parallelism": f"replicas x{world}"},
        "accuracy": accuracy,
        "e2e": e2e,
        "gpu_launches": launches,
        "roofline": roof,
        "roofline_plain": roof_plain,
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "per_step_ms": per_step,
    }
    print(json.dumps(line), flush=True)
    plan_s.close()
    plan_c.close()
    plan_p.close()
    if dist:
        dist.destroy_process_group()


def run_side_workload(args):
    """--workload c3 | c4: the other configurations' throughput, one JSON line (not the headline).
    c3: 3840x2160, FOV 40, 700 steps, r = 20, inclination 88 deg, mixed FP32/FP64 precision.
    c4: 64 views of uneven size and budget (seed 1) as one autotuned CUDA-graph plan, with
        per-view latency."""
    import torch

    from blackholerender_gb300 import HIT_BYTES, PREC_MIXED, PREC_FP32, TERM_CONFIG, Tracer, workloads

    dev = torch.device("cuda", 0)
    tr = Tracer(0)
    if args.workload == "c3":
        views = [workloads.c3_view(TERM_CONFIG)]
        precision = PREC_MIXED
        name = "3840x2160, FOV 40, 700 steps, r=20, inclination 88 deg, mixed FP32/FP64 (band 1e-2, r<2.5)"
    else:
        views = workloads.c4_views(TERM_CONFIG)
        precision = PREC_FP32
        name = "64 views (seed 1), 320x180..3840x2160 log-uniform, FOV 30-90, r 6.5-200, budgets 200-700"
    rays = sum(v.rays for v in views)
    outs = [torch.empty(v.rays * HIT_BYTES, dtype=torch.uint8, device=dev) for v in views]
    t0 = time.perf_counter()
    plan = tr.plan(views, outs, precision=precision, autotune=True)
    tune_s = time.perf_counter() - t0
    st = torch.cuda.current_stream(dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    for _ in range(max(args.warmup, 3)):
        plan.launch(st)
    torch.cuda.synchronize(dev)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(0) as clk:
        for a, b in ev:
            flush.zero_()
            a.record(st)
            plan.launch(st)
            b.record(st)
        torch.cuda.synchronize(dev)
    per = [a.elapsed_time(b) for a, b in ev]
    ms = sum(per) / len(per)
    stats = plan.stats()
    line = {"metric": f"Mrays/s ({args.workload})", "value": rays / (ms * 1e-3) / 1e6, "unit": "Mrays/s",
            "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms,
            "higher_is_better": True, "dtype": "f32+f64" if precision == PREC_MIXED else "f32",
            "data": "synthetic", "config": {"workload": name, "rays_per_step": rays, "views": len(views),
                                            "graph": True, "autotune_s": tune_s,
                                            "launch_shape": plan.launch_shape.as_dict()},
            "gpu_launches": (1 + (1 if precision == PREC_MIXED else 0)) * args.steps,
            "march_steps_per_ray": stats.steps / rays, "fp64_rays": stats.fp64_rays,
            "fp64_steps": stats.fp64_steps, "clocks": clk.summary()}
    if len(views) > 1:
        lat = plan.view_times_ms()
        line["view_latency_ms"] = {"p50": float(np.median(lat)), "p90": float(np.percentile(lat, 90)),
                                   "max": float(lat.max())}
    print(json.dumps(line), flush=True)
    plan.close()
    tr.close()


def cpu_shade_sample(view, hits, params, seconds: float):
    """The oracle's shading (FP32 restatement, all host threads) of one view's records, repeated
    until `seconds` elapse; returns (Mpixels/s, threads). The noise volume is baked first,
    outside the timed region, as the GPU path bakes it once per seed."""
    L = _oracle()
    threads = os.cpu_count() or 1
    noise = np.zeros(128 ** 3, dtype=np.uint16)
    lut = np.zeros(256 * 4, dtype=np.float32)
    assert L.oracle_noise_bake(ctypes.c_uint32(params.noise_seed), ctypes.c_void_p(noise.ctypes.data), threads) == 0
    assert L.oracle_blackbody_lut(ctypes.c_void_p(lut.ctypes.data)) == 0
    out = np.zeros(view.rays * 4, dtype=np.float32)
    px = 0
    t0 = time.perf_counter()
    while True:
        rc = L.oracle_shade_view(ctypes.byref(view), ctypes.c_void_p(hits.ctypes.data), ctypes.byref(params),
                                 ctypes.c_void_p(noise.ctypes.data), ctypes.c_void_p(lut.ctypes.data),
                                 ctypes.c_void_p(out.ctypes.data), threads)
        assert rc == 0
        px += view.rays
        dt = time.perf_counter() - t0
        if dt >= seconds:
            return px / dt / 1e6, threads


def shade_traffic():
    """DRAM bytes of one k_shade launch (one 1080p view) from the committed ncu capture."""
    tfile = ROOT / "profiles" / "traffic.json"
    try:
        return json.loads(tfile.read_text())["k_shade"]["dram_bytes_per_launch"]
    except (OSError, KeyError, ValueError):
        return None


def run_shade_workload(args):
    """--workload shade: the consumer of the hit records. The 16 poses at 1920x1080 are traced
    once (plain FP32 plan, untimed); each step shades all 16 views from their records
    (bhr_shade: thin disk, star sky, default look). One JSON line, not the headline."""
    import torch

    from blackholerender_gb300 import HIT_BYTES, TERM_CONFIG, Tracer, hits_numpy, shade_params, workloads

    dev = torch.device("cuda", 0)
    tr = Tracer(0)
    views = workloads.c2_views(TERM_CONFIG)[: args.views]
    px = sum(v.rays for v in views)
    hits = [torch.empty(v.rays * HIT_BYTES, dtype=torch.uint8, device=dev) for v in views]
    tr.trace(views, hits)
    params = shade_params()
    outs = [torch.empty((v.height, v.width, 4), dtype=torch.float32, device=dev) for v in views]
    st = torch.cuda.current_stream(dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    for _ in range(max(args.warmup, 3)):
        tr.shade(views, hits, params, outs, st)
    torch.cuda.synchronize(dev)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(0) as clk:
        for a, b in ev:
            flush.zero_()
            a.record(st)
            tr.shade(views, hits, params, outs, st)
            b.record(st)
        torch.cuda.synchronize(dev)
    per = [a.elapsed_time(b) for a, b in ev]
    ms = sum(per) / len(per)
    peaks = {}
    pfile = ROOT / "MEASURED_PEAKS.json"
    if pfile.exists():
        try:
            peaks = json.loads(pfile.read_text())
        except Exception:
            peaks = {}
    hbm = peaks.get("hbm_gbs") or 6800.0
    bytes_px = HIT_BYTES + 16  # one record read, one float4 written
    achieved = px * bytes_px / (ms * 1e-3) / 1e9
    esc = sum(int((hits_numpy(h.cpu())["status"] == 1).sum()) for h in hits[:1]) / views[0].rays
    line = {"metric": "Mpixels/s (shade)", "value": px / (ms * 1e-3) / 1e6, "unit": "Mpixels/s", "n_gpus": 1,
            "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"shade {len(views)} poses (seed 0) at 1920x1080 from plain FP32 records; thin "
                                   "disk + analytic star layers, default look", "pixels_per_step": px,
                       "l2": "flushed (256 MiB write) between steps", "escaped_fraction_view0": esc},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                         "bytes_per_pixel": bytes_px, "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks.get(
                             "hbm_gbs") else "fallback 6800 GB/s",
                         "traffic": shade_traffic(),
                         "note": "issue-bound on the CUDA cores (star hashes and Gaussians); traffic is one "
                                 "view's launch from the committed ncu capture (writes partly still in L2)"},
            "gpu_launches": len(views) * args.steps, "clocks": clk.summary()}
    if not args.no_cpu:
        small = views[0].copy()
        small.width, small.height = 480, 270
        (h,) = tr.trace([small])
        torch.cuda.synchronize(dev)
        hs = np.ascontiguousarray(hits_numpy(h.cpu()))
        mpx, threads = cpu_shade_sample(small, hs, params, min(args.cpu_seconds, 10.0))
        line["cpu_baseline"] = {"value": mpx, "unit": "Mpixels/s", "cores": threads, "kind": "port",
                                "sample": "oracle shading of pose 0 at 480x270, repeated for up to 10 s",
                                "cpu": cpu_model()}
    print(json.dumps(line), flush=True)
    tr.close()


def run_vol_workload(args):
    """--workload vol: the volumetric disk (the reference's default disk) on the 16 poses at
    1920x1080, 450 steps, default look; each step marches the 16 views (bhr_trace_volumetric)
    into records and (rgb, transmittance). One JSON line, not the headline."""
    import torch

    from blackholerender_gb300 import DISK_VOLUMETRIC, HIT_BYTES, TERM_CONFIG, Tracer, hits_numpy, shade_params, workloads

    dev = torch.device("cuda", 0)
    tr = Tracer(0)
    views = workloads.c2_views(TERM_CONFIG)[: args.views]
    for v in views:
        v.disk_mode = DISK_VOLUMETRIC
    rays = sum(v.rays for v in views)
    p = shade_params()
    hits = [torch.empty(v.rays * HIT_BYTES, dtype=torch.uint8, device=dev) for v in views]
    rgbt = [torch.empty((v.height, v.width, 4), dtype=torch.float32, device=dev) for v in views]
    st = torch.cuda.current_stream(dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    for _ in range(max(args.warmup, 3)):
        tr.trace_volumetric(views, p, hits, rgbt, st)
    torch.cuda.synchronize(dev)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(0) as clk:
        for a, b in ev:
            flush.zero_()
            a.record(st)
            tr.trace_volumetric(views, p, hits, rgbt, st)
            b.record(st)
        torch.cuda.synchronize(dev)
    per = [a.elapsed_time(b) for a, b in ev]
    ms = sum(per) / len(per)
    h0 = hits_numpy(hits[0].cpu())
    steps = sum(int(hits_numpy(h.cpu())["steps"].astype(np.int64).sum()) for h in hits)
    line = {"metric": "Mrays/s (volumetric disk)", "value": rays / (ms * 1e-3) / 1e6, "unit": "Mrays/s", "n_gpus": 1,
            "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"{len(views)} poses (seed 0) x 1920x1080, FOV 60, 450 steps, volumetric disk "
                                   "[6, 20], default look", "rays_per_step": rays,
                       "l2": "flushed (256 MiB write) between steps",
                       "opaque_fraction_view0": float(np.mean(h0["status"] == 4))},
            "march_steps_per_ray": steps / rays, "gpu_launches": len(views) * args.steps, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    tr.close()


def run_bodies_workload(args):
    """--workload bodies: the BHS_BODIES variant on the 16 poses at 1920x1080, 450 steps, twelve
    bodies in front of every camera (workloads.body_gallery), thin disk (--disk volumetric: the
    reference's default disk). Each step marches the 16 views with their bodies
    (bhr_trace_bodies, or bhr_trace_bodies_volumetric into the image's rgbt) and shades them
    (bhr_shade_bodies). One JSON line, not the headline."""
    import torch

    from blackholerender_gb300 import (DISK_VOLUMETRIC, HIT_BYTES, STATUS_BODY, TERM_CONFIG, Tracer, hits_numpy,
                                       shade_params, workloads)

    dev = torch.device("cuda", 0)
    tr = Tracer(0)
    views = workloads.c2_views(TERM_CONFIG)[: args.views]
    vol = args.disk == "volumetric"
    if vol:
        for v in views:
            v.disk_mode = DISK_VOLUMETRIC
    scenes = [workloads.body_gallery(v) for v in views]
    rays = sum(v.rays for v in views)
    p = shade_params(time=10.0)
    hits = [torch.empty(v.rays * HIT_BYTES, dtype=torch.uint8, device=dev) for v in views]
    bh = [torch.empty(v.rays * 64, dtype=torch.uint8, device=dev) for v in views]
    img = [torch.empty((v.height, v.width, 4), dtype=torch.float32, device=dev) for v in views]
    st = torch.cuda.current_stream(dev)

    def step():
        for v, b, h, q, o in zip(views, scenes, hits, bh, img):
            if vol:  # the march gathers the disk's light into the image, which the shading completes
                tr.trace_bodies_volumetric(v, b, p, h, q, o, st)
            else:
                tr.trace_bodies(v, b, h, q, st)
        mid = torch.cuda.Event(enable_timing=True)
        mid.record(st)
        for v, b, h, q, o in zip(views, scenes, hits, bh, img):
            tr.shade_bodies(v, h, q, b, p, o, st)
        return mid

    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize(dev)
    rec = []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            flush.zero_()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(st)
            mid = step()
            b.record(st)
            rec.append((a, mid, b))
        torch.cuda.synchronize(dev)
    ms = sum(a.elapsed_time(b) for a, _, b in rec) / len(rec)
    ms_trace = sum(a.elapsed_time(m) for a, m, _ in rec) / len(rec)
    on = sum(int((hits_numpy(h.cpu())["status"] == STATUS_BODY).sum()) for h in hits)
    line = {"metric": "Mrays/s (bodies: march + shading)", "value": rays / (ms * 1e-3) / 1e6, "unit": "Mrays/s",
            "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms,
            "higher_is_better": True, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"{len(views)} poses (seed 0) x 1920x1080, FOV 60, 450 steps, {args.disk} disk, 12 bodies "
                                   "per view (nine planet looks, a star, an exploding photosphere, a ringed translucent "
                                   "planet), time 10", "rays_per_step": rays, "body_pixel_fraction": on / rays,
                       "march_ms": ms_trace, "shade_ms": ms - ms_trace, "l2": "flushed (256 MiB write) between steps"},
            "gpu_launches": 2 * len(views) * args.steps, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    tr.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--retrain", action="store_true", help="train the surrogate here instead of loading it")
    ap.add_argument("--block", type=int, default=0)
    ap.add_argument("--chunk", type=int, default=0)
    ap.add_argument("--refill", type=int, default=0)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--views", type=int, default=16, help="first N of the 16 poses (small profiling cases)")
    ap.add_argument("--disk", default="thin", choices=["thin", "volumetric"], help="the bodies workload's disk")
    ap.add_argument("--workload", default="c2", choices=["c2", "c3", "c4", "shade", "vol", "bodies"],
                    help="c2: the headline (16 poses at 1080p); c3 / c4: the other configurations; "
                         "shade: the records' shading consumer; vol: the volumetric disk march; "
                         "bodies: the march and shading with bodies")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        log("note: fewer than 3 warm-up steps")
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "shade":
        run_shade_workload(args)
    elif args.workload == "vol":
        run_vol_workload(args)
    elif args.workload == "bodies":
        run_bodies_workload(args)
    elif args.workload != "c2":
        run_side_workload(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
