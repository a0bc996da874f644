"""Batched launch under a CUDA graph with autotuned launch shapes (the 64-view configuration):
every launch shape gives bit-identical records, a plan's graph replays bhr_trace exactly, and
the full 64-view batch (uneven sizes and step budgets) agrees with the FP64 oracle."""
import time

import numpy as np
import pytest

import parity
from blackholerender_gb300 import (PREC_FP32, PREC_MIXED, TERM_CONFIG, LaunchShape, Tracer, hits_numpy,
                                   workloads)

pytestmark = pytest.mark.gpu


def _host(outs):
    import torch

    torch.cuda.synchronize()
    return [hits_numpy(o.cpu()) for o in outs]


def _bytes(hs):
    return [h.view(np.uint8) for h in hs]


@pytest.fixture(scope="module")
def small_views():
    return workloads.c4_views(TERM_CONFIG, scale=0.01)


def test_every_launch_shape_gives_identical_records(small_views):
    with Tracer(0) as t:
        ref = _bytes(_host(t.trace(small_views)))
        for sh in ((256, 0, 32, 4, 32), (512, 0, 128, 16, 16), (512, 1, 256, 24, 8), (256, 0, 64, 8, 8)):
            t.launch_shape = LaunchShape(*sh, 0.0)
            got = _bytes(_host(t.trace(small_views)))
            for a, b in zip(ref, got):
                assert np.array_equal(a, b), sh


def test_autotune_picks_a_valid_shape_and_caches_it(small_views):
    import torch

    with Tracer(0) as t:
        outs = [torch.empty(v.rays * 64, dtype=torch.uint8, device="cuda") for v in small_views]
        best = t.autotune(small_views, outs, PREC_FP32, reps=2)
        assert best.block_size in (256, 512) and best.tile_w in (32, 16, 8) and best.ms > 0
        assert t.launch_shape.as_dict() == best.as_dict()
        t0 = time.perf_counter()
        again = t.autotune(small_views, outs, PREC_FP32, reps=2)  # cached: no measuring
        assert time.perf_counter() - t0 < 0.05
        assert again.as_dict() == best.as_dict()


def test_plan_replays_bhr_trace_exactly(small_views):
    import torch

    with Tracer(0) as t:
        direct = _bytes(_host(t.trace(small_views)))
        steps_direct = t.stats().steps
        outs = [torch.zeros(v.rays * 64, dtype=torch.uint8, device="cuda") for v in small_views]
        p = t.plan(small_views, outs)
        for _ in range(2):  # replays start from zeroed work queues
            for o in outs:
                o.zero_()
            p.launch()
            got = _bytes(_host(outs))
            for a, b in zip(direct, got):
                assert np.array_equal(a, b)
            assert p.stats().steps == steps_direct
            ms = p.view_times_ms()
            assert np.all(ms > 0)
        p.close()


def test_plan_update_moves_the_cameras(small_views):
    import torch

    moved = workloads.c4_views(TERM_CONFIG, scale=0.01, seed=9)
    # same sizes and rules as small_views, other poses and FOVs
    for a, b in zip(moved, small_views):
        a.width, a.height = b.width, b.height
        a.max_steps, a.step_scale, a.disk_step = b.max_steps, b.step_scale, b.disk_step
    with Tracer(0) as t:
        want = _bytes(_host(t.trace(moved)))
        outs = [torch.zeros(v.rays * 64, dtype=torch.uint8, device="cuda") for v in small_views]
        p = t.plan(small_views, outs)
        p.update(moved)
        p.launch()
        got = _bytes(_host(outs))
        for a, b in zip(want, got):
            assert np.array_equal(a, b)
        p.close()


def test_plan_mixed_precision_matches_trace():
    import torch

    v = workloads.c3_view(TERM_CONFIG, width=960, height=540)
    with Tracer(0) as t:
        (want,) = _bytes(_host(t.trace([v], precision=PREC_MIXED)))
        out = torch.zeros(v.rays * 64, dtype=torch.uint8, device="cuda")
        p = t.plan([v], [out], precision=PREC_MIXED)
        p.launch()
        (got,) = _bytes(_host([out]))
        assert np.array_equal(want, got)
        assert p.stats().fp64_rays > 0
        p.close()


def test_plan_full_64_views_autotuned_vs_oracle():
    """The 64-view configuration at full size (120 M rays) as one autotuned graph launch."""
    import torch

    views = workloads.c4_views(TERM_CONFIG)
    rays = sum(v.rays for v in views)
    assert 1.0e8 < rays < 1.4e8  # 120.1 M for seed 1
    with Tracer(0) as t:
        outs = [torch.empty(v.rays * 64, dtype=torch.uint8, device="cuda") for v in views]
        p = t.plan(views, outs, autotune=True)
        st = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p.launch()
        e0.record(st)
        p.launch()
        e1.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        lat = p.view_times_ms()
        assert np.all(lat > 0) and lat.max() <= ms * 1.05
        print(f"\n64 views, {rays / 1e6:.1f} M rays: {ms:.2f} ms, {rays / ms / 1e3:.0f} Mrays/s; "
              f"shape {p.launch_shape.as_dict()}; view latency p50 {np.median(lat):.2f} ms max {lat.max():.2f} ms")
        rng = np.random.default_rng(5)
        cases = []
        for k in range(0, 64, 4):
            idx = rng.choice(views[k].rays, 1000, replace=False)
            cases.append((hits_numpy(outs[k].cpu()), views[k], idx))
        rep = parity.check_fp32_pooled(cases, where="64-view plan, 16 views x 1000 rays")
        print(rep.as_dict())
        p.close()
