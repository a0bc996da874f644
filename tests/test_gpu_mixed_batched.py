"""Mixed FP32/FP64 precision (4K edge-on configuration) and batched multi-view launches
(64 uneven views) against the FP64 oracle, through the C ABI."""
import numpy as np
import pytest

import oracle_lib as O
import parity
from blackholerender_gb300 import (FLAG_FP64, PREC_FP32, PREC_MIXED, SQRT27, TERM_CONFIG, TERM_SHADER, Tracer,
                                   hits_numpy, workloads)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tracer():
    with Tracer(0) as t:
        yield t


def _run(tr, views, precision=PREC_FP32):
    import torch

    outs = tr.trace(views, precision=precision)
    torch.cuda.synchronize()
    return [hits_numpy(o.cpu()) for o in outs]


def test_mixed_4k_edge_on_reduced(tracer):
    # the 4K, FOV 40, r=20, i=88 deg, 700-step configuration at 960x540 (every pixel checked)
    v = workloads.c3_view(TERM_CONFIG, width=960, height=540)
    (mixed,) = _run(tracer, [v], PREC_MIXED)
    (fp32,) = _run(tracer, [v], PREC_FP32)
    ref = O.trace_view(v, fp64=True)
    b = ref["b"].astype(np.float64)
    band = np.abs(b - SQRT27) < v.promote_band
    # band rays and rays that reached r < promote_r ran in FP64
    assert np.all(mixed["flags"][band & (mixed["status"] > 0)] & FLAG_FP64)
    assert np.all((mixed["flags"] & FLAG_FP64)[ref["min_r"] < v.promote_r - 0.05] != 0)
    rep = parity.compare(mixed, ref, max_steps=v.max_steps, band=1e-6)
    assert rep.class_mismatch == 0, rep.as_dict()
    # inside the FP32 band the FP64 path classifies at least as well as FP32
    cls_m = (mixed["status"] == ref["status"]) & ((mixed["ncross"] > 0) == (ref["ncross"] > 0))
    cls_f = (fp32["status"] == ref["status"]) & ((fp32["ncross"] > 0) == (ref["ncross"] > 0))
    assert (~cls_m & band).sum() <= (~cls_f & band).sum()
    # FP64 band rays follow the FP64 oracle closely
    esc = band & (ref["status"] == 1) & cls_m & (np.abs(b - SQRT27) > 1e-4)
    if esc.any():
        assert np.percentile(O.angle(mixed["dir"][esc], ref["dir"][esc]), 99) < 1e-5


def test_mixed_4k_full_res_sampled(tracer):
    v = workloads.c3_view(TERM_CONFIG)
    (mixed,) = _run(tracer, [v], PREC_MIXED)
    rng = np.random.default_rng(3)
    ref_b = mixed["b"].astype(np.float64)
    near = np.nonzero(np.abs(ref_b - SQRT27) < 2e-2)[0]
    uni = rng.choice(v.rays, 6000, replace=False)
    nb = rng.choice(near, min(3000, len(near)), replace=False)
    ref_u = O.trace_pixels(v, uni, fp64=True)
    rep = parity.compare(mixed[uni], ref_u, max_steps=v.max_steps, band=1e-6)
    assert rep.class_mismatch == 0, rep.as_dict()
    # edge-on at r=20 most of the frame is photon ring: FP32 rays just outside the FP64 band
    # (|b - sqrt27| in [1e-2, 5e-2]) set the 99th percentile here
    assert rep.dir_p99 < 5e-5, rep.as_dict()
    # near the photon sphere: classification must hold; FP64-run rays track the FP64 oracle
    ref_n = O.trace_pixels(v, nb, fp64=True)
    rep = parity.compare(mixed[nb], ref_n, max_steps=v.max_steps, band=1e-6)
    assert rep.class_mismatch == 0, rep.as_dict()
    m = mixed[nb]
    fp64 = ((m["flags"] & FLAG_FP64) != 0) & (m["status"] == 1) & (ref_n["status"] == 1) & \
        (np.abs(ref_n["b"].astype(np.float64) - SQRT27) > 1e-4)
    if fp64.any():
        assert np.percentile(O.angle(m["dir"][fp64], ref_n["dir"][fp64]), 99) < 1e-5


def test_batched_equals_single_view_launches(tracer):
    views = workloads.c4_views(TERM_CONFIG, scale=0.01)
    multi = _run(tracer, views)
    for v, m in zip(views[::7], multi[::7]):
        (one,) = _run(tracer, [v])
        assert np.array_equal(one.view(np.uint8), m.view(np.uint8))


def test_batched_c4_vs_oracle(tracer):
    views = workloads.c4_views(TERM_CONFIG, scale=0.01)
    multi = _run(tracer, views)
    ms = tracer.view_times_ms(len(views))
    assert np.all(ms > 0)
    rng = np.random.default_rng(11)
    for v, m in zip(views, multi):
        idx = rng.choice(v.rays, min(300, v.rays), replace=False)
        parity.check_fp32(m, v, idx, where=f"C4 view {v.width}x{v.height}")


def test_batched_mixed_rules(tracer):
    # views with different termination rules in one call run as one launch per rule
    views = workloads.c4_views(TERM_CONFIG, scale=0.005, n=6) + workloads.c4_views(TERM_SHADER, scale=0.005, n=6, seed=5)
    multi = _run(tracer, views)
    for v, m in zip(views, multi):
        parity.check_fp32(m, v, where="mixed-rule batch")


def _hist(x, edges):
    h, _ = np.histogram(np.clip(x, edges[0], edges[-1] * 0.999), bins=edges)
    return ", ".join(f"<{e:.0e}: {n}" for e, n in zip(edges[1:], h))


def test_mixed_4k_every_pixel_error_histograms(tracer):
    """The 3840x2160 edge-on configuration, every pixel against the FP64 oracle: histograms of the
    deflection-angle and crossing-radius errors, and misclassified rays inside and outside the
    FP64 band (|b - sqrt27| < 1e-2)."""
    v = workloads.c3_view(TERM_CONFIG)
    (mixed,) = _run(tracer, [v], PREC_MIXED)
    ref = O.trace_view(v, fp64=True)
    b = ref["b"].astype(np.float64)
    band = np.abs(b - SQRT27) < v.promote_band
    cls = (mixed["status"] == ref["status"]) & ((mixed["ncross"] > 0) == (ref["ncross"] > 0))
    rep = parity.compare(mixed, ref, max_steps=v.max_steps, band=1e-6)
    esc = (mixed["status"] == 1) & (ref["status"] == 1) & (mixed["steps"] == ref["steps"])
    ang = O.angle(mixed["dir"][esc], ref["dir"][esc])
    same = esc & (mixed["ncross"] == ref["ncross"]) & (ref["ncross"] > 0)
    rel = np.abs(mixed["cross_r"][same, 0].astype(np.float64) - ref["cross_r"][same, 0]) / ref["cross_r"][same, 0]
    edges = np.array([0.0, 1e-9, 1e-8, 1e-7, 1e-6, 1e-5, 1e-4, 1e-3, 1e-2, 1.0])
    print(f"\n4K edge-on, {v.rays} rays, mixed precision vs FP64 oracle")
    print(f"  misclassified: inside the FP64 band {int((~cls & band).sum())} of {int(band.sum())}, "
          f"outside {int((~cls & ~band).sum())} of {int((~band).sum())} "
          f"(ill-conditioned and excluded: {rep.n_band} near b_crit, {rep.n_budget_amb} at the budget, {rep.n_edge_amb} at a disk edge)")
    print(f"  direction error (rad), {len(ang)} escaped rays: {_hist(ang, edges)}")
    print(f"  first crossing radius, relative, {len(rel)} rays: {_hist(rel, edges)}")
    assert rep.class_mismatch == 0, rep.as_dict()
    assert np.percentile(ang, 99) < 5e-5 and np.percentile(rel, 99) < 5e-5
