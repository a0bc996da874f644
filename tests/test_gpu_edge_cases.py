"""Edge cases of the traced path through the C ABI, against the FP64 oracle: straight rays
(lensing off), far mode, no disk, sub-pixel jitter, tiny and ragged images under every pixel
tile, zero and one step budgets, cameras inside the photon sphere and inside the horizon, the
host-buffer entry point, argument errors, and the surrogate on rules it was not trained for."""
import numpy as np
import pytest

import oracle_lib as O
import parity
from blackholerender_gb300 import (DISK_NONE, DISK_VOLUMETRIC, FLAG_FALLBACK, FLAG_SURROGATE, HIT_DTYPE,
                                   STATUS_BUDGET, STATUS_CAPTURED, STATUS_ESCAPED, TERM_CONFIG, TERM_SHADER,
                                   BhrError, LaunchShape, Tracer, hits_numpy, make_view, workloads)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tracer():
    with Tracer(0) as t:
        yield t


def _run(tr, views):
    import torch

    outs = tr.trace(views)
    torch.cuda.synchronize()
    return [hits_numpy(o.cpu()) for o in outs]


def _bitwise(a, b):
    return np.array_equal(a.view(np.uint8), b.view(np.uint8))


def test_lensing_off_straight_rays(tracer):
    v = make_view(TERM_SHADER, width=160, height=90, preset=0, pose=(30.0, 1.45, 0.2), lensing=0)
    (g,) = _run(tracer, [v])
    parity.check_fp32(g, v, where="lensing off")
    # straight rays that miss the horizon escape along their pixel direction
    esc = g["status"] == STATUS_ESCAPED
    d = O.primary_rays(v, np.nonzero(esc)[0])
    assert np.percentile(O.angle(g["dir"][esc], d), 99) < 1e-6


def test_far_mode_escapes_along_the_pixel(tracer):
    v = make_view(TERM_SHADER, width=64, height=36, preset=0, pose=(30.0, 1.2, 0.0), far_mode=1)
    (g,) = _run(tracer, [v])
    ref = O.trace_view(v, fp64=True)
    assert np.all(g["status"] == STATUS_ESCAPED) and np.all(ref["status"] == STATUS_ESCAPED)
    assert np.max(O.angle(g["dir"], ref["dir"])) < 1e-6 and np.all(g["steps"] == 0)


def test_no_disk_and_jitter(tracer):
    v = make_view(TERM_CONFIG, width=200, height=120, preset=1, pose=(18.0, 1.5, 2.0), disk_mode=DISK_NONE)
    v.jitter[0], v.jitter[1] = 0.37, -0.21
    (g,) = _run(tracer, [v])
    assert np.all(g["ncross"] == 0)
    parity.check_fp32(g, v, where="no disk, jitter")


@pytest.mark.parametrize("wh", [(1, 1), (3, 2), (17, 5), (33, 1), (1, 40)])
def test_tiny_and_ragged_images_every_tile(wh):
    w, h = wh
    v = make_view(TERM_SHADER, width=w, height=h, preset=0, pose=(25.0, 1.5, 0.0), fov_deg=20.0)
    ref = O.trace_view(v, fp64=True)
    with Tracer(0) as t:
        first = None
        for tile in (32, 16, 8):
            t.launch_shape = LaunchShape(512, 0, 64, 8, tile, 0.0)
            (g,) = _run(t, [v])
            assert len(g) == w * h
            rep = parity.compare(g, ref, max_steps=v.max_steps)
            assert rep.class_mismatch == 0, (wh, tile, rep.as_dict())
            if first is None:
                first = g
            assert _bitwise(g, first), (wh, tile)
        # the same tiny views inside a multi-view batch of uneven sizes
        big = make_view(TERM_SHADER, width=64, height=48, preset=0, pose=(25.0, 1.5, 0.0))
        (gb, gs) = _run(t, [big, v])
        assert _bitwise(gs, first)


@pytest.mark.parametrize("budget", [0, 1, 2])
def test_zero_and_one_step_budgets(tracer, budget):
    v = make_view(TERM_SHADER, width=48, height=27, preset=0, pose=(30.0, 1.5, 0.0), max_steps=budget)
    (g,) = _run(tracer, [v])
    ref = O.trace_view(v, fp64=True)
    assert np.all(g["status"] == ref["status"]) and np.all(g["steps"] == ref["steps"])
    assert np.all(g["status"] == STATUS_BUDGET) and np.all(g["steps"] == budget)


@pytest.mark.parametrize("r", [2.6, 1.9])
def test_camera_inside_photon_sphere_and_horizon(tracer, r):
    v = make_view(TERM_SHADER, width=64, height=36, preset=2, pose=(r, 1.3, 0.4))
    (g,) = _run(tracer, [v])
    ref = O.trace_view(v, fp64=True)
    if r < 2.0:  # already inside the capture radius: captured at the first loop head
        assert np.all(g["status"] == STATUS_CAPTURED) and np.all(g["steps"] == 0)
        assert np.all(ref["status"] == STATUS_CAPTURED)
    else:
        parity.check_fp32(g, v, where=f"camera at r={r}")


def test_host_buffers_equal_device_buffers(tracer):
    views = [workloads.c1_view(TERM_CONFIG), make_view(TERM_SHADER, width=77, height=31, pose=(40.0, 1.0, 1.0))]
    dev = _run(tracer, views)
    host = [np.zeros(v.rays, dtype=HIT_DTYPE) for v in views]
    tracer.trace_host(views, host)
    for a, b in zip(dev, host):
        assert _bitwise(a, b)


def test_argument_errors_are_reported(tracer):
    import torch

    good = make_view(TERM_SHADER, width=8, height=8)
    out = torch.empty(64 * 64, dtype=torch.uint8, device="cuda")
    bad = good.copy()
    bad.width = 0
    with pytest.raises(BhrError) as e:
        tracer.trace([bad], [out])
    assert e.value.code == -1 and "width" in str(e.value)
    vol = good.copy()
    vol.disk_mode = DISK_VOLUMETRIC
    with pytest.raises(BhrError) as e:
        tracer.trace([vol], [out])
    assert e.value.code == -5
    with pytest.raises(BhrError):  # outputs must be 16-byte aligned
        tracer.trace_ptrs([good], [out.data_ptr() + 4])
    with pytest.raises(BhrError):
        tracer.trace_ptrs([good], [0])
    # the context stays usable after errors
    (g,) = _run(tracer, [good])
    assert len(g) == 64


def test_surrogate_refuses_views_it_does_not_answer():
    """The surrogate answers lensed rays under the CONFIG rule at its trained exit radius and
    under the SHADER / CPU tolerance escape; lensing off, far mode, the volumetric disk and a
    CONFIG escape radius other than the trained one are the plain integrator's (bhr_trace): the
    surrogate says so with BHR_ERR_UNSUPPORTED and stays usable."""
    import torch

    from blackholerender_gb300.surrogate import DEFAULT_CHECKPOINT, Surrogate

    s = Surrogate(seed=2)
    s.load(DEFAULT_CHECKPOINT)
    pose = (30.0, 1.45, 0.0)
    far = make_view(TERM_CONFIG, width=64, height=36, preset=2, pose=pose)
    far.far_mode = 1
    vol = make_view(TERM_CONFIG, width=64, height=36, preset=2, pose=pose)
    vol.disk_mode = DISK_VOLUMETRIC
    esc = make_view(TERM_CONFIG, width=64, height=36, preset=2, pose=pose)
    esc.escape_r = 500.0
    cases = [(make_view(TERM_CONFIG, width=64, height=36, preset=2, pose=pose, lensing=0), "lensing"),
             (far, "far mode"), (vol, "volumetric"), (esc, "escape radius")]
    for v, why in cases:
        with pytest.raises(BhrError) as e:
            s.trace([v])
        assert e.value.code == -5 and why in str(e.value), str(e.value)
    (o,) = s.trace([make_view(TERM_SHADER, width=64, height=36, preset=2, pose=pose)])
    torch.cuda.synchronize()
    g = hits_numpy(o.cpu())
    assert np.all((g["flags"] & (FLAG_SURROGATE | FLAG_FALLBACK)) != 0)
    (o,) = s.trace([make_view(TERM_CONFIG, width=64, height=36, preset=2, pose=pose)])
    torch.cuda.synchronize()
    g = hits_numpy(o.cpu())
    s.close()
    assert np.all((g["flags"] & (FLAG_SURROGATE | FLAG_FALLBACK)) != 0)
