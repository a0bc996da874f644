"""Lens table (the second consumer of the integrator, shaders/gas_lens.comp): the GPU build with
the reference's RK4 construction against the FP64 and FP32 CPU restatements, and the closed-form
build (every texel from the elliptic-integral orbit) against the converged FP64 construction."""
import math
import time

import numpy as np
import pytest

import oracle_lib as O
from blackholerender_gb300 import METHOD_PLAIN, METHOD_SURROGATE, SQRT27, Tracer, _abi

pytestmark = pytest.mark.gpu


def _fan_b(cam_r):
    """Impact parameter of every fan ray (double), as the builders compute alpha."""
    L = _abi.lib()
    ac = np.float32(L.bhr_shadow_angular_radius(cam_r))
    a = np.array([L.bhr_lens_alpha(np.float32((i + 0.5) / 1024), ac) for i in range(1024)], dtype=np.float64)
    return float(ac), cam_r * np.sin(a) / math.sqrt(1 - 2 / cam_r)


@pytest.fixture(scope="module")
def tracer():
    with Tracer(0) as t:
        yield t


@pytest.mark.parametrize("cam_r", [8.0, 30.0, 120.0])
def test_integrator_table_matches_the_restatement(tracer, cam_r):
    import torch

    ac, b = _fan_b(cam_r)
    gpu = tracer.lens_table(cam_r, METHOD_PLAIN)
    torch.cuda.synchronize()
    gpu = gpu.cpu().numpy()
    ref = O.lens_table(cam_r, ac, fp64=True)
    ref32 = O.lens_table(cam_r, ac, fp64=False)
    ok = np.abs(b - SQRT27) > 1e-3  # rays off the shadow's edge (there FP32 winding diverges)
    d = np.abs(gpu - ref)[:, ok]
    d32 = np.abs(ref32 - ref)[:, ok]
    assert np.array_equal(gpu[0], ref[0])
    p99, p99_32 = np.percentile(d, 99), np.percentile(d32, 99)
    print(f"\nr_cam {cam_r}: integrator table vs FP64, |d log r| p99 {p99:.1e} p99.9 {np.percentile(d, 99.9):.1e} "
          f"(FP32 restatement p99 {p99_32:.1e})")
    assert p99 <= max(2e-4, 3 * p99_32)
    assert np.mean(d > 1e-2) < 2e-3  # texels at a capture / escape boundary


@pytest.mark.parametrize("cam_r", [8.0, 30.0, 120.0])
def test_closed_form_table_matches_the_converged_construction(tracer, cam_r):
    import torch

    ac, b = _fan_b(cam_r)
    gpu = tracer.lens_table(cam_r, METHOD_SURROGATE)
    torch.cuda.synchronize()
    gpu = gpu.cpu().numpy()
    ref = O.lens_table(cam_r, ac, fp64=True)
    ok = np.abs(b - SQRT27) > 1e-3
    d = np.abs(gpu - ref)[:, ok]
    print(f"\nr_cam {cam_r}: closed-form table vs the FP64 RK4 construction, |d log r| p50 {np.percentile(d, 50):.1e} "
          f"p99 {np.percentile(d, 99):.1e} p99.9 {np.percentile(d, 99.9):.1e}")
    assert np.percentile(d, 99) < 1e-3
    assert np.mean(d > 1e-2) < 5e-3


def test_closed_form_builds_faster(tracer):
    import torch

    out = torch.empty((1024, 1024), dtype=torch.float32, device="cuda")
    times = {}
    for m in (METHOD_PLAIN, METHOD_SURROGATE):
        tracer.lens_table(30.0, m, out)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(5):
            tracer.lens_table(30.0, m, out)
        torch.cuda.synchronize()
        times[m] = (time.perf_counter() - t0) / 5 * 1e3
    print(f"\nlens table at r_cam 30: integrator {times[METHOD_PLAIN]:.3f} ms, closed form {times[METHOD_SURROGATE]:.3f} ms")
    assert times[METHOD_SURROGATE] < times[METHOD_PLAIN]


def test_closed_form_refuses_cameras_inside_the_photon_sphere(tracer):
    with pytest.raises(_abi.BhrError) as e:
        tracer.lens_table(2.9, METHOD_SURROGATE)
    assert e.value.code == -5
    t = tracer.lens_table(2.9, METHOD_PLAIN)  # the integrator builds it
    assert t.shape == (1024, 1024)
