"""The volumetric disk's march in the CPU restatement (blackhole.frag:169-181,217-234 with
volumetricDiskStep, disk.glsl:88-110): transmittance and colour bounds, an empty disk changes
nothing but the step clamp, rays that never enter the slab march as in the thin-disk mode,
and the FP32 restatement against the FP64 one."""
from __future__ import annotations

import numpy as np
import pytest

import oracle_lib as O
from blackholerender_gb300 import (DISK_THIN, DISK_VOLUMETRIC, STATUS_ESCAPED, STATUS_OPAQUE, TERM_CONFIG, make_view,
                                   shade_params)


@pytest.fixture(scope="module")
def tex():
    return O.noise_bake(7), O.blackbody_lut()


def _view(**kw):
    base = dict(width=96, height=54, preset=0, pose=(30.0, np.radians(80.0), 0.4), disk_mode=DISK_VOLUMETRIC)
    base.update(kw)
    return make_view(TERM_CONFIG, **base)


def test_transmittance_and_colour_bounds(tex):
    v = _view()
    hits, rgbt = O.trace_volumetric(v, shade_params(disk_density=4.0), *tex)  # dense enough to turn opaque
    T = rgbt[..., 3].reshape(-1)
    assert np.all((T >= 0.0) & (T <= 1.0)) and np.all(rgbt[..., :3] >= 0.0)
    op = hits["status"] == STATUS_OPAQUE
    assert op.sum() > 50 and np.all(T[op] < 0.004) and np.all(T[~op] >= 0.004)
    assert np.all(hits["ncross"] == 0)  # no crossing slots in the volumetric mode
    lit = rgbt[..., :3].sum(-1).reshape(-1) > 0
    assert np.all(lit[op]) and np.all(T[~lit] == 1.0)


def test_empty_disk_gathers_nothing(tex):
    v = _view()
    hits, rgbt = O.trace_volumetric(v, shade_params(disk_density=0.0), *tex)
    assert np.all(rgbt[..., 3] == 1.0) and np.all(rgbt[..., :3] == 0.0)
    assert not np.any(hits["status"] == STATUS_OPAQUE)


def test_rays_that_miss_the_slab_march_as_in_the_thin_mode(tex):
    v = _view()
    hits, rgbt = O.trace_volumetric(v, shade_params(), *tex)
    thin = O.trace_view(_view(disk_mode=DISK_THIN), fp64=True)
    # the slab clamp applies only inside the slab; rays that never reach it agree exactly
    far = (thin["nplane"] == 0) & (hits["nplane"] == 0) & (rgbt[..., 3].reshape(-1) == 1.0)
    assert far.sum() > 500
    same = (hits["status"][far] == thin["status"][far]) & (hits["steps"][far] == thin["steps"][far])
    assert same.mean() > 0.99
    esc = far & (hits["status"] == STATUS_ESCAPED) & (thin["status"] == STATUS_ESCAPED)
    assert np.max(O.angle(hits["dir"][esc], thin["dir"][esc])) < 1e-6


def test_fp32_restatement_against_fp64(tex):
    v = _view()
    p = shade_params(disk_density=4.0)
    h64, c64 = O.trace_volumetric(v, p, *tex, fp64=True)
    h32, c32 = O.trace_volumetric(v, p, *tex, fp64=False)
    T64 = c64[..., 3].reshape(-1)
    amb = (np.abs(h64["b"] - 27 ** 0.5) < 1e-2) | (np.abs(T64 - 0.004) < 0.002)
    agree = (h64["status"] == h32["status"])[~amb].mean()
    d = np.abs(c32 - c64).reshape(-1, 4)[~amb]
    scale = np.abs(c64).reshape(-1, 4)[~amb] + 1e-3
    print(f"\nFP32 vs FP64 restatement: status agreement {agree:.5f}, |d rgbt| / (|ref| + 1e-3) p50 "
          f"{np.median(d / scale):.2e} p99 {np.percentile(d / scale, 99):.2e}")
    assert agree > 0.995
    assert np.percentile(d / scale, 99) < 0.05


def test_sampled_pixels_equal_the_whole_view():
    """The restatement's sampled-pixel entry marches exactly the pixels the whole-view entry does."""
    v = make_view(TERM_CONFIG, disk_mode=DISK_VOLUMETRIC, width=48, height=27, preset=0,
                  pose=(30.0, np.radians(85.0), 0.0))
    p = shade_params()
    noise, lut = O.noise_bake(7), O.blackbody_lut()
    h, c = O.trace_volumetric(v, p, noise, lut, fp64=True)
    idx = np.array([0, 7, 300, 1295, 640, 641])
    hs, cs = O.trace_volumetric_pixels(v, p, noise, lut, idx, fp64=True)
    assert hs.tobytes() == h[idx].tobytes() and np.array_equal(cs, c.reshape(-1, 4)[idx])
