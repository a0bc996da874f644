"""The shading consumer's restatement on the CPU, pinned where the reference or published
values allow: the blackbody table (the library's host bake against the oracle's, bit for bit;
the 6500 K chromaticity against the CIE Planckian locus; luminance normalisation), the
shader's redshift factor against the reference's compiled redshiftFactor (Geodesic.h:90-95)
and its own known-answer test (geodesic_tests.cpp:114-143), the R16F store against numpy's
binary16 rounding, pcg3d against a Python restatement, and the host-side shading rules on
synthetic records (opacity stop, sky weight, mixed quads, NaN clear)."""
from __future__ import annotations

import math

import numpy as np
import pytest

import oracle_lib as O
from blackholerender_gb300 import (DISK_THIN, HIT_DTYPE, STATUS_CAPTURED, STATUS_ESCAPED, TERM_CONFIG, blackbody_lut,
                                   make_view, shade_params)


def test_library_blackbody_table_equals_the_oracle():
    lib_lut = blackbody_lut()
    ref = O.blackbody_lut()
    assert lib_lut.shape == (256, 4)
    assert np.array_equal(lib_lut.view(np.uint32), ref.view(np.uint32))


def test_blackbody_table_known_answers():
    lut = O.blackbody_lut()
    # rgb normalised to Rec.709 luminance 1 wherever the colour is not clipped to black
    lum = 0.2126 * lut[:, 0].astype(np.float64) + 0.7152 * lut[:, 1] + 0.0722 * lut[:, 2]
    assert np.max(np.abs(lum - 1.0)) < 1e-6
    # 6500 K through the CIE 1931 lobe fits: chromaticity on the Planckian locus (0.3135, 0.3236)
    X, Y, Z = O.blackbody_xyz(6500.0)
    x, y = X / (X + Y + Z), Y / (X + Y + Z)
    assert abs(x - 0.3135) < 3e-3 and abs(y - 0.3236) < 3e-3
    # a = Y(T) / Y(6500 K): 1 between the entries that bracket 6500 K, rising with T
    T = np.exp(np.log(1000.0) + (np.log(40000.0) - np.log(1000.0)) * np.arange(256) / 255)
    k = int(np.searchsorted(T, 6500.0))
    assert lut[k - 1, 3] < 1.0 < lut[k, 3]
    assert np.all(np.diff(lut[:, 3]) > 0)
    # cool stars red, hot stars blue
    assert lut[0, 0] > lut[0, 1] > lut[0, 2] and lut[-1, 2] > lut[-1, 0]


def test_shader_redshift_matches_the_reference_cpu_mirror():
    ref = O.ref_lib()
    if ref is None:
        pytest.skip("the reference's Geodesic.h was not compiled here")
    rng = np.random.default_rng(3)
    for _ in range(200):
        r = float(np.float32(rng.uniform(6.0, 20.0)))
        rc = float(np.float32(rng.uniform(8.0, 200.0)))
        b = float(np.float32(rng.uniform(-8.0, 8.0)))
        g = O.redshift_factor(r, b, rc)
        gr = ref.ref_redshift_factor(r, b, rc)
        assert abs(g - gr) <= 2e-6 * abs(gr), (r, b, rc, g, gr)


def test_redshift_known_answers():
    # geodesic_tests.cpp:114-143: receding side redder than the approaching side, closed form,
    # face-on factor sqrt(1 - 3/r) / sqrt(1 - 2/rc)
    g_away = O.redshift_factor(8.0, -8.0, 30.0)
    g_toward = O.redshift_factor(8.0, 8.0, 30.0)
    assert g_away < 1.0 < g_toward
    expect = 1.0 / (math.sqrt(1 - 2 / 30) / math.sqrt(1 - 3 / 8) * (1 - 8 ** -1.5 * -8.0))
    assert abs(g_away - expect) < 2e-6 * expect
    assert abs(O.redshift_factor(8.0, 0.0, 30.0) - math.sqrt(1 - 3 / 8) / math.sqrt(1 - 2 / 30)) < 1e-6


def test_half_store_rounds_to_nearest_even():
    rng = np.random.default_rng(5)
    xs = np.concatenate([rng.uniform(0, 1.4, 20000), rng.uniform(0, 1e-4, 5000), 10.0 ** rng.uniform(-9, 4.9, 5000),
                         [0.0, 6.1035156e-05, 5.9604645e-08, 2.9802322e-08, 65504.0, 65520.0, 1.0 + 2.0 ** -11]])
    xs = np.concatenate([xs, -xs]).astype(np.float32)
    with np.errstate(over="ignore"):
        want = xs.astype(np.float16).view(np.uint16)
    got = np.array([O.to_half(float(x)) for x in xs], dtype=np.uint16)
    assert np.array_equal(got, want)


def _pcg3d_py(v):
    M = 0xFFFFFFFF
    x, y, z = [(int(a) * 1664525 + 1013904223) & M for a in v]
    x = (x + y * z) & M
    y = (y + z * x) & M
    z = (z + x * y) & M
    x, y, z = x ^ (x >> 16), y ^ (y >> 16), z ^ (z >> 16)
    x = (x + y * z) & M
    y = (y + z * x) & M
    z = (z + x * y) & M
    return x, y, z


def test_pcg3d_restatement():
    rng = np.random.default_rng(9)
    for v in [(0, 0, 0), (1, 2, 3), (0xFFFFFFFF, 7, 131)] + [tuple(rng.integers(0, 2 ** 32, 3)) for _ in range(200)]:
        assert O.pcg3d(v) == _pcg3d_py(v)


def test_noise_volume_is_seamless_and_spread():
    n = O.noise_bake(7).view(np.float16).astype(np.float32)
    assert n.shape == (128, 128, 128) and np.all(np.isfinite(n))
    assert 0.0 <= n.min() and n.max() <= 1.3
    assert 0.3 < n.mean() < 0.6 and n.std() > 0.08
    # the lattice wraps: the step across the tile edge is like any other step
    inner = np.abs(np.diff(n, axis=2)).mean()
    edge = np.abs(n[:, :, 0] - n[:, :, -1]).mean()
    assert edge < 1.5 * inner
    assert not np.array_equal(n, O.noise_bake(8).view(np.float16).astype(np.float32))


def _records(view, status, ncross=0, cross_r=(10.0, 12.0, 14.0)):
    h = np.zeros(view.width * view.height, dtype=HIT_DTYPE)
    h["status"] = status
    h["ncross"] = ncross
    h["cross_r"] = cross_r
    h["cross_phi"] = (0.3, 1.2, -2.0)
    h["b_axis"] = 3.0
    d = O.primary_rays(view, np.arange(h.size))
    if status == STATUS_ESCAPED:
        h["dir"] = d.astype(np.float32)
    return h


def test_shading_rules_on_synthetic_records():
    v = make_view(TERM_CONFIG, width=32, height=18, pose=(30.0, 1.5, 0.0), disk_mode=DISK_THIN)
    noise = O.noise_bake(7)
    lut = O.blackbody_lut()
    p = shade_params()
    # captured, no crossings: black, no sky weight
    img = O.shade_view(v, _records(v, STATUS_CAPTURED), p, noise, lut)
    assert np.all(img == 0.0)
    # escaped along the pixel direction: star light only, and the full sky-cube weight
    img = O.shade_view(v, _records(v, STATUS_ESCAPED), p, noise, lut)
    assert np.all(img[..., 3] == 1.0) and np.all(img[..., :3] >= 0.0) and img[..., :3].max() > 0.0
    # three crossings in a dense disk: opaque after the first or second, no sky weight left
    dense = shade_params(disk_density=50.0)
    img = O.shade_view(v, _records(v, STATUS_ESCAPED, 3), dense, noise, lut)
    assert np.all(img[..., 3] == 0.0) and img[..., :3].min() > 0.0
    # a thin disk passes part of the sky weight: transmittance x sky_brightness
    thin = shade_params(disk_density=0.05, sky_brightness=2.0)
    img = O.shade_view(v, _records(v, STATUS_ESCAPED, 1), thin, noise, lut)
    assert np.all((img[..., 3] > 0.0) & (img[..., 3] < 2.0))
    # crossings outside [r_in, r_out] add nothing
    img0 = O.shade_view(v, _records(v, STATUS_ESCAPED, 0), p, noise, lut)
    img1 = O.shade_view(v, _records(v, STATUS_ESCAPED, 3, cross_r=(3.0, 25.0, 40.0)), p, noise, lut)
    assert np.array_equal(img0, img1)
    # a non-finite direction: no star light there (its Gaussians are NaN and skipped, and min /
    # max as fminf / fmaxf keep the rest finite), and the image stays finite (blackhole.frag:377)
    h = _records(v, STATUS_ESCAPED)
    h["dir"][5] = np.nan
    img = O.shade_view(v, h, p, noise, lut)
    assert np.all(img[0, 5, :3] == 0.0) and np.all(np.isfinite(img))


def test_shadow_overlay_rings_the_shadow():
    v = make_view(TERM_CONFIG, width=96, height=54, pose=(30.0, 1.5, 0.0), fov_deg=40.0)
    noise = O.noise_bake(7)
    lut = O.blackbody_lut()
    img = O.shade_view(v, _records(v, STATUS_CAPTURED), shade_params(shadow_overlay=1), noise, lut)
    green = img[..., 1] > 0.5
    # the ring sits at the shadow's angular radius around the image centre
    a = math.asin(math.sqrt(27.0) / 30.0 * math.sqrt(1 - 2 / 30.0))
    rad_px = math.tan(a) / math.tan(math.radians(20.0)) * 27.0
    jj, ii = np.nonzero(green)
    rr = np.hypot(ii + 0.5 - 48.0, jj + 0.5 - 27.0)
    assert green.sum() > 20 and np.all(np.abs(rr - rad_px) < 2.5)
