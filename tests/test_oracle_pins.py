"""Pins the CPU oracle (no GPU): against the reference's own integrator, its known answers, and
hand-computed cases for the shader-only rules.

- Golden vectors from the reference's src/physics/Geodesic.h compiled unmodified
  (tests/golden/make_golden.py): the oracle's CPU rule reproduces trace(), rk4Step,
  initialVelocity and farFieldDirection bit for bit.
- The known-answer checks of tests/geodesic_tests.cpp, restated against the oracle.
- Shader rules no reference test pins (crossing interpolation, step rule): a straight-ray
  crossing known in closed form, crossings on the orbit's nodal line, RK4's fifth-order local
  error, and the farMul / 0.02-floor / slab-clamp step sizes against the formulas.
"""
from __future__ import annotations

import ctypes
import math
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle_lib as O
from blackholerender_gb300 import DISK_NONE, HIT_DTYPE, TERM_CONFIG, TERM_SHADER, make_view, workloads

GOLDEN = Path(__file__).resolve().parent / "golden"
D3 = ctypes.c_double * 3


def dir_for_b(D, b):
    """tests/geodesic_tests.cpp:27-31: camera on +z at D, ray in the xz-plane with impact parameter b."""
    a = math.asin(min(1.0, b * math.sqrt(1.0 - 2.0 / D) / D))
    return np.array([math.sin(a), 0.0, -math.cos(a)])


def shadow_angular_radius(r):
    """Geodesic.h:78-82 restated: sin(alpha) = 3 sqrt(3) sqrt(1 - 2/r) / r for a static observer."""
    return math.asin(min(1.0, 3.0 * math.sqrt(3.0) * math.sqrt(1.0 - 2.0 / r) / r))


def march(view, cam, d, fp64=True):
    hit = np.zeros(1, dtype=HIT_DTYPE)
    st = (ctypes.c_double * 9)()
    rc = O.lib().oracle_march_ray(ctypes.byref(view), D3(*cam), D3(*d), int(fp64), hit.ctypes.data, st)
    assert rc == 0
    return hit[0], np.array(st[:])


# ----------------------------------------------------------------------------- golden vectors
def test_cpu_rule_bit_exact_against_reference_golden():
    g = np.load(GOLDEN / "ref_cpu_trace.npz")
    n = len(g["cam"])
    assert n >= 150
    for k in range(n):
        ms, ss, et, re = g["params"][k]
        st, steps, nc, d, mr = O.cpu_trace(g["cam"][k], g["dir"][k], int(ms), ss, et, re)
        s_ref, steps_ref, nc_ref = g["status_steps_crossings"][k]
        assert (st, steps, nc) == (s_ref, steps_ref, nc_ref), (k, g["tag"][k])
        assert np.array_equal(d, g["out_dir"][k]), (k, d, g["out_dir"][k])
        assert mr == g["min_r"][k]


def test_components_bit_exact_against_reference_golden():
    g = np.load(GOLDEN / "ref_components.npz")
    L = O.lib()
    for k in range(len(g["x0"])):
        x, v = D3(*g["x0"][k]), D3(*g["v0"][k])
        L.oracle_rk4_step(x, v, float(g["h2"][k]), float(g["dt"][k]))
        assert np.array_equal(np.array(x[:]), g["x1"][k])
        assert np.array_equal(np.array(v[:]), g["v1"][k])
        o = D3()
        L.oracle_initial_velocity(D3(*g["x0"][k]), D3(*g["v0"][k]), o)
        assert np.array_equal(np.array(o[:]), g["initial_velocity"][k])
        o = D3()
        L.oracle_far_field(D3(*g["x0"][k]), D3(*g["v0"][k]), float(g["h2"][k]), o)
        assert np.array_equal(np.array(o[:]), g["far_field"][k])


def test_impact_parameter_matches_reference():
    """b of the hit record (h / |v_inf|) equals the reference's impactParameter (r sin a / sqrt(1-2/r))
    to 1e-9 relative, as tests/geodesic_tests.cpp:36-48 requires of the round trip."""
    g = np.load(GOLDEN / "ref_cpu_trace.npz")
    v = make_view(TERM_CONFIG, max_steps=1)
    for k in range(len(g["cam"])):
        b_ref = g["b_baxis_shadow"][k][0]
        if not np.isfinite(b_ref):
            continue
        cam = g["cam"][k]
        if np.linalg.norm(cam) < 2.5:
            continue
        hit, _ = march(v, cam, g["dir"][k])
        # the record stores b in float32; the double value is checked through the round trip below
        assert abs(float(hit["b"]) - b_ref) <= 2e-7 * max(1.0, b_ref), (k, hit["b"], b_ref)
    for D in (10.0, 25.0, 2000.0):
        for b in (1.0, 5.196, 8.0):
            if b * math.sqrt(1 - 2 / D) / D >= 1:
                continue
            st, _, _, _, _ = O.cpu_trace((0, 0, D), dir_for_b(D, b), 1, 0.05, 1e-4, 30.0)
            x = np.array([0, 0, D], dtype=np.float64)
            vel = D3()
            O.lib().oracle_initial_velocity(D3(*x), D3(*dir_for_b(D, b)), vel)
            vel = np.array(vel[:])
            h = np.linalg.norm(np.cross(x, vel))
            b2 = h / math.sqrt(np.dot(vel, vel) - 2 * h * h / D ** 3)
            assert abs(b2 - b) < 1e-9 * max(1.0, b)


def test_reference_geodesic_tests_binary_passes():
    exe = O.ORACLE_DIR / "_ref" / "geodesic_tests"
    if not exe.exists():
        pytest.skip("oracle/_ref/geodesic_tests was not built (reference sources absent)")
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:]
    assert "0 failures" in r.stdout


def test_oracle_c1_regression_pin():
    g = np.load(GOLDEN / "oracle_c1.npz")
    for name, term in (("config", TERM_CONFIG), ("shader", TERM_SHADER)):
        v = workloads.c1_view(term)
        idx = g[f"{name}_idx"]
        h = O.trace_pixels(v, idx, fp64=True)
        assert np.array_equal(h.view(np.uint8).reshape(len(idx), 64), g[f"{name}_hits"]), name


# ----------------------------------------------------------------------------- known answers
@pytest.mark.parametrize("b", [50.0, 100.0, 200.0])
def test_weak_field_deflection(b):
    D = 2000.0
    d = dir_for_b(D, b)
    st, _, _, out, _ = O.cpu_trace((0, 0, D), d, 400000, 0.002, 1e-6, 50.0)
    expected = 4.0 / b + 15.0 * math.pi / (4.0 * b * b)
    got = float(O.angle(d, out))
    assert st == 0 and abs(got - expected) / expected < 0.01


@pytest.mark.parametrize("D", [10.0, 25.0, 2000.0])
def test_capture_threshold(D):
    assert O.cpu_trace((0, 0, D), dir_for_b(D, 5.15), 400000, 0.002, 1e-4, 30.0)[0] == 1
    assert O.cpu_trace((0, 0, D), dir_for_b(D, 5.25), 400000, 0.002, 1e-4, 30.0)[0] == 0


@pytest.mark.parametrize("r", [4.0, 6.0, 25.0, 100.0])
def test_shadow_edge(r):
    a = shadow_angular_radius(r)
    da = 0.004
    inside = (math.sin(a - da), 0.0, -math.cos(a - da))
    outside = (math.sin(a + da), 0.0, -math.cos(a + da))
    assert O.cpu_trace((0, 0, r), inside, 400000, 0.002, 1e-4, 30.0)[0] == 1
    assert O.cpu_trace((0, 0, r), outside, 400000, 0.002, 1e-4, 30.0)[0] == 0


def test_photon_sphere_two_orbits():
    L = O.lib()
    x = np.array([3.0, 0.0, 0.0])
    vel = D3()
    L.oracle_initial_velocity(D3(*x), D3(0.0, 0.0, 1.0), vel)
    v = np.array(vel[:])
    h2 = float(np.sum(np.cross(x, v) ** 2))
    X, V = D3(*x), D3(*v)
    ds, path = 0.01, 2.0 * 2.0 * math.pi * 3.0
    dev, s = 0.0, 0.0
    while s < path:
        L.oracle_rk4_step(X, V, h2, ds / math.sqrt(V[0] ** 2 + V[1] ** 2 + V[2] ** 2))
        dev = max(dev, abs(math.sqrt(X[0] ** 2 + X[1] ** 2 + X[2] ** 2) - 3.0))
        s += ds
    assert dev < 1e-4


@pytest.mark.parametrize("b", [8.0, 20.0, 60.0])
def test_far_field_correction_early_vs_late(b):
    d = dir_for_b(2000.0, b)
    e = O.cpu_trace((0, 0, 2000.0), d, 400000, 0.002, 1e-2, 12.0)
    late = O.cpu_trace((0, 0, 2000.0), d, 400000, 0.002, 1e-7, 12.0)
    assert e[0] == 0 and late[0] == 0
    assert float(O.angle(e[3], late[3])) < 5e-4


def test_crossings_above_and_below_the_shadow():
    cam = np.array([0.0, 2.6, 24.9])
    rc = np.linalg.norm(cam)
    to_hole = -cam / rc
    up = np.array([0, 1.0, 0]) - to_hole * to_hole[1]
    up /= np.linalg.norm(up)
    a = shadow_angular_radius(rc) + 0.01
    for sgn in (1.0, -1.0):
        d = to_hole * math.cos(a) + sgn * up * math.sin(a)
        d /= np.linalg.norm(d)
        st, _, nc, _, _ = O.cpu_trace(cam, d, 400000, 0.002, 1e-4, 30.0)
        assert st == 0 and nc >= 1


# ----------------------------------------------------------------------------- shader-only rules
def test_straight_ray_crossing_is_exact():
    """lensing off: straight steps, so the chord interpolation of blackhole.frag:209-216 is exact and
    the crossing is the ray's intersection with y = 0 (disk.glsl:113-116 gives r = |hit.xz|,
    phi = atan(hit.z, hit.x))."""
    v = make_view(TERM_SHADER, lensing=0, max_steps=450)
    cam = np.array([3.0, 4.0, 25.0])
    target = np.array([-9.0, 0.0, 4.0])  # r = sqrt(97) ~ 9.85, inside [6, 20]
    d = (target - cam) / np.linalg.norm(target - cam)
    hit, _ = march(v, cam, d)
    assert hit["ncross"] == 1
    assert abs(float(hit["cross_r"][0]) - math.hypot(-9.0, 4.0)) < 1e-5
    assert abs(float(hit["cross_phi"][0]) - math.atan2(4.0, -9.0)) < 1e-6


def test_lensed_crossings_lie_on_the_nodal_line():
    """Central force: the orbit stays in the plane of x0 and v0, so every crossing of y = 0 lies on
    the line where that plane meets y = 0; its azimuth is fixed up to pi."""
    v = make_view(TERM_CONFIG, max_steps=4000)
    rng = np.random.default_rng(3)
    n_checked = 0
    for _ in range(40):
        cam = np.array([0.0, 3.0, 28.0]) + rng.normal(size=3)
        d = -cam / np.linalg.norm(cam) + 0.12 * rng.normal(size=3)
        d /= np.linalg.norm(d)
        hit, _ = march(v, cam, d)
        if hit["ncross"] == 0:
            continue
        vel = D3()
        O.lib().oracle_initial_velocity(D3(*cam), D3(*d), vel)
        nrm = np.cross(cam, np.array(vel[:]))
        line = np.cross(nrm, [0.0, 1.0, 0.0])  # in the orbit plane and in y = 0
        phi_line = math.atan2(line[2], line[0])
        for c in range(int(hit["ncross"])):
            dphi = (float(hit["cross_phi"][c]) - phi_line) % math.pi
            assert min(dphi, math.pi - dphi) < 1e-5
            n_checked += 1
    assert n_checked >= 10


def test_rk4_local_error_is_fifth_order():
    L = O.lib()
    x0 = np.array([12.0, 1.0, -3.0])
    v0 = np.array([-0.6, 0.1, 0.4])
    v0 /= np.linalg.norm(v0)
    h2 = float(np.sum(np.cross(x0, v0) ** 2))

    def steps(dt, n):
        X, V = D3(*x0), D3(*v0)
        for _ in range(n):
            L.oracle_rk4_step(X, V, h2, dt)
        return np.array(X[:])

    T = 0.8
    truth = steps(T / 4096, 4096)
    e1 = np.linalg.norm(steps(T, 1) - truth)
    e2 = np.linalg.norm(steps(T / 2, 1) - steps(T / 4096, 2048))
    assert 20.0 < e1 / e2 < 45.0  # 2^5 = 32 for a fifth-order local error


def test_step_rule_farmul_floor_and_slab_clamp():
    """The first step of the shader march follows ds = max(stepScale r farMul, 0.02)
    (blackhole.frag:169-170, farMul = clamp((h - 6) / 3, 1, 3)) with the slab clamp of
    blackhole.frag:171-181 near the disk; one step moves the ray by about ds."""
    # far from the disk plane: no clamp
    for cam, d in (((0.0, 40.0, 0.5), (0.0, -1.0, 0.0)), ((0.0, 30.0, 30.0), (0.6, -0.8, 0.0))):
        v = make_view(TERM_SHADER, max_steps=1, disk_mode=DISK_NONE)
        cam = np.array(cam)
        d = np.array(d) / np.linalg.norm(d)
        _, st = march(v, cam, d)
        r = np.linalg.norm(cam)
        vel = D3()
        O.lib().oracle_initial_velocity(D3(*cam), D3(*d), vel)
        h = np.linalg.norm(np.cross(cam, np.array(vel[:])))
        far = min(max((h - 6.0) / 3.0, 1.0), 3.0)
        ds = max(v.step_scale * r * far, 0.02)
        moved = np.linalg.norm(st[0:3] - cam)
        assert abs(moved - ds) < 0.02 * ds, (moved, ds)
    # just above the slab at r_cyl = 15: the step lands on the slab surface (blackhole.frag:178)
    v = make_view(TERM_SHADER, max_steps=1)
    cam = np.array([15.0, 1.6, 0.0])
    d = np.array([0.0, -1.0, 0.0])
    _, st = march(v, cam, d)
    r = np.linalg.norm(cam)
    vel = D3()
    O.lib().oracle_initial_velocity(D3(*cam), D3(*d), vel)
    vel = np.array(vel[:])
    h = np.linalg.norm(np.cross(cam, vel))
    base = max(v.step_scale * r * min(max((h - 6.0) / 3.0, 1.0), 3.0), 0.02)
    outside = 1.6 - 2.5 * v.disk_thickness * 15.0
    ds_slab = min(base, max(v.disk_step, outside / (abs(vel[1]) / np.linalg.norm(vel) + 2.5 * v.disk_thickness)))
    assert ds_slab < 0.5 * base  # the clamp is what sets this step
    moved = np.linalg.norm(st[0:3] - cam)
    assert abs(moved - ds_slab) < 0.02 * ds_slab, (moved, ds_slab)
