#!/usr/bin/env python3
"""Writes the golden vectors under tests/golden/ -- TEST INFRASTRUCTURE ONLY.

Sources:
  ref_cpu_trace.npz   the reference's own CPU integrator (src/physics/Geodesic.h, compiled
                      unmodified by `make -C oracle ref` into oracle/_ref/libbhs_ref.so):
                      trace(), impactParameter, impactParameterAboutAxis, shadowAngularRadius
                      on the known-answer inputs of tests/geodesic_tests.cpp plus seeded rays.
  ref_components.npz  the same library's rk4Step, initialVelocity and farFieldDirection on
                      seeded states.
  oracle_c1.npz       the oracle's FP64 shader-rule trace of the 256x144 view (r=30,
                      inclination 85 deg, 200 steps) on every 17th pixel, CONFIG and SHADER
                      termination. The shader cannot run here, so this one is a regression pin
                      of the restatement, not a reference output.

Run from the repository root in a checkout that has the reference sources (REF=... for make):
    make -C oracle all ref && python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import oracle_lib as O  # noqa: E402
from blackholerender_gb300 import TERM_CONFIG, TERM_SHADER, workloads  # noqa: E402


def dir_for_b(D, b):
    """Camera on +z at distance D, ray in the xz-plane with impact parameter b (the reference
    test's construction, tests/geodesic_tests.cpp:27-31)."""
    s = min(1.0, b * np.sqrt(1.0 - 2.0 / D) / D)
    a = np.arcsin(s)
    return np.array([np.sin(a), 0.0, -np.cos(a)])



def trace_cases():
    """(cam[3], dir[3], max_steps, step_scale, esc_tol, r_esc_min, tag) rows."""
    rows = []
    for D in (10.0, 25.0, 2000.0):  # b round trip inputs (:36-48)
        for b in (1.0, 5.196, 8.0):
            if b * np.sqrt(1 - 2 / D) / D < 1:
                rows.append(((0, 0, D), dir_for_b(D, b), 2000, 0.05, 1e-4, 30.0, "b_roundtrip"))
    for b in (50.0, 100.0, 200.0):  # weak field (:50-64)
        rows.append(((0, 0, 2000.0), dir_for_b(2000.0, b), 400000, 0.002, 1e-6, 50.0, "weak_field"))
    for D in (10.0, 25.0, 2000.0):  # capture threshold (:66-78)
        for b in (5.15, 5.25):
            rows.append(((0, 0, D), dir_for_b(D, b), 400000, 0.002, 1e-4, 30.0, "capture_threshold"))
    for b in (8.0, 20.0, 60.0):  # far-field early / late (:145-159)
        d = dir_for_b(2000.0, b)
        rows.append(((0, 0, 2000.0), d, 400000, 0.002, 1e-2, 12.0, "far_early"))
        rows.append(((0, 0, 2000.0), d, 400000, 0.002, 1e-7, 12.0, "far_late"))
    rng = np.random.default_rng(20261203)  # seeded general rays
    for k in range(160):
        r = float(np.exp(rng.uniform(np.log(4.0), np.log(2000.0))))
        cam = rng.normal(size=3)
        cam = cam / np.linalg.norm(cam) * r
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        if k % 2 == 0:  # aim near the hole
            d = -cam / r + 0.3 * d
            d /= np.linalg.norm(d)
        rows.append((tuple(cam), d, 200000, float(rng.uniform(0.005, 0.05)), 1e-4, 30.0, "random"))
    return rows


def ref_trace_full(cam, d, ms, ss, et, re):
    L = O.ref_lib()
    D3 = ctypes.c_double * 3
    o9 = (ctypes.c_double * 9)()
    oi = (ctypes.c_int * 3)()
    om = ctypes.c_double()
    L.ref_trace(D3(*cam), D3(*d), ms, ss, et, re, o9, oi, ctypes.byref(om))
    return list(oi), list(o9), om.value


def main():
    if O.ref_lib() is None:
        sys.exit("oracle/_ref/libbhs_ref.so is missing: run `make -C oracle ref` where the reference sources are")
    rows = trace_cases()
    cams = np.array([r[0] for r in rows], dtype=np.float64)
    dirs = np.array([r[1] for r in rows], dtype=np.float64)
    params = np.array([(r[2], r[3], r[4], r[5]) for r in rows], dtype=np.float64)
    tags = np.array([r[6] for r in rows])
    ints, dir_out, aux, minr = [], [], [], []
    for c, d, p in zip(cams, dirs, params):
        oi, o9, m = ref_trace_full(c, d, int(p[0]), p[1], p[2], p[3])
        ints.append(oi)
        dir_out.append(o9[0:3])
        aux.append(o9[3:6])
        minr.append(m)
    np.savez_compressed(HERE / "ref_cpu_trace.npz", cam=cams, dir=dirs, params=params, tag=tags,
                        status_steps_crossings=np.array(ints, dtype=np.int64), out_dir=np.array(dir_out),
                        b_baxis_shadow=np.array(aux), min_r=np.array(minr))

    L = O.ref_lib()
    D3 = ctypes.c_double * 3
    rng = np.random.default_rng(7)
    n = 64
    x0 = rng.normal(size=(n, 3)) * rng.uniform(3, 50, size=(n, 1))
    v0 = rng.normal(size=(n, 3))
    v0 /= np.linalg.norm(v0, axis=1, keepdims=True)
    h2 = np.sum(np.cross(x0, v0) ** 2, axis=1)
    dt = rng.uniform(0.01, 0.5, size=n)
    x1, v1, iv, ff = [], [], [], []
    for k in range(n):
        X, V = D3(*x0[k]), D3(*v0[k])
        L.ref_rk4_step(X, V, ctypes.c_double(h2[k]), ctypes.c_double(dt[k]))
        x1.append(list(X))
        v1.append(list(V))
        o = D3()
        L.ref_initial_velocity(D3(*x0[k]), D3(*v0[k]), o)
        iv.append(list(o))
        o = D3()
        L.ref_far_field(D3(*x0[k]), D3(*v0[k]), ctypes.c_double(h2[k]), o)
        ff.append(list(o))
    np.savez_compressed(HERE / "ref_components.npz", x0=x0, v0=v0, h2=h2, dt=dt, x1=np.array(x1),
                        v1=np.array(v1), initial_velocity=np.array(iv), far_field=np.array(ff))

    out = {}
    for name, term in (("config", TERM_CONFIG), ("shader", TERM_SHADER)):
        v = workloads.c1_view(term)
        idx = np.arange(0, v.rays, 17, dtype=np.int64)
        h = O.trace_pixels(v, idx, fp64=True)
        out[f"{name}_idx"] = idx
        out[f"{name}_hits"] = h.view(np.uint8).reshape(len(idx), 64)
    np.savez_compressed(HERE / "oracle_c1.npz", **out)
    for f in sorted(HERE.glob("*.npz")):
        print(f.name, f.stat().st_size)


if __name__ == "__main__":
    main()
