"""ctypes loader of the CPU oracle (oracle/_build/liboracle.so) for the tests.

The oracle is test infrastructure: it checks the CUDA path and is never imported by the
product package. It is built from oracle/Makefile on first use.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

from blackholerender_gb300 import BODY_HIT_DTYPE, HIT_DTYPE, Body, ShadeParams, View

ROOT = Path(__file__).resolve().parent.parent
ORACLE_DIR = ROOT / "oracle"
LIB = ORACLE_DIR / "_build" / "liboracle.so"
REF_LIB = ORACLE_DIR / "_ref" / "libbhs_ref.so"

_lib = None
_ref = None


def build():
    subprocess.run(["make", "-s", "-C", str(ORACLE_DIR), "all"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = ctypes.CDLL(str(LIB))
        VP = ctypes.POINTER(View)
        D = ctypes.POINTER(ctypes.c_double)
        L.oracle_trace_view.argtypes = [VP, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.oracle_trace_pixels.argtypes = [VP, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int,
                                          ctypes.c_int]
        L.oracle_primary_rays.argtypes = [VP, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]
        L.oracle_march_ray.argtypes = [VP, D, D, ctypes.c_int, ctypes.c_void_p, D]
        L.oracle_cpu_trace.argtypes = [D, D, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, D,
                                       ctypes.POINTER(ctypes.c_int), D]
        L.oracle_lens_table.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.oracle_rk4_step.argtypes = [D, D, ctypes.c_double, ctypes.c_double]
        L.oracle_initial_velocity.argtypes = [D, D, D]
        L.oracle_far_field.argtypes = [D, D, ctypes.c_double, D]
        L.oracle_noise_bake.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.c_int]
        L.oracle_blackbody_lut.argtypes = [ctypes.c_void_p]
        L.oracle_shade_view.argtypes = [VP, ctypes.c_void_p, ctypes.POINTER(ShadeParams), ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        L.oracle_trace_volumetric.argtypes = [VP, ctypes.POINTER(ShadeParams), ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.oracle_trace_volumetric_pixels.argtypes = [VP, ctypes.POINTER(ShadeParams), ctypes.c_void_p, ctypes.c_void_p,
                                                     ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                                     ctypes.c_int, ctypes.c_int]
        L.oracle_trace_bodies_pixels.argtypes = [VP, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int64,
                                                 ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.oracle_shade_volumetric.argtypes = [VP, ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ShadeParams),
                                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        L.oracle_trace_bodies.argtypes = [VP, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_int, ctypes.c_int]
        L.oracle_shade_bodies.argtypes = [VP, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                          ctypes.POINTER(ShadeParams), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_int]
        L.oracle_trace_bodies_volumetric.argtypes = [VP, ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ShadeParams),
                                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                     ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.oracle_trace_bodies_volumetric_pixels.argtypes = [VP, ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ShadeParams),
                                                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                            ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                                            ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.oracle_shade_bodies_volumetric.argtypes = [VP, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                                     ctypes.c_void_p, ctypes.POINTER(ShadeParams), ctypes.c_void_p,
                                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        L.oracle_redshift_factor.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_float]
        L.oracle_redshift_factor.restype = ctypes.c_float
        L.oracle_blackbody_xyz.argtypes = [ctypes.c_double, D]
        L.oracle_to_half.argtypes = [ctypes.c_float]
        L.oracle_to_half.restype = ctypes.c_uint16
        L.oracle_pcg3d.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.oracle_orbit_view.argtypes = [ctypes.POINTER(View), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_float, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        assert L.oracle_hit_size() == 64 and L.oracle_view_size() == ctypes.sizeof(View)
        _lib = L
    return _lib


def ref_lib():
    """The reference's own Geodesic.h compiled by oracle/Makefile (only where its sources are)."""
    global _ref
    if _ref is None:
        if not REF_LIB.exists():
            return None
        L = ctypes.CDLL(str(REF_LIB))
        D = ctypes.POINTER(ctypes.c_double)
        L.ref_trace.argtypes = [D, D, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, D,
                                ctypes.POINTER(ctypes.c_int), D]
        L.ref_redshift_factor.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double]
        L.ref_redshift_factor.restype = ctypes.c_double
        _ref = L
    return _ref


def orbit_view(term_mode: int, preset: int, width: int, height: int, fov_deg: float, pose) -> View:
    """The oracle's own view of a camera on a sphere looking at the hole (no product library)."""
    v = View()
    r, inc, az = pose
    assert lib().oracle_orbit_view(ctypes.byref(v), term_mode, preset, width, height, fov_deg, r, inc, az) == 0
    return v


def nthreads() -> int:
    return max(1, os.cpu_count() or 1)


def trace_view(view: View, fp64: bool = True, threads: int | None = None) -> np.ndarray:
    out = np.zeros(view.rays, dtype=HIT_DTYPE)
    rc = lib().oracle_trace_view(ctypes.byref(view), out.ctypes.data, threads or nthreads(), int(fp64))
    assert rc == 0, rc
    return out


def trace_pixels(view: View, idx: np.ndarray, fp64: bool = True, threads: int | None = None) -> np.ndarray:
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    out = np.zeros(len(idx), dtype=HIT_DTYPE)
    rc = lib().oracle_trace_pixels(ctypes.byref(view), idx.ctypes.data, len(idx), out.ctypes.data,
                                   threads or nthreads(), int(fp64))
    assert rc == 0, rc
    return out


def lens_table(cam_r: float, alpha_crit: float, fp64: bool = True, threads: int | None = None) -> np.ndarray:
    """The reference's lens-table construction (gas_lens.comp) on the CPU: [1024 angles][1024 rays]."""
    out = np.zeros((1024, 1024), dtype=np.float32)
    rc = lib().oracle_lens_table(ctypes.c_float(cam_r), ctypes.c_float(alpha_crit), out.ctypes.data,
                                 threads or nthreads(), int(fp64))
    assert rc == 0, rc
    return out


def primary_rays(view: View, idx: np.ndarray) -> np.ndarray:
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    out = np.zeros((len(idx), 3), dtype=np.float64)
    assert lib().oracle_primary_rays(ctypes.byref(view), idx.ctypes.data, len(idx), out.ctypes.data) == 0
    return out


def cpu_trace(cam, d, max_steps=200000, step_scale=0.005, esc_tol=1e-4, r_esc_min=30.0):
    """oracle restatement of Geodesic.h trace(): (status, steps, crossings, dir[3], minR)."""
    D3 = ctypes.c_double * 3
    o9 = (ctypes.c_double * 9)()
    oi = (ctypes.c_int * 3)()
    om = ctypes.c_double()
    lib().oracle_cpu_trace(D3(*cam), D3(*d), max_steps, step_scale, esc_tol, r_esc_min, o9, oi, ctypes.byref(om))
    return oi[0], oi[1], oi[2], np.array(o9[6:9]), om.value


def ref_trace(cam, d, max_steps=200000, step_scale=0.005, esc_tol=1e-4, r_esc_min=30.0):
    """The reference's own trace() through oracle/_ref (same return layout as cpu_trace)."""
    L = ref_lib()
    D3 = ctypes.c_double * 3
    o9 = (ctypes.c_double * 9)()
    oi = (ctypes.c_int * 3)()
    om = ctypes.c_double()
    L.ref_trace(D3(*cam), D3(*d), max_steps, step_scale, esc_tol, r_esc_min, o9, oi, ctypes.byref(om))
    return oi[0], oi[1], oi[2], np.array(o9[0:3]), om.value


def angle(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Angle (rad) between direction rows, robust near zero: atan2(|a x b|, a . b) in float64."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    c = np.linalg.norm(np.cross(a, b), axis=-1)
    d = np.sum(a * b, axis=-1)
    return np.arctan2(c, d)


# ---------------------------------------------------------------- shading

def noise_bake(seed: int = 7, threads: int | None = None) -> np.ndarray:
    """The disk's noise volume (noise_bake.comp) as uint16 half bits, shape (z, y, x)."""
    out = np.zeros((128, 128, 128), dtype=np.uint16)
    rc = lib().oracle_noise_bake(seed, out.ctypes.data, threads or nthreads())
    assert rc == 0
    return out


def blackbody_lut() -> np.ndarray:
    out = np.zeros((256, 4), dtype=np.float32)
    assert lib().oracle_blackbody_lut(out.ctypes.data) == 0
    return out


def shade_view(view: View, hits: np.ndarray, params: ShadeParams, noise: np.ndarray, lut: np.ndarray,
               threads: int | None = None) -> np.ndarray:
    """Shades one view from its records; (height, width, 4) float32."""
    hits = np.ascontiguousarray(hits, dtype=HIT_DTYPE)
    noise = np.ascontiguousarray(noise, dtype=np.uint16)
    lut = np.ascontiguousarray(lut, dtype=np.float32)
    assert hits.size == view.width * view.height and noise.size == 128 ** 3 and lut.size == 1024
    out = np.zeros((view.height, view.width, 4), dtype=np.float32)
    rc = lib().oracle_shade_view(ctypes.byref(view), hits.ctypes.data, ctypes.byref(params), noise.ctypes.data,
                                 lut.ctypes.data, out.ctypes.data, threads or nthreads())
    assert rc == 0
    return out


def redshift_factor(r: float, b_axis: float, rcam: float) -> float:
    return lib().oracle_redshift_factor(r, b_axis, rcam)


def blackbody_xyz(T: float) -> np.ndarray:
    out = np.zeros(3)
    lib().oracle_blackbody_xyz(T, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return out


def pcg3d(v) -> tuple[int, int, int]:
    a = np.asarray(v, dtype=np.uint32)
    o = np.zeros(3, dtype=np.uint32)
    lib().oracle_pcg3d(a.ctypes.data, o.ctypes.data)
    return tuple(int(x) for x in o)


def to_half(x: float) -> int:
    return int(lib().oracle_to_half(x))


def trace_volumetric(view: View, params: ShadeParams, noise: np.ndarray, lut: np.ndarray, fp64: bool = True,
                     threads: int | None = None):
    """The volumetric disk's march of every pixel: (records, rgbt (height, width, 4))."""
    noise = np.ascontiguousarray(noise, dtype=np.uint16)
    lut = np.ascontiguousarray(lut, dtype=np.float32)
    hits = np.zeros(view.width * view.height, dtype=HIT_DTYPE)
    rgbt = np.zeros((view.height, view.width, 4), dtype=np.float32)
    rc = lib().oracle_trace_volumetric(ctypes.byref(view), ctypes.byref(params), noise.ctypes.data, lut.ctypes.data,
                                       hits.ctypes.data, rgbt.ctypes.data, threads or nthreads(), int(fp64))
    assert rc == 0
    return hits, rgbt


def trace_volumetric_pixels(view: View, params: ShadeParams, noise: np.ndarray, lut: np.ndarray, idx: np.ndarray,
                            fp64: bool = True, threads: int | None = None):
    """The volumetric march of the listed pixels (j * width + i): (records, rgbt (n, 4))."""
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    noise = np.ascontiguousarray(noise, dtype=np.uint16)
    lut = np.ascontiguousarray(lut, dtype=np.float32)
    hits = np.zeros(len(idx), dtype=HIT_DTYPE)
    rgbt = np.zeros((len(idx), 4), dtype=np.float32)
    rc = lib().oracle_trace_volumetric_pixels(ctypes.byref(view), ctypes.byref(params), noise.ctypes.data,
                                              lut.ctypes.data, idx.ctypes.data, len(idx), hits.ctypes.data,
                                              rgbt.ctypes.data, threads or nthreads(), int(fp64))
    assert rc == 0
    return hits, rgbt


def shade_volumetric(view: View, hits: np.ndarray, rgbt: np.ndarray, params: ShadeParams, noise: np.ndarray,
                     lut: np.ndarray, threads: int | None = None) -> np.ndarray:
    hits = np.ascontiguousarray(hits, dtype=HIT_DTYPE)
    rgbt = np.ascontiguousarray(rgbt, dtype=np.float32)
    out = np.zeros((view.height, view.width, 4), dtype=np.float32)
    rc = lib().oracle_shade_volumetric(ctypes.byref(view), hits.ctypes.data, rgbt.ctypes.data, ctypes.byref(params),
                                       np.ascontiguousarray(noise, dtype=np.uint16).ctypes.data,
                                       np.ascontiguousarray(lut, dtype=np.float32).ctypes.data, out.ctypes.data,
                                       threads or nthreads())
    assert rc == 0
    return out


def trace_bodies(view: View, bodies, fp64: bool = True, threads: int | None = None):
    """The body-aware march of every pixel: (records, body records)."""
    n = len(bodies)
    arr = (Body * max(n, 1))(*bodies)
    hits = np.zeros(view.width * view.height, dtype=HIT_DTYPE)
    bh = np.zeros(view.width * view.height, dtype=BODY_HIT_DTYPE)
    rc = lib().oracle_trace_bodies(ctypes.byref(view), ctypes.cast(arr, ctypes.c_void_p), n, hits.ctypes.data,
                                   bh.ctypes.data, threads or nthreads(), int(fp64))
    assert rc == 0
    return hits, bh


def trace_bodies_pixels(view: View, bodies, idx: np.ndarray, fp64: bool = True, threads: int | None = None):
    """The body-aware march of the listed pixels (j * width + i): (records, body records)."""
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    n = len(bodies)
    arr = (Body * max(n, 1))(*bodies)
    hits = np.zeros(len(idx), dtype=HIT_DTYPE)
    bh = np.zeros(len(idx), dtype=BODY_HIT_DTYPE)
    rc = lib().oracle_trace_bodies_pixels(ctypes.byref(view), ctypes.cast(arr, ctypes.c_void_p), n, idx.ctypes.data,
                                          len(idx), hits.ctypes.data, bh.ctypes.data, threads or nthreads(), int(fp64))
    assert rc == 0
    return hits, bh


def trace_bodies_volumetric(view: View, bodies, params: ShadeParams, noise: np.ndarray, lut: np.ndarray,
                            fp64: bool = True, idx: np.ndarray | None = None, threads: int | None = None):
    """The body-aware march with the volumetric disk, of every pixel or of the listed ones
    (j * width + i): (records, body records, rgbt (n, 4))."""
    n = len(bodies)
    arr = (Body * max(n, 1))(*bodies)
    m = view.width * view.height if idx is None else len(idx)
    hits = np.zeros(m, dtype=HIT_DTYPE)
    bh = np.zeros(m, dtype=BODY_HIT_DTYPE)
    rgbt = np.zeros((m, 4), dtype=np.float32)
    noise = np.ascontiguousarray(noise, dtype=np.uint16)
    lut = np.ascontiguousarray(lut, dtype=np.float32)
    if idx is None:
        rc = lib().oracle_trace_bodies_volumetric(ctypes.byref(view), ctypes.cast(arr, ctypes.c_void_p), n,
                                                  ctypes.byref(params), noise.ctypes.data, lut.ctypes.data,
                                                  hits.ctypes.data, bh.ctypes.data, rgbt.ctypes.data,
                                                  threads or nthreads(), int(fp64))
    else:
        idx = np.ascontiguousarray(idx, dtype=np.int64)
        rc = lib().oracle_trace_bodies_volumetric_pixels(ctypes.byref(view), ctypes.cast(arr, ctypes.c_void_p), n,
                                                         ctypes.byref(params), noise.ctypes.data, lut.ctypes.data,
                                                         idx.ctypes.data, len(idx), hits.ctypes.data, bh.ctypes.data,
                                                         rgbt.ctypes.data, threads or nthreads(), int(fp64))
    assert rc == 0
    return hits, bh, rgbt


def shade_bodies_volumetric(view: View, hits: np.ndarray, body_hits: np.ndarray, bodies, rgbt: np.ndarray,
                            params: ShadeParams, noise: np.ndarray, lut: np.ndarray,
                            threads: int | None = None) -> np.ndarray:
    """Shades a view marched with bodies and the volumetric disk; (height, width, 4) float32."""
    n = len(bodies)
    arr = (Body * max(n, 1))(*bodies)
    hits = np.ascontiguousarray(hits, dtype=HIT_DTYPE)
    body_hits = np.ascontiguousarray(body_hits, dtype=BODY_HIT_DTYPE)
    rgbt = np.ascontiguousarray(rgbt, dtype=np.float32)
    out = np.zeros((view.height, view.width, 4), dtype=np.float32)
    rc = lib().oracle_shade_bodies_volumetric(ctypes.byref(view), hits.ctypes.data, body_hits.ctypes.data,
                                              ctypes.cast(arr, ctypes.c_void_p), n, rgbt.ctypes.data,
                                              ctypes.byref(params), np.ascontiguousarray(noise, dtype=np.uint16).ctypes.data,
                                              np.ascontiguousarray(lut, dtype=np.float32).ctypes.data, out.ctypes.data,
                                              threads or nthreads())
    assert rc == 0
    return out


def shade_bodies(view: View, hits: np.ndarray, body_hits: np.ndarray, bodies, params: ShadeParams, noise: np.ndarray,
                 lut: np.ndarray, threads: int | None = None) -> np.ndarray:
    """Shades a view marched with bodies; (height, width, 4) float32."""
    n = len(bodies)
    arr = (Body * max(n, 1))(*bodies)
    hits = np.ascontiguousarray(hits, dtype=HIT_DTYPE)
    body_hits = np.ascontiguousarray(body_hits, dtype=BODY_HIT_DTYPE)
    out = np.zeros((view.height, view.width, 4), dtype=np.float32)
    rc = lib().oracle_shade_bodies(ctypes.byref(view), hits.ctypes.data, body_hits.ctypes.data, ctypes.cast(arr, ctypes.c_void_p),
                                   n, ctypes.byref(params), np.ascontiguousarray(noise, dtype=np.uint16).ctypes.data,
                                   np.ascontiguousarray(lut, dtype=np.float32).ctypes.data, out.ctypes.data,
                                   threads or nthreads())
    assert rc == 0
    return out
