"""ctypes mirror of include/bhr.h and the loader of the in-tree libbhr.so.

The library is the CUDA path; there is no CPU fallback. Loading fails loudly when
libbhr.so has not been built (``python -c "import __graft_entry__ as g; g.build()"``).
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libbhr.so"

OK = 0
ERR_INVALID_ARG = -1
ERR_OOM = -2
ERR_CUDA = -3
ERR_TIMEOUT = -4
ERR_UNSUPPORTED = -5
ERR_NOT_READY = -6
ERR_IO = -7

STATUS_ESCAPED = 1
STATUS_CAPTURED = 2
STATUS_BUDGET = 3
STATUS_OPAQUE = 4
STATUS_BODY = 5

FLAG_FP64 = 0x01
FLAG_SURROGATE = 0x02
FLAG_FALLBACK = 0x04
FLAG_NONFINITE = 0x08

DISK_NONE = 0
DISK_THIN = 1
DISK_VOLUMETRIC = 2

TERM_SHADER = 0
TERM_CONFIG = 1
TERM_CPU = 2

PREC_FP32 = 0
PREC_MIXED = 1
METHOD_PLAIN = 0
METHOD_SURROGATE = 1

SQRT27 = 27.0 ** 0.5
LENS_RAYS = 1024
LENS_PHIS = 1024
NOISE_SIZE = 128       # BHR_NOISE_SIZE
BLACKBODY_LUT = 256    # BHR_BLACKBODY_LUT


class View(ctypes.Structure):
    _fields_ = [
        ("cam_pos", ctypes.c_float * 3),
        ("cam_basis", ctypes.c_float * 9),
        ("tan_half_fov", ctypes.c_float),
        ("jitter", ctypes.c_float * 2),
        ("width", ctypes.c_int32),
        ("height", ctypes.c_int32),
        ("max_steps", ctypes.c_int32),
        ("step_scale", ctypes.c_float),
        ("disk_step", ctypes.c_float),
        ("disk_inner", ctypes.c_float),
        ("disk_outer", ctypes.c_float),
        ("disk_thickness", ctypes.c_float),
        ("disk_mode", ctypes.c_int32),
        ("lensing", ctypes.c_int32),
        ("far_mode", ctypes.c_int32),
        ("term_mode", ctypes.c_int32),
        ("capture_r", ctypes.c_float),
        ("escape_r", ctypes.c_float),
        ("esc_tol", ctypes.c_float),
        ("r_esc_min", ctypes.c_float),
        ("ds_floor", ctypes.c_float),
        ("promote_band", ctypes.c_float),
        ("promote_r", ctypes.c_float),
        ("reserved", ctypes.c_int32 * 6),
    ]

    def copy(self) -> "View":
        v = View()
        ctypes.memmove(ctypes.byref(v), ctypes.byref(self), ctypes.sizeof(View))
        return v

    @property
    def rays(self) -> int:
        return int(self.width) * int(self.height)


class Options(ctypes.Structure):
    _fields_ = [
        ("device", ctypes.c_int32),
        ("block_size", ctypes.c_int32),
        ("blocks_per_sm", ctypes.c_int32),
        ("chunk", ctypes.c_int32),
        ("refill", ctypes.c_int32),
        ("tile_w", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 2),
    ]


class LaunchShape(ctypes.Structure):
    _fields_ = [
        ("block_size", ctypes.c_int32),
        ("blocks_per_sm", ctypes.c_int32),
        ("chunk", ctypes.c_int32),
        ("refill", ctypes.c_int32),
        ("tile_w", ctypes.c_int32),
        ("ms", ctypes.c_float),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class ShadeParams(ctypes.Structure):
    """bhr_shade_params: the shading uniforms of Renderer::setTraceUniforms (Renderer.cpp:327-346)."""

    _fields_ = [
        ("disk_density", ctypes.c_float),
        ("disk_opacity", ctypes.c_float),
        ("disk_peak_temp", ctypes.c_float),
        ("disk_brightness", ctypes.c_float),
        ("disk_noise_scale", ctypes.c_float),
        ("disk_noise_strength", ctypes.c_float),
        ("disk_time", ctypes.c_float),
        ("disk_warmth", ctypes.c_float),
        ("disk_inflow", ctypes.c_float),
        ("doppler_strength", ctypes.c_float),
        ("sky_brightness", ctypes.c_float),
        ("star_density", ctypes.c_float),
        ("star_brightness", ctypes.c_float),
        ("shadow_overlay", ctypes.c_int32),
        ("noise_seed", ctypes.c_uint32),
        ("time", ctypes.c_float),
        ("reserved", ctypes.c_int32 * 4),
    ]


class Body(ctypes.Structure):
    """bhr_body: the reference's BodyGpu (src/Bodies.h:40-49)."""

    _fields_ = [(f, ctypes.c_float * 4) for f in ("pos_radius", "rel_pos", "look", "tint", "light", "light_color",
                                                  "axis", "ring")]


MAX_BODIES = 32

# numpy view of bhr_body_hit (64 bytes)
BODY_HIT_DTYPE = np.dtype([("body", np.int32), ("t", np.float32), ("ro", np.float32, (3,)), ("rd", np.float32, (3,)),
                           ("x", np.float32, (3,)), ("near_mask", np.uint32), ("near_idx", np.int32),
                           ("near_t", np.float32), ("travelled", np.float32), ("reserved", np.float32)])
assert BODY_HIT_DTYPE.itemsize == 64


class Stats(ctypes.Structure):
    _fields_ = [
        ("rays", ctypes.c_uint64),
        ("steps", ctypes.c_uint64),
        ("fp64_rays", ctypes.c_uint64),
        ("fp64_steps", ctypes.c_uint64),
        ("surrogate_rays", ctypes.c_uint64),
        ("fallback_rays", ctypes.c_uint64),
        ("nonfinite", ctypes.c_uint64),
        ("reserved", ctypes.c_uint64),
    ]


# numpy view of bhr_hit (64 bytes)
HIT_DTYPE = np.dtype(
    [
        ("status", np.uint8),
        ("ncross", np.uint8),
        ("flags", np.uint8),
        ("nplane", np.uint8),
        ("steps", np.uint32),
        ("dir", np.float32, (3,)),
        ("min_r", np.float32),
        ("reserved", np.float32, (2,)),
        ("b_axis", np.float32),
        ("b", np.float32),
        ("cross_r", np.float32, (3,)),
        ("cross_phi", np.float32, (3,)),
    ]
)
assert HIT_DTYPE.itemsize == 64
assert ctypes.sizeof(View) == 160
assert ctypes.sizeof(ShadeParams) == 80

# every entry point include/bhr.h declares, with its ctypes signature
_P = ctypes.c_void_p
_VP = ctypes.POINTER(View)
SIGNATURES = {
    "bhr_abi_version": (ctypes.c_int, []),
    "bhr_create": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.POINTER(Options)]),
    "bhr_destroy": (ctypes.c_int, [_P]),
    "bhr_last_error": (ctypes.c_char_p, [_P]),
    "bhr_view_init": (ctypes.c_int, [_VP, ctypes.c_int]),
    "bhr_view_apply_preset": (ctypes.c_int, [_VP, ctypes.c_int]),
    "bhr_view_look_at": (ctypes.c_int, [_VP, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "bhr_view_set_fov": (ctypes.c_int, [_VP, ctypes.c_float]),
    "bhr_look_rotation": (ctypes.c_int, [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                         ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]),
    "bhr_view_set_pose": (ctypes.c_int, [_VP, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_float)]),
    "bhr_view_orbit_pose": (ctypes.c_int, [_VP, ctypes.c_double, ctypes.c_double, ctypes.c_double]),
    "bhr_view_rays": (ctypes.c_int64, [_VP]),
    "bhr_trace": (ctypes.c_int, [_P, _VP, ctypes.c_int, ctypes.POINTER(_P), ctypes.c_int, ctypes.c_int, _P]),
    "bhr_trace_host": (ctypes.c_int, [_P, _VP, ctypes.c_int, ctypes.POINTER(_P), ctypes.c_int, ctypes.c_int]),
    "bhr_ctx_set_surrogate": (ctypes.c_int, [_P, _P]),
    "bhr_trace_noalloc": (ctypes.c_int, [_VP, _P, _P]),
    "bhr_trace_stats": (ctypes.c_int, [_P, ctypes.POINTER(Stats)]),
    "bhr_trace_view_times": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double), ctypes.c_int]),
    "bhr_lens_table": (ctypes.c_int, [_P, ctypes.c_float, ctypes.c_int, _P, _P]),
    "bhr_lens_alpha": (ctypes.c_float, [ctypes.c_float, ctypes.c_float]),
    "bhr_shadow_angular_radius": (ctypes.c_double, [ctypes.c_double]),
    "bhr_shade_default_params": (ctypes.c_int, [ctypes.POINTER(ShadeParams)]),
    "bhr_shade": (ctypes.c_int, [_P, _VP, ctypes.c_int, ctypes.POINTER(_P), ctypes.POINTER(ShadeParams),
                                 ctypes.POINTER(_P), _P]),
    "bhr_trace_volumetric": (ctypes.c_int, [_P, _VP, ctypes.c_int, ctypes.POINTER(_P), ctypes.POINTER(ShadeParams),
                                            ctypes.POINTER(_P), _P]),
    "bhr_trace_bodies": (ctypes.c_int, [_P, _VP, ctypes.POINTER(Body), ctypes.c_int, _P, _P, _P]),
    "bhr_trace_bodies_volumetric": (ctypes.c_int, [_P, _VP, ctypes.POINTER(Body), ctypes.c_int,
                                                   ctypes.POINTER(ShadeParams), _P, _P, _P, _P]),
    "bhr_shade_bodies": (ctypes.c_int, [_P, _VP, _P, _P, ctypes.POINTER(Body), ctypes.c_int, ctypes.POINTER(ShadeParams),
                                        _P, _P]),
    "bhr_noise_bake": (ctypes.c_int, [_P, ctypes.c_uint32, _P, _P]),
    "bhr_blackbody_lut": (ctypes.c_int, [ctypes.POINTER(ctypes.c_float)]),
    "bhr_get_launch_shape": (ctypes.c_int, [_P, ctypes.POINTER(LaunchShape)]),
    "bhr_set_launch_shape": (ctypes.c_int, [_P, ctypes.POINTER(LaunchShape)]),
    "bhr_autotune": (ctypes.c_int, [_P, _VP, ctypes.c_int, ctypes.POINTER(_P), ctypes.c_int, ctypes.c_int,
                                    ctypes.POINTER(LaunchShape)]),
    "bhr_plan_create": (ctypes.c_int, [_P, _VP, ctypes.c_int, ctypes.POINTER(_P), ctypes.c_int, ctypes.c_int,
                                       ctypes.POINTER(_P)]),
    "bhr_plan_update": (ctypes.c_int, [_P, _VP, ctypes.c_int]),
    "bhr_plan_launch": (ctypes.c_int, [_P, _P]),
    "bhr_plan_launch_shape": (ctypes.c_int, [_P, ctypes.POINTER(LaunchShape)]),
    "bhr_plan_stats": (ctypes.c_int, [_P, ctypes.POINTER(Stats)]),
    "bhr_plan_view_times": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double), ctypes.c_int]),
    "bhr_plan_destroy": (ctypes.c_int, [_P]),
}

class SurrogateConfig(ctypes.Structure):
    _fields_ = [
        ("rc_lo", ctypes.c_float), ("rc_hi", ctypes.c_float), ("b_max", ctypes.c_float), ("band", ctypes.c_float),
        ("t_eps", ctypes.c_float), ("t_scale", ctypes.c_float), ("y_scale", ctypes.c_float),
        ("escape_r", ctypes.c_float), ("reserved", ctypes.c_int32 * 8),
    ]


_F = ctypes.POINTER(ctypes.c_float)
SIGNATURES.update({
    "bhr_surrogate_default_config": (ctypes.c_int, [ctypes.POINTER(SurrogateConfig)]),
    "bhr_surrogate_create": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int, ctypes.POINTER(SurrogateConfig),
                                            ctypes.c_uint64]),
    "bhr_surrogate_destroy": (ctypes.c_int, [_P]),
    "bhr_surrogate_generate": (ctypes.c_int, [_P, ctypes.c_int64, ctypes.c_int, ctypes.c_uint64, _P,
                                              ctypes.POINTER(ctypes.c_uint64)]),
    "bhr_surrogate_train": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                           ctypes.c_float, ctypes.c_uint64, _P, _F]),
    "bhr_surrogate_samples": (ctypes.c_int, [_P, ctypes.c_int64, ctypes.c_int64, _F, ctypes.POINTER(ctypes.c_int8)]),
    "bhr_surrogate_param_count": (ctypes.c_int, []),
    "bhr_surrogate_params": (ctypes.c_int, [_P, _F, ctypes.c_int]),
    "bhr_surrogate_set_params": (ctypes.c_int, [_P, _F, ctypes.c_int]),
    "bhr_surrogate_gradients": (ctypes.c_int, [_P, _F, ctypes.POINTER(ctypes.c_int8), ctypes.c_int, ctypes.c_float,
                                               _F, _F]),
    "bhr_surrogate_eval": (ctypes.c_int, [_P, _F, ctypes.c_int, _F]),
    "bhr_surrogate_wait_selftest": (ctypes.c_int, [_P]),
    "bhr_surrogate_save": (ctypes.c_int, [_P, ctypes.c_char_p]),
    "bhr_surrogate_load": (ctypes.c_int, [_P, ctypes.c_char_p]),
    "bhr_surrogate_trace": (ctypes.c_int, [_P, _VP, ctypes.c_int, ctypes.POINTER(_P), _P]),
    "bhr_surrogate_use_network": (ctypes.c_int, [_P, ctypes.c_int]),
    "bhr_surrogate_trace_stats": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_uint64)]),
    "bhr_surrogate_trace_host": (ctypes.c_int, [_P, _VP, ctypes.c_int, ctypes.POINTER(_P)]),
    "bhr_surrogate_trace_times": (ctypes.c_int, [_P, _F]),
    "bhr_surrogate_plan_create": (ctypes.c_int, [_P, _VP, ctypes.c_int, ctypes.POINTER(_P), ctypes.POINTER(_P)]),
    "bhr_surrogate_plan_launch": (ctypes.c_int, [_P, _P]),
    "bhr_surrogate_plan_update": (ctypes.c_int, [_P, _VP, ctypes.c_int]),
    "bhr_surrogate_plan_destroy": (ctypes.c_int, [_P]),
})

_lib = None


class BhrError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"bhr error {code}: {msg}")
        self.code = code


def lib() -> ctypes.CDLL:
    """The loaded libbhr.so; raises if it was not built (no CPU fallback exists)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is missing: build the CUDA library first "
                "(python -c 'import __graft_entry__ as g; g.build()')"
            )
        L = ctypes.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(code: int, ctx=None) -> None:
    if code != OK:
        msg = lib().bhr_last_error(ctx)
        raise BhrError(code, msg.decode() if msg else "")
