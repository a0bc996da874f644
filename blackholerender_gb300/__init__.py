"""GB300-native Schwarzschild ray tracer: the per-pixel march of DeepjotG/BlackHoleRender.

Python face of the C ABI in include/bhr.h (libbhr.so, built in-tree for sm_103a). Device
buffers and streams come from PyTorch; the work runs in the library's CUDA kernels. There is
no CPU fallback: on a machine without the library or a GB300 the calls raise.
"""
from __future__ import annotations

import ctypes
from typing import Sequence

import numpy as np

from . import _abi
from ._abi import (  # noqa: F401
    DISK_NONE, DISK_THIN, DISK_VOLUMETRIC, FLAG_FALLBACK, FLAG_FP64, FLAG_NONFINITE, FLAG_SURROGATE,
    HIT_DTYPE, METHOD_PLAIN, METHOD_SURROGATE, PREC_FP32, PREC_MIXED, SQRT27, STATUS_BUDGET,
    STATUS_CAPTURED, STATUS_ESCAPED, STATUS_OPAQUE, STATUS_BODY, Body, BODY_HIT_DTYPE, TERM_CONFIG, TERM_CPU, TERM_SHADER, BhrError, LaunchShape, Options,
    ShadeParams, Stats, View,
)

HIT_BYTES = 64


def make_view(term_mode: int = TERM_SHADER, *, width: int | None = None, height: int | None = None,
              fov_deg: float | None = None, preset: int | None = None, pose=None, look_at=None,
              **fields) -> View:
    """A view with the reference defaults (bhr_view_init), then the given overrides.

    pose=(r, inclination_rad, azimuth_rad) places the camera on a sphere looking at the hole;
    look_at=(pos, target) uses Camera::lookAt semantics. Other keyword arguments set fields.
    """
    L = _abi.lib()
    v = View()
    _abi.check(L.bhr_view_init(ctypes.byref(v), term_mode))
    if preset is not None:
        _abi.check(L.bhr_view_apply_preset(ctypes.byref(v), preset))
    if width is not None:
        v.width = width
    if height is not None:
        v.height = height
    if fov_deg is not None:
        _abi.check(L.bhr_view_set_fov(ctypes.byref(v), ctypes.c_float(fov_deg)))
    if pose is not None:
        r, inc, az = pose
        _abi.check(L.bhr_view_orbit_pose(ctypes.byref(v), float(r), float(inc), float(az)))
    if look_at is not None:
        pos, tgt = look_at
        P = (ctypes.c_double * 3)(*map(float, pos))
        T = (ctypes.c_double * 3)(*map(float, tgt))
        _abi.check(L.bhr_view_look_at(ctypes.byref(v), P, T))
    for k, val in fields.items():
        if not hasattr(v, k):
            raise AttributeError(f"bhr_view has no field {k!r}")
        setattr(v, k, val)
    return v


def hits_numpy(buf) -> np.ndarray:
    """Structured numpy view (HIT_DTYPE) of a host uint8 buffer or CPU tensor of records."""
    arr = buf.numpy() if hasattr(buf, "numpy") else np.asarray(buf)
    return arr.view(np.uint8).reshape(-1).view(HIT_DTYPE)


class Tracer:
    """A bhr context on one CUDA device (bhr_create / bhr_trace / bhr_destroy)."""

    def __init__(self, device: int = 0, block_size: int = 0, blocks_per_sm: int = 0, chunk: int = 0,
                 refill: int = 0, tile_w: int = 0):
        L = _abi.lib()
        self._ctx = ctypes.c_void_p()
        opts = Options(device, block_size, blocks_per_sm, chunk, refill, tile_w)
        _abi.check(L.bhr_create(ctypes.byref(self._ctx), ctypes.byref(opts)))
        self.device = device

    def close(self) -> None:
        if self._ctx:
            _abi.lib().bhr_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_surrogate(self, surrogate) -> None:
        """Binds a Surrogate (bhr_ctx_set_surrogate; None unbinds) for method=METHOD_SURROGATE.
        The Tracer does not own it: keep it alive while it is bound."""
        self._surrogate = surrogate
        _abi.check(_abi.lib().bhr_ctx_set_surrogate(self._ctx, surrogate.h if surrogate is not None else None),
                   self._ctx)

    def trace_ptrs(self, views: Sequence[View], out_ptrs: Sequence[int], precision: int = PREC_FP32,
                   method: int = METHOD_PLAIN, stream: int = 0) -> None:
        """bhr_trace on raw device pointers (one per view) and a raw cudaStream_t."""
        n = len(views)
        arr = (View * n)(*views)
        ptrs = (ctypes.c_void_p * n)(*out_ptrs)
        _abi.check(_abi.lib().bhr_trace(self._ctx, arr, n, ptrs, precision, method, ctypes.c_void_p(stream)),
                   self._ctx)

    def trace(self, views: Sequence[View] | View, outs=None, precision: int = PREC_FP32,
              method: int = METHOD_PLAIN, stream=None):
        """Traces views into device tensors (uint8, rays*64 bytes each; allocated if None).

        Runs on `stream` (a torch.cuda.Stream; default: the current stream) and returns the
        list of output tensors without synchronising.
        """
        import torch

        if isinstance(views, View):
            views = [views]
        dev = torch.device("cuda", self.device)
        if outs is None:
            outs = [torch.empty(v.rays * HIT_BYTES, dtype=torch.uint8, device=dev) for v in views]
        if stream is None:
            stream = torch.cuda.current_stream(dev)
        self.trace_ptrs(views, [o.data_ptr() for o in outs], precision, method, stream.cuda_stream)
        return outs

    def trace_host(self, views: Sequence[View], outs: Sequence[np.ndarray], precision: int = PREC_FP32,
                   method: int = METHOD_PLAIN) -> None:
        """bhr_trace_host: records land in host arrays (HIT_DTYPE or uint8, one per view)."""
        n = len(views)
        for v, o in zip(views, outs):
            if o.nbytes < v.rays * HIT_BYTES:
                raise ValueError("host output buffer too small")
        arr = (View * n)(*views)
        ptrs = (ctypes.c_void_p * n)(*[o.ctypes.data for o in outs])
        _abi.check(_abi.lib().bhr_trace_host(self._ctx, arr, n, ptrs, precision, method), self._ctx)

    def stats(self) -> Stats:
        s = Stats()
        _abi.check(_abi.lib().bhr_trace_stats(self._ctx, ctypes.byref(s)), self._ctx)
        return s

    def view_times_ms(self, nviews: int) -> np.ndarray:
        out = (ctypes.c_double * nviews)()
        _abi.check(_abi.lib().bhr_trace_view_times(self._ctx, out, nviews), self._ctx)
        return np.array(out[:], dtype=np.float64)

    # ---- launch shapes, autotuner, graph plans
    @property
    def launch_shape(self) -> LaunchShape:
        sh = LaunchShape()
        _abi.check(_abi.lib().bhr_get_launch_shape(self._ctx, ctypes.byref(sh)), self._ctx)
        return sh

    @launch_shape.setter
    def launch_shape(self, sh: LaunchShape) -> None:
        _abi.check(_abi.lib().bhr_set_launch_shape(self._ctx, ctypes.byref(sh)), self._ctx)

    def autotune(self, views: Sequence[View], outs, precision: int = PREC_FP32, reps: int = 3) -> LaunchShape:
        """bhr_autotune on device tensors `outs` (one per view); returns the chosen shape."""
        n = len(views)
        arr = (View * n)(*views)
        ptrs = (ctypes.c_void_p * n)(*[o.data_ptr() for o in outs])
        best = LaunchShape()
        _abi.check(_abi.lib().bhr_autotune(self._ctx, arr, n, ptrs, precision, reps, ctypes.byref(best)), self._ctx)
        return best

    def lens_table(self, cam_r: float, method: int = METHOD_PLAIN, out=None, stream=None):
        """bhr_lens_table: the 1024 x 1024 lens table (log r, [angle j][ray i]) as a device tensor."""
        import torch

        dev = torch.device("cuda", self.device)
        if out is None:
            out = torch.empty((_abi.LENS_PHIS, _abi.LENS_RAYS), dtype=torch.float32, device=dev)
        if stream is None:
            stream = torch.cuda.current_stream(dev)
        _abi.check(_abi.lib().bhr_lens_table(self._ctx, ctypes.c_float(cam_r), method,
                                             ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream)),
                   self._ctx)
        return out

    def shade(self, views: Sequence[View], hits, params: ShadeParams | None = None, outs=None, stream=None):
        """bhr_shade: hit records (device tensors) -> linear RGB images (height, width, 4) float32.

        rgb is the fragment shader's colour without the sky cube's term; alpha is that term's
        weight. Returns the output tensors."""
        import torch

        dev = torch.device("cuda", self.device)
        n = len(views)
        if params is None:
            params = shade_params()
        if outs is None:
            outs = [torch.empty((v.height, v.width, 4), dtype=torch.float32, device=dev) for v in views]
        if stream is None:
            stream = torch.cuda.current_stream(dev)
        arr = (View * n)(*views)
        hp = (ctypes.c_void_p * n)(*[h.data_ptr() for h in hits])
        op = (ctypes.c_void_p * n)(*[o.data_ptr() for o in outs])
        _abi.check(_abi.lib().bhr_shade(self._ctx, arr, n, hp, ctypes.byref(params), op,
                                        ctypes.c_void_p(stream.cuda_stream)), self._ctx)
        return outs

    def trace_volumetric(self, views: Sequence[View], params: ShadeParams | None = None, hits=None, rgbt=None,
                         stream=None):
        """bhr_trace_volumetric: marches views with the volumetric disk. Returns (hits, rgbt): the
        records (uint8 device tensors) and (height, width, 4) float32 tensors of the gathered rgb
        and transmittance, which shade() completes in place with the sky."""
        import torch

        dev = torch.device("cuda", self.device)
        n = len(views)
        if params is None:
            params = shade_params()
        if hits is None:
            hits = [torch.empty(v.rays * HIT_BYTES, dtype=torch.uint8, device=dev) for v in views]
        if rgbt is None:
            rgbt = [torch.empty((v.height, v.width, 4), dtype=torch.float32, device=dev) for v in views]
        if stream is None:
            stream = torch.cuda.current_stream(dev)
        arr = (View * n)(*views)
        hp = (ctypes.c_void_p * n)(*[h.data_ptr() for h in hits])
        op = (ctypes.c_void_p * n)(*[o.data_ptr() for o in rgbt])
        _abi.check(_abi.lib().bhr_trace_volumetric(self._ctx, arr, n, hp, ctypes.byref(params), op,
                                                   ctypes.c_void_p(stream.cuda_stream)), self._ctx)
        return hits, rgbt

    def trace_bodies(self, view: View, bodies: Sequence[Body], hits=None, body_hits=None, stream=None):
        """bhr_trace_bodies: one view marched with bodies. Returns (hits, body_hits): uint8 device
        tensors of bhr_hit and bhr_body_hit records."""
        import torch

        dev = torch.device("cuda", self.device)
        if hits is None:
            hits = torch.empty(view.rays * HIT_BYTES, dtype=torch.uint8, device=dev)
        if body_hits is None:
            body_hits = torch.empty(view.rays * 64, dtype=torch.uint8, device=dev)
        if stream is None:
            stream = torch.cuda.current_stream(dev)
        n = len(bodies)
        arr = (Body * max(n, 1))(*bodies)
        _abi.check(_abi.lib().bhr_trace_bodies(self._ctx, ctypes.byref(view), arr, n, ctypes.c_void_p(hits.data_ptr()),
                                               ctypes.c_void_p(body_hits.data_ptr()),
                                               ctypes.c_void_p(stream.cuda_stream)), self._ctx)
        return hits, body_hits

    def trace_bodies_volumetric(self, view: View, bodies: Sequence[Body], params: ShadeParams | None = None,
                                hits=None, body_hits=None, rgbt=None, stream=None):
        """bhr_trace_bodies_volumetric: one view marched with bodies and the volumetric disk.
        Returns (hits, body_hits, rgbt): the records, the body records and a (height, width, 4)
        float32 tensor of the gathered rgb and transmittance, which shade_bodies(..., out=rgbt)
        completes in place."""
        import torch

        dev = torch.device("cuda", self.device)
        if params is None:
            params = shade_params()
        if hits is None:
            hits = torch.empty(view.rays * HIT_BYTES, dtype=torch.uint8, device=dev)
        if body_hits is None:
            body_hits = torch.empty(view.rays * 64, dtype=torch.uint8, device=dev)
        if rgbt is None:
            rgbt = torch.empty((view.height, view.width, 4), dtype=torch.float32, device=dev)
        if stream is None:
            stream = torch.cuda.current_stream(dev)
        n = len(bodies)
        arr = (Body * max(n, 1))(*bodies)
        _abi.check(_abi.lib().bhr_trace_bodies_volumetric(
            self._ctx, ctypes.byref(view), arr, n, ctypes.byref(params), ctypes.c_void_p(hits.data_ptr()),
            ctypes.c_void_p(body_hits.data_ptr()), ctypes.c_void_p(rgbt.data_ptr()),
            ctypes.c_void_p(stream.cuda_stream)), self._ctx)
        return hits, body_hits, rgbt

    def shade_bodies(self, view: View, hits, body_hits, bodies: Sequence[Body], params: ShadeParams | None = None,
                     out=None, stream=None):
        """bhr_shade_bodies: shades a view marched by trace_bodies; (height, width, 4) float32. A
        volumetric view is shaded in place: pass the rgbt of trace_bodies_volumetric as `out`."""
        import torch

        dev = torch.device("cuda", self.device)
        if params is None:
            params = shade_params()
        if out is None:
            out = torch.empty((view.height, view.width, 4), dtype=torch.float32, device=dev)
        if stream is None:
            stream = torch.cuda.current_stream(dev)
        n = len(bodies)
        arr = (Body * max(n, 1))(*bodies)
        _abi.check(_abi.lib().bhr_shade_bodies(self._ctx, ctypes.byref(view), ctypes.c_void_p(hits.data_ptr()),
                                               ctypes.c_void_p(body_hits.data_ptr()), arr, n, ctypes.byref(params),
                                               ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream)),
                   self._ctx)
        return out

    def noise_bake(self, seed: int = 7, out=None, stream=None):
        """bhr_noise_bake: the disk's 128^3 noise volume as a device int16 tensor of half bits."""
        import torch

        dev = torch.device("cuda", self.device)
        if out is None:
            out = torch.empty((_abi.NOISE_SIZE,) * 3, dtype=torch.int16, device=dev)
        if stream is None:
            stream = torch.cuda.current_stream(dev)
        _abi.check(_abi.lib().bhr_noise_bake(self._ctx, seed, ctypes.c_void_p(out.data_ptr()),
                                             ctypes.c_void_p(stream.cuda_stream)), self._ctx)
        return out

    def plan(self, views: Sequence[View], outs, precision: int = PREC_FP32, autotune: bool = False) -> "Plan":
        return Plan(self, views, outs, precision, autotune)


def shade_params(**fields) -> ShadeParams:
    """bhr_shade_default_params (the reference's Settings defaults), then the given fields."""
    p = ShadeParams()
    _abi.check(_abi.lib().bhr_shade_default_params(ctypes.byref(p)))
    for k, val in fields.items():
        if not hasattr(p, k):
            raise AttributeError(f"bhr_shade_params has no field {k}")
        setattr(p, k, val)
    return p


def blackbody_lut() -> np.ndarray:
    """bhr_blackbody_lut: (256, 4) float32, rgb of luminance 1 and a = Y / Y(6500 K)."""
    out = np.zeros((_abi.BLACKBODY_LUT, 4), dtype=np.float32)
    _abi.check(_abi.lib().bhr_blackbody_lut(out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
    return out


class Plan:
    """bhr_plan_*: a fixed batch of views traced by one instantiated CUDA graph."""

    def __init__(self, tracer: Tracer, views: Sequence[View], outs, precision: int = PREC_FP32,
                 autotune: bool = False):
        self._tracer = tracer
        self._outs = list(outs)  # keeps the bound device buffers alive
        n = len(views)
        self.nviews = n
        arr = (View * n)(*views)
        ptrs = (ctypes.c_void_p * n)(*[o.data_ptr() for o in self._outs])
        self._p = ctypes.c_void_p()
        _abi.check(_abi.lib().bhr_plan_create(tracer._ctx, arr, n, ptrs, precision, int(autotune),
                                              ctypes.byref(self._p)), tracer._ctx)

    def launch(self, stream=None) -> None:
        import torch

        if stream is None:
            stream = torch.cuda.current_stream(torch.device("cuda", self._tracer.device))
        _abi.check(_abi.lib().bhr_plan_launch(self._p, ctypes.c_void_p(stream.cuda_stream)), self._tracer._ctx)

    def update(self, views: Sequence[View]) -> None:
        n = len(views)
        arr = (View * n)(*views)
        _abi.check(_abi.lib().bhr_plan_update(self._p, arr, n), self._tracer._ctx)

    @property
    def launch_shape(self) -> LaunchShape:
        sh = LaunchShape()
        _abi.check(_abi.lib().bhr_plan_launch_shape(self._p, ctypes.byref(sh)), self._tracer._ctx)
        return sh

    def stats(self) -> Stats:
        s = Stats()
        _abi.check(_abi.lib().bhr_plan_stats(self._p, ctypes.byref(s)), self._tracer._ctx)
        return s

    def view_times_ms(self) -> np.ndarray:
        out = (ctypes.c_double * self.nviews)()
        _abi.check(_abi.lib().bhr_plan_view_times(self._p, out, self.nviews), self._tracer._ctx)
        return np.array(out[:], dtype=np.float64)

    def close(self) -> None:
        if self._p:
            _abi.lib().bhr_plan_destroy(self._p)
            self._p = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
