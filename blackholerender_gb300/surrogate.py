"""The learned orbit surrogate: a context object over the bhr_surrogate_* entry points.

Typical use: generate training orbits with the integrator, train on the GPU, save; later load
the checkpoint and trace views with the surrogate-plus-fallback path.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from . import _abi

DEFAULT_CHECKPOINT = Path(__file__).resolve().parent / "data" / "surrogate.bhrs"

CHECKPOINT_MAGIC = 0x53524842  # "BHRS"
NORM_FIELDS = ("rc_lo", "rc_hi", "b_max", "t_eps", "t_scale", "y_scale", "band", "ue")


def read_checkpoint(path) -> dict:
    """Reads a checkpoint written by bhr_surrogate_save without a GPU: header (magic, version,
    parameter count), the input normalisation, the Adam step and the FP32 parameters in the
    flat layout [W1 (64x3), b1, W2 (64x64), b2, W3 (64x64), b3, W4 (2x64), b4]."""
    raw = Path(path).read_bytes()
    magic, version, n = np.frombuffer(raw, dtype="<u4", count=3)
    if magic != CHECKPOINT_MAGIC or version != 1:
        raise ValueError(f"{path}: not a surrogate checkpoint (magic {magic:#x}, version {version})")
    norm = np.frombuffer(raw, dtype="<f4", count=len(NORM_FIELDS), offset=12)
    step = int(np.frombuffer(raw, dtype="<i4", count=1, offset=12 + 4 * len(NORM_FIELDS))[0])
    off = 16 + 4 * len(NORM_FIELDS)
    if len(raw) != off + 4 * int(n):
        raise ValueError(f"{path}: size {len(raw)} does not match {n} parameters")
    params = np.frombuffer(raw, dtype="<f4", count=int(n), offset=off).copy()
    return {"norm": dict(zip(NORM_FIELDS, map(float, norm))), "adam_step": step, "params": params}


class Surrogate:
    def __init__(self, device=0, seed=1, **cfg):
        L = _abi.lib()
        c = _abi.SurrogateConfig()
        _abi.check(L.bhr_surrogate_default_config(ctypes.byref(c)))
        for k, v in cfg.items():
            setattr(c, k, v)
        self.cfg = c
        self.h = ctypes.c_void_p()
        _abi.check(L.bhr_surrogate_create(ctypes.byref(self.h), device, ctypes.byref(c), seed))

    def close(self):
        if self.h:
            _abi.lib().bhr_surrogate_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def nparams():
        return _abi.lib().bhr_surrogate_param_count()

    def params(self):
        p = np.zeros(self.nparams(), dtype=np.float32)
        _abi.check(_abi.lib().bhr_surrogate_params(self.h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), len(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        _abi.check(_abi.lib().bhr_surrogate_set_params(self.h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), len(p)))

    def gradients(self, samples, labels, w_c):
        s = np.ascontiguousarray(samples, dtype=np.float32)
        lab = np.ascontiguousarray(labels, dtype=np.int8)
        g = np.zeros(self.nparams(), dtype=np.float32)
        loss = np.zeros(3, dtype=np.float32)
        F = ctypes.POINTER(ctypes.c_float)
        _abi.check(_abi.lib().bhr_surrogate_gradients(self.h, s.ctypes.data_as(F),
                                                      lab.ctypes.data_as(ctypes.POINTER(ctypes.c_int8)), len(s),
                                                      ctypes.c_float(w_c), g.ctypes.data_as(F), loss.ctypes.data_as(F)))
        return loss, g

    def eval(self, queries):
        q = np.ascontiguousarray(queries, dtype=np.float32)
        out = np.zeros((len(q), 2), dtype=np.float32)
        F = ctypes.POINTER(ctypes.c_float)
        _abi.check(_abi.lib().bhr_surrogate_eval(self.h, q.ctypes.data_as(F), len(q), out.ctypes.data_as(F)))
        return out

    def wait_selftest(self):
        """Runs the timeout self-test of the forward pass's bounded waits; returns the status code
        (ERR_TIMEOUT when the expired waits were reported)."""
        return int(_abi.lib().bhr_surrogate_wait_selftest(self.h))

    def generate(self, n_orbits, per_orbit=4, seed=7):
        c = (ctypes.c_uint64 * 3)()
        _abi.check(_abi.lib().bhr_surrogate_generate(self.h, n_orbits, per_orbit, seed, None, c))
        return list(c)

    def samples(self, offset, n):
        out = np.zeros((n, 4), dtype=np.float32)
        lab = np.zeros(n, dtype=np.int8)
        _abi.check(_abi.lib().bhr_surrogate_samples(self.h, offset, n, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                                    lab.ctypes.data_as(ctypes.POINTER(ctypes.c_int8))))
        return out, lab

    def features_to_orbit(self, X):
        """(r_cam, beta) of training features (inverse of the input transform)."""
        c = self.cfg
        lrc = (X[:, 0].astype(np.float64) + 1.0) / 2.0 * (np.log(c.rc_hi) - np.log(c.rc_lo)) + np.log(c.rc_lo)
        t = X[:, 1].astype(np.float64) / c.t_scale
        beta = np.sign(t) * c.t_eps * np.expm1(np.abs(t))
        return np.exp(lrc), beta

    def train(self, steps, batch=8192, lr_max=2e-3, lr_min=1e-5, w_c=0.01, seed=11):
        loss = np.zeros(2 * steps, dtype=np.float32)
        _abi.check(_abi.lib().bhr_surrogate_train(self.h, steps, batch, ctypes.c_float(lr_max), ctypes.c_float(lr_min),
                                                  ctypes.c_float(w_c), seed, None,
                                                  loss.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return loss.reshape(steps, 2)

    def save(self, path):
        _abi.check(_abi.lib().bhr_surrogate_save(self.h, str(path).encode()))

    def load(self, path):
        _abi.check(_abi.lib().bhr_surrogate_load(self.h, str(path).encode()))

    def use_network(self, on: bool = True) -> None:
        """bhr_surrogate_use_network: False traces with the non-learned variant (tables from the
        converged closed form, no network)."""
        _abi.check(_abi.lib().bhr_surrogate_use_network(self.h, int(bool(on))))

    def trace(self, views, outs=None, stream=None):
        """Surrogate-plus-fallback trace into device tensors (allocated if None); returns them."""
        import torch

        if isinstance(views, _abi.View):
            views = [views]
        if outs is None:
            outs = [torch.empty(v.rays * 64, dtype=torch.uint8, device="cuda") for v in views]
        if stream is None:
            stream = torch.cuda.current_stream()
        self.trace_ptrs(views, outs, stream)
        return outs

    def trace_ptrs(self, views, outs, stream):
        n = len(views)
        arr = (_abi.View * n)(*views)
        ptrs = (ctypes.c_void_p * n)(*[o.data_ptr() for o in outs])
        _abi.check(_abi.lib().bhr_surrogate_trace(self.h, arr, n, ptrs, ctypes.c_void_p(stream.cuda_stream)))

    def plan(self, views, outs):
        """bhr_surrogate_plan_*: the trace of these views into these device tensors as one CUDA graph."""
        return SurrogatePlan(self, views, outs)

    def trace_host(self, views, outs):
        """bhr_surrogate_trace_host: records land in host arrays (one per view)."""
        n = len(views)
        for v, o in zip(views, outs):
            if o.nbytes < v.rays * 64:
                raise ValueError("host output buffer too small")
        arr = (_abi.View * n)(*views)
        ptrs = (ctypes.c_void_p * n)(*[o.ctypes.data for o in outs])
        _abi.check(_abi.lib().bhr_surrogate_trace_host(self.h, arr, n, ptrs))

    def trace_times_ms(self):
        o = (ctypes.c_float * 2)()
        _abi.check(_abi.lib().bhr_surrogate_trace_times(self.h, o))
        return float(o[0]), float(o[1])

    def trace_stats(self):
        o = (ctypes.c_uint64 * 6)()
        _abi.check(_abi.lib().bhr_surrogate_trace_stats(self.h, o))
        return {"surrogate": o[0], "fallback": o[1], "capture_disagree": o[2], "fallback_steps": o[3],
                "mlp_queries": o[4], "mlp_rows": o[5]}


class SurrogatePlan:
    """A fixed batch of views traced by the surrogate as one replayed CUDA graph."""

    def __init__(self, sur: Surrogate, views, outs):
        self._sur = sur
        self._outs = list(outs)
        n = len(views)
        arr = (_abi.View * n)(*views)
        ptrs = (ctypes.c_void_p * n)(*[o.data_ptr() for o in self._outs])
        self._p = ctypes.c_void_p()
        _abi.check(_abi.lib().bhr_surrogate_plan_create(sur.h, arr, n, ptrs, ctypes.byref(self._p)))

    def launch(self, stream=None):
        import torch

        if stream is None:
            stream = torch.cuda.current_stream()
        _abi.check(_abi.lib().bhr_surrogate_plan_launch(self._p, ctypes.c_void_p(stream.cuda_stream)))

    def update(self, views):
        """New cameras for the plan's views (same count and sizes)."""
        n = len(views)
        arr = (_abi.View * n)(*views)
        _abi.check(_abi.lib().bhr_surrogate_plan_update(self._p, arr, n))

    def close(self):
        if self._p:
            _abi.lib().bhr_surrogate_plan_destroy(self._p)
            self._p = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
