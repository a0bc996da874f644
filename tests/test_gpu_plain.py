"""Plain FP32 kernel vs the FP64 oracle, ray by ray (through the C ABI)."""
import numpy as np
import pytest

import oracle_lib as O
import parity
from blackholerender_gb300 import TERM_CONFIG, TERM_CPU, TERM_SHADER, Tracer, hits_numpy, make_view, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tracer():
    import torch

    with Tracer(0) as t:
        yield t
    torch.cuda.synchronize()


def _run(tr, view):
    import torch

    (out,) = tr.trace(view)
    torch.cuda.synchronize()
    return hits_numpy(out.cpu())


@pytest.mark.parametrize("term", [TERM_SHADER, TERM_CONFIG])
def test_c1_full_image(tracer, term):
    v = workloads.c1_view(term)
    gpu = _run(tracer, v)
    rep = parity.check_fp32(gpu, v, where=f"C1 term={term}")
    assert rep.n_compared > 0.95 * rep.n


def test_c2_pose0_reduced(tracer):
    v = workloads.c2_views(TERM_CONFIG, width=480, height=270)[0]
    gpu = _run(tracer, v)
    parity.check_fp32(gpu, v, where="C2 pose0 480x270")


def test_c2_full_res_sampled(tracer):
    views = workloads.c2_views(TERM_CONFIG)
    rng = np.random.default_rng(7)
    for v in views[:4]:
        gpu = _run(tracer, v)
        idx = rng.choice(v.rays, 4000, replace=False)
        parity.check_fp32(gpu, v, idx, where="C2 1080p sample")


def test_cpu_rule(tracer):
    v = make_view(TERM_CPU, width=96, height=54, fov_deg=60.0, pose=(25.0, 1.4, 0.3), max_steps=20000,
                  step_scale=0.02)
    gpu = _run(tracer, v)
    parity.check_fp32(gpu, v, where="CPU rule")
