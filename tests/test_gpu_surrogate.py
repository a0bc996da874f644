"""Learned orbit surrogate: gradient check of the GPU training kernels against the FP64 CPU
network, training data from the integrator against the exact elliptic integral, and a short
training run."""
import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent.parent / "oracle"))
import mlp_ref  # noqa: E402
import orbit_math  # noqa: E402
from blackholerender_gb300.surrogate import Surrogate  # noqa: E402

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


def test_gradients_match_fp64_reference():
    s = Surrogate(seed=3)
    rng = np.random.default_rng(0)
    n = 256
    samples = np.column_stack([rng.uniform(-1, 1, (n, 3)), rng.normal(0, 0.3, n)]).astype(np.float32)
    labels = rng.choice([0, 0, 0, 1, 2], n).astype(np.int8)
    p = s.params()
    loss_g, g_gpu = s.gradients(samples, labels, 0.05)
    loss_c, g_cpu = mlp_ref.loss_and_grad(p, samples, labels, 0.05, quantize=True)
    assert abs(loss_g[2] - loss_c[2]) < 0.5
    assert abs(loss_g[0] - loss_c[0]) < 1e-2 * loss_c[0] + 1e-6
    rels = {}
    for name, (o, sz) in mlp_ref.OFF.items():
        a, b = g_gpu[o:o + sz].astype(np.float64), g_cpu[o:o + sz]
        cos = a @ b / (np.linalg.norm(a) * np.linalg.norm(b) + 1e-30)
        rels[name] = _rel(a, b)
        # the reference mirrors the kernel's BF16 roundings; what differs is the order of the FP32
        # sums and the SFU tanh: measured at most 2.9e-3 (b1), 1.5e-5 to 2e-3 elsewhere
        assert _rel(a, b) < 1e-2 and cos > 0.9999, (name, _rel(a, b), cos)
    print("\ngradient relative L2 error per tensor: " + ", ".join(f"{k} {v:.1e}" for k, v in rels.items()))
    # forward pass of the inference kernel against the same reference
    q = samples[:64, :3]
    out = s.eval(q)
    ref, _ = mlp_ref.forward(p, q.astype(np.float64), quantize=True)
    assert np.max(np.abs(out - ref)) < 1e-2 * np.max(np.abs(ref)) + 1e-4


def test_training_data_matches_exact_orbits():
    # the integrator's polar angle at each sample, minus the closed-form baseline, against the exact
    # elliptic integral (Carlson R_F to convergence) minus the same baseline
    s = Surrogate(seed=5)
    counts = s.generate(4096, per_orbit=4, seed=21)
    assert counts[0] > 2000 and counts[1] > 100 and counts[2] < 0.02 * sum(counts)
    X, lab = s.samples(0, 4096 * 4)
    m = lab == 0
    rc, beta = s.features_to_orbit(X[m])
    sig = X[m, 2].astype(np.float64)
    uc = 1.0 / rc
    u1, u2, u3, d32 = orbit_math.roots(beta)
    u = np.where(sig < 0, u2 - sig ** 2 * (u2 - uc), u2 - sig ** 2 * u2)
    leg = (sig > 0).astype(int)
    exact = orbit_math.phi_of_u(u, uc, beta, leg, ndup=None)
    ic_b, iu_b = orbit_math.base_sweep(uc, beta), orbit_math.base_sweep(u, beta)  # the blended baseline
    base = np.where(leg == 0, ic_b - iu_b, ic_b + iu_b)
    y_exact = (exact - base) / s.cfg.y_scale
    err = np.abs(X[m, 3] - y_exact) * s.cfg.y_scale
    far = np.abs(beta) > 4e-4   # outside the fallback band
    assert np.percentile(err[far], 99) < 2e-6 and err[far].max() < 2e-5, (np.percentile(err[far], 99), err[far].max())
    # captured orbits are exactly those with b < sqrt(27)
    rc_c, beta_c = s.features_to_orbit(X[lab == 1])
    assert np.all(beta_c < 1e-4)


def test_short_training_reduces_loss():
    s = Surrogate(seed=9)
    s.generate(200_000, per_orbit=4, seed=3)
    hist = s.train(600, batch=8192, lr_max=3e-3)
    first = hist[:20, 0].mean()
    last = hist[-20:, 0].mean()
    assert np.all(np.isfinite(hist))
    assert last < 0.2 * first, (first, last)


def test_tensor_core_forward_pass_matches_reference():
    """The evaluation kernel runs the network exactly as the production table build (k_tables)
    does: 128-row tiles through tc::mlp_tile_l1f, layer 1 in FP32 on the CUDA cores, layers 2 and 3
    and the output layer on tcgen05 with TMEM accumulators, biases and W4 as split BF16 parts.
    Against the FP64 network with the GPU's BF16 roundings, on 8192 queries of the trained range."""
    from blackholerender_gb300.surrogate import DEFAULT_CHECKPOINT
    s = Surrogate(seed=1)
    s.load(str(DEFAULT_CHECKPOINT))
    rng = np.random.default_rng(5)
    n = 8192
    q = np.stack([rng.uniform(-1, 1, n), rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)], axis=1).astype(np.float32)
    out = s.eval(q)
    ref, _ = mlp_ref.forward(s.params().astype(np.float64), q.astype(np.float64), quantize=True)
    assert np.all(np.isfinite(out))
    scale = np.abs(ref).max(axis=0)
    p99 = np.percentile(np.abs(out - ref), 99, axis=0)
    # measured p99 4.1e-4 and 4.6e-5 of the output scales (tanh.approx and BF16 rounding flips)
    assert p99[0] < 2e-3 * scale[0] and p99[1] < 3e-4 * scale[1], (p99, scale)


def test_tensor_core_wait_timeout_is_reported():
    """The forward pass's completion waits are bounded: with the MMAs withheld (nothing in flight)
    every wait runs out, the kernel reports it, the call returns ERR_TIMEOUT, and the context is
    still usable for a normal pass afterwards."""
    from blackholerender_gb300 import _abi
    s = Surrogate(seed=2)
    assert s.wait_selftest() == _abi.ERR_TIMEOUT
    q = np.zeros((256, 3), dtype=np.float32)
    out = s.eval(q)
    ref, _ = mlp_ref.forward(s.params().astype(np.float64), q.astype(np.float64), quantize=True)
    assert np.all(np.isfinite(out)) and np.max(np.abs(out - ref)) < 1e-2 * np.max(np.abs(ref)) + 1e-3
