"""The learned surrogate trained from scratch by the library's own kernels, with the production
recipe (blackholerender_gb300.train_surrogate's defaults: 1e7 integrator orbits, 200,000 Adam steps
at batch 16,384, learning rate 2e-3 -> 1e-6), and then held to the bars the committed checkpoint
meets: the exit angle on held-out integrator orbits, classification equal to the FP64 oracle and
every escaped surrogate ray within 1e-4 rad of the converged orbit on the 1080p poses, and the rays
just outside the photon-sphere band. About 30 s on one GB300 (orbit generation and training)."""
import numpy as np
import pytest

import oracle_lib as O
import parity
from blackholerender_gb300 import FLAG_SURROGATE, TERM_CONFIG, hits_numpy, workloads
from blackholerender_gb300.surrogate import Surrogate

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def trained():
    import time

    s = Surrogate(seed=1)
    t0 = time.perf_counter()
    counts = s.generate(10_000_000, per_orbit=4, seed=1 * 7919 + 1)
    hist = s.train(200_000, batch=16384, lr_max=2e-3, lr_min=1e-6, w_c=0.01, seed=1)
    print(f"\ngenerated {counts} orbits and trained 200000 steps in {time.perf_counter() - t0:.1f} s; "
          f"loss {hist[:1000, 0].mean():.3e} -> {hist[-1000:, 0].mean():.3e}")
    assert np.all(np.isfinite(hist))
    yield s
    s.close()


def test_fresh_network_exit_angles_on_held_out_orbits(trained):
    held = Surrogate(seed=4)
    held.generate(50_000, per_orbit=4, seed=987654)
    X, lab = held.samples(0, 200_000)
    held.close()
    exit_ = np.zeros(len(lab), bool)
    exit_[3::4] = True
    rc, beta = trained.features_to_orbit(X)
    m = (lab == 0) & exit_ & (np.abs(beta) > 2e-3 / 27 ** 0.5)
    err = np.abs(trained.eval(X[m, :3])[:, 0] - X[m, 3]) * trained.cfg.y_scale
    print(f"\nfresh network, held-out exit angles: p99 {np.percentile(err, 99):.2e} max {err.max():.2e} rad")
    assert np.percentile(err, 99) < 2e-5 and err.max() < 1e-4, (np.percentile(err, 99), err.max())


def test_fresh_network_traces_the_1080p_poses(trained):
    import torch

    views = workloads.c2_views(TERM_CONFIG)[:4]
    outs = trained.trace(views)
    torch.cuda.synchronize()
    st = trained.trace_stats()
    assert st["capture_disagree"] == 0 and st["surrogate"] > 0.999 * sum(v.rays for v in views)
    rng = np.random.default_rng(13)
    worst = 0.0
    for k, (v, o) in enumerate(zip(views, outs)):
        g = hits_numpy(o.cpu())
        idx = rng.choice(v.rays, 2000, replace=False)
        worst = max(worst, parity.check_surrogate(g, v, idx, where=f"fresh network, pose {k}")["dir_max"])
        # rays just outside the fallback band, where the orbit is most sensitive to b
        pool = rng.choice(v.rays, 200_000, replace=False)
        ref = O.trace_pixels(v, pool, fp64=True)
        d = np.abs(ref["b"].astype(np.float64) - 27 ** 0.5)
        near = pool[(d > 2e-3) & (d < 2e-2)][:600]
        if len(near):
            worst = max(worst, parity.check_surrogate(g, v, near, where=f"fresh network near the ring, pose {k}")["dir_max"])
    print(f"\nfresh network vs the converged orbit: max {worst:.2e} rad")
