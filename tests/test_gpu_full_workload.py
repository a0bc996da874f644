"""Every ray of the benchmark workload (16 poses x 1920x1080, 450 steps, CONFIG rule: 33.2 M
rays) against the FP64 oracle of the same rule, for the learned-surrogate path and for the plain
FP32 path, and the surrogate's escape direction against the converged FP64 orbit on every ray
where the two GPU paths disagree by more than 5e-5 rad.

The sampled tests elsewhere check a few thousand rays per pose; this one leaves no ray out:
  - classification (status and disk yes/no) must match the oracle on every ray outside the
    stated ill-conditioned sets (the photon-sphere band, the budget's last steps, crossings at
    a disk edge), for both paths;
  - the plain path must also meet its FP32 direction and crossing tolerances on the whole image
    (those of the other FP32 tests, against the same statistics of the FP32 oracle);
  - where the two GPU paths' directions differ by more than 5e-5 rad, the converged orbit
    (step scale 0.002, no slab clamp) decides: the surrogate must be within 1e-4 rad of it on
    every such ray.
The oracles run on all host cores (about 9 s per precision for the 33.2 M rays on 16 cores)."""
import numpy as np
import pytest

import oracle_lib as O
import parity
from blackholerender_gb300 import FLAG_SURROGATE, TERM_CONFIG, PREC_FP32, Tracer, hits_numpy, workloads
from blackholerender_gb300.surrogate import DEFAULT_CHECKPOINT, Surrogate

pytestmark = pytest.mark.gpu

SURR_BAND = 2e-3          # the surrogate's fallback band |b - sqrt 27| (those rays are the plain march's)
SURR_EDGE_REL = 1e-3      # surrogate crossings this close to a disk edge are ambiguous both ways
DISAGREE_RAD = 5e-5       # GPU-path disagreement that sends a ray to the converged orbit
DIR_MAX_RAD = 1e-4        # the surrogate's bar against the converged orbit


def converged(view):
    fine = view.copy()
    fine.step_scale = 0.002
    fine.ds_floor = 1e-4
    fine.max_steps = 200000
    fine.disk_mode = 0  # no slab clamp: the orbit itself (directions only)
    return fine


def test_full_workload_against_fp64_oracle():
    import torch

    views = workloads.c2_views(TERM_CONFIG)
    sur = Surrogate(seed=2)
    sur.load(DEFAULT_CHECKPOINT)
    s_out = sur.trace(views)
    with Tracer(0) as tr:
        p_out = tr.trace(views, precision=PREC_FP32)
        torch.cuda.synchronize()
    st = sur.trace_stats()
    tot = {"rays": 0, "s_compared": 0, "s_band": 0, "s_edge": 0, "s_budget": 0, "s_mismatch": 0,
           "p_compared": 0, "p_mismatch": 0, "disagree": 0, "conv_checked": 0}
    worst_s, worst_p = 0.0, 0.0
    for k, (v, so, po) in enumerate(zip(views, s_out, p_out)):
        gs = hits_numpy(so.cpu())
        gp = hits_numpy(po.cpu())
        ref = O.trace_view(v, fp64=True)
        tot["rays"] += v.rays
        # the surrogate path (surrogate records and the plain march's fallback rays)
        rs = parity.compare(gs, ref, max_steps=v.max_steps, band=SURR_BAND, edge_rel=SURR_EDGE_REL)
        assert rs.class_mismatch == 0, (k, rs.as_dict())
        tot["s_compared"] += rs.n_compared
        tot["s_band"] += rs.n_band
        tot["s_edge"] += rs.n_edge_amb
        tot["s_budget"] += rs.n_budget_amb
        tot["s_mismatch"] += rs.class_mismatch
        # the plain FP32 path: classification and its FP32 tolerances on the whole image
        rp = parity.compare(gp, ref, max_steps=v.max_steps, band=1e-2)
        r32 = parity.compare(O.trace_view(v, fp64=False), ref, max_steps=v.max_steps, band=1e-2)
        rp.ref32_dir_p99_scaled = r32.dir_p99_scaled
        rp.ref32_dir_max_scaled = r32.dir_max_scaled
        rp.ref32_cross_r_rel_p99 = r32.cross_r_rel_p99
        parity.assert_fp32_parity(rp, f"pose {k}")
        tot["p_compared"] += rp.n_compared
        tot["p_mismatch"] += rp.class_mismatch
        # where the two GPU paths disagree, the converged orbit decides
        both = ((gs["flags"] & FLAG_SURROGATE) != 0) & (gs["status"] == 1) & (gp["status"] == 1)
        idx = np.nonzero(both)[0]
        a = O.angle(gs["dir"][idx], gp["dir"][idx])
        idx = idx[a > DISAGREE_RAD]
        tot["disagree"] += len(idx)
        if len(idx):
            conv = O.trace_pixels(converged(v), idx, fp64=True)
            ok = conv["status"] == 1
            tot["conv_checked"] += int(ok.sum())
            es = O.angle(gs["dir"][idx][ok], conv["dir"][ok])
            ep = O.angle(gp["dir"][idx][ok], conv["dir"][ok])
            worst_s = max(worst_s, float(es.max(initial=0.0)))
            worst_p = max(worst_p, float(ep.max(initial=0.0)))
            assert es.max(initial=0.0) < DIR_MAX_RAD, (k, float(es.max()), int(idx[ok][np.argmax(es)]))
    print(f"\nfull workload: {tot}; surrogate rays {st['surrogate']}, fallback {st['fallback']}; "
          f"on the disagreeing rays vs the converged orbit: surrogate max {worst_s:.2e} rad, "
          f"plain FP32 max {worst_p:.2e} rad")
    assert tot["rays"] == 16 * 1920 * 1080
    assert tot["s_compared"] > 0.99 * tot["rays"] and tot["p_compared"] > 0.99 * tot["rays"]
    sur.close()
