"""The shading consumer on the GPU (bhr_shade, bhr_noise_bake) against the CPU restatement:
the noise volume bit for bit, and images shaded from the same hit records within the rounding
of the transcendental functions, across the disk, sky, mixed-quad, odd-size, overlay, Doppler,
far-mode and lensing-off branches, for records of the plain and the surrogate paths."""
import numpy as np
import pytest

import oracle_lib as O
from blackholerender_gb300 import (DISK_NONE, STATUS_ESCAPED, TERM_CONFIG, TERM_SHADER, BhrError,
                                   Tracer, hits_numpy, make_view, shade_params, workloads)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tracer():
    with Tracer(0) as t:
        yield t


@pytest.fixture(scope="module")
def tex(tracer):
    import torch

    noise = tracer.noise_bake(7)
    torch.cuda.synchronize()
    return noise.cpu().numpy().view(np.uint16), O.blackbody_lut()


def test_noise_volume_equals_the_oracle(tracer, tex):
    noise, _ = tex
    ref = O.noise_bake(7)
    assert noise.shape == (128, 128, 128)
    assert np.array_equal(noise, ref)


def _compare(img, ref, where, rel=1e-4, frac=2e-3):
    """Per channel |d| <= rel |ref| + 1e-7 on all but `frac` of the pixels, and every pixel
    within 1e-3 of the image's scale. Only the transcendental functions (logf, expf, powf,
    asinf, acosf) round differently from the CPU's; the star Gaussians exp(-e/2), e < 30,
    carry their last-bit differences into a few pixels."""
    d = np.abs(img - ref)
    tol = rel * np.abs(ref) + 1e-7
    bad_px = np.any(d > tol, axis=-1)
    scale = np.maximum(np.abs(ref), 1e-6)
    r = d / scale
    stats = dict(px=bad_px.size, bad=int(bad_px.sum()), rel_p99=float(np.percentile(r, 99)),
                 rel_max=float(r.max()), abs_max=float(d.max()))
    print(f"\n{where}: {stats}")
    assert np.all(np.isfinite(img))
    assert bad_px.mean() <= frac, (where, stats)
    # the pixels outside the tolerance stay close in absolute terms
    assert d.max() <= 1e-3 * max(1.0, float(np.abs(ref).max())), (where, stats)
    return stats


def _trace_and_shade(tracer, v, params, tex, surrogate=None):
    import torch

    if surrogate is None:
        (h,) = tracer.trace([v])
    else:
        (h,) = surrogate.trace([v])
    (img,) = tracer.shade([v], [h], params)
    torch.cuda.synchronize()
    hits = hits_numpy(h.cpu())
    img = img.cpu().numpy()
    ref = O.shade_view(v, hits, params, *tex)
    return hits, img, ref


def test_c1_default_look(tracer, tex):
    v = workloads.c1_view(TERM_CONFIG)
    hits, img, ref = _trace_and_shade(tracer, v, shade_params(), tex)
    assert np.any(hits["ncross"] > 0) and np.any(hits["status"] == STATUS_ESCAPED)
    _compare(img, ref, "C1 256x144")
    # disk pixels are lit, the shadow is black and carries no sky weight
    disk = hits["ncross"] > 0
    assert img.reshape(-1, 4)[disk, :3].sum(axis=1).min() > 0.0
    cap = (hits["status"] != STATUS_ESCAPED) & (hits["ncross"] == 0)
    assert np.all(img.reshape(-1, 4)[cap] == 0.0)


def test_edge_on_odd_size_doppler_overlay(tracer, tex):
    v = make_view(TERM_CONFIG, width=201, height=113, preset=3, pose=(20.0, np.radians(88.0), 0.7), fov_deg=40.0)
    p = shade_params(doppler_strength=1.0, disk_time=17.3, disk_inflow=0.08, shadow_overlay=1, star_density=2.0,
                     sky_brightness=1.5)
    hits, img, ref = _trace_and_shade(tracer, v, p, tex)
    _compare(img, ref, "edge-on 201x113, Doppler, overlay")
    assert np.any(img[..., 1] > 0.5)  # the overlay's green ring


def test_shader_rule_far_mode_and_lensing_off(tracer, tex):
    for v, where in ((make_view(TERM_SHADER, width=160, height=90, preset=1, pose=(45.0, 1.2, 2.0)), "shader rule"),
                     (make_view(TERM_SHADER, width=64, height=36, pose=(30.0, 1.2, 0.0), far_mode=1), "far mode"),
                     (make_view(TERM_SHADER, width=96, height=54, pose=(30.0, 1.45, 0.2), lensing=0), "lensing off"),
                     (make_view(TERM_CONFIG, width=96, height=54, pose=(30.0, 1.45, 0.2), disk_mode=DISK_NONE),
                      "no disk")):
        _, img, ref = _trace_and_shade(tracer, v, shade_params(), tex)
        _compare(img, ref, where)


def test_surrogate_records_shade_like_the_plain_ones(tracer, tex):
    """Shading parity on the surrogate's records, and the picture the surrogate gives against
    the plain integrator's on a 480x270 pose of the 16-pose workload."""
    from blackholerender_gb300.surrogate import DEFAULT_CHECKPOINT, Surrogate

    v = workloads.c2_views(TERM_CONFIG, width=480, height=270)[0]
    s = Surrogate(seed=2)
    s.load(DEFAULT_CHECKPOINT)
    try:
        p = shade_params()
        hs, img_s, ref_s = _trace_and_shade(tracer, v, p, tex, surrogate=s)
        _compare(img_s, ref_s, "surrogate records 480x270")
    finally:
        s.close()
    hp, img_p, _ = _trace_and_shade(tracer, v, p, tex)
    lum_s = img_s[..., :3].sum(-1)
    lum_p = img_p[..., :3].sum(-1)
    disk = (hp["ncross"] > 0).reshape(lum_p.shape)
    # the disk: per-pixel relative difference of the surrogate's picture against the plain one
    rel = np.abs(lum_s - lum_p)[disk] / np.maximum(lum_p[disk], 1e-6)
    print(f"\nsurrogate vs plain picture: disk pixels {disk.sum()}, |d lum| / lum p50 {np.median(rel):.2e} "
          f"p99 {np.percentile(rel, 99):.2e}; total flux ratio {lum_s.sum() / lum_p.sum():.5f}")
    assert np.median(rel) < 1e-3
    assert abs(lum_s.sum() / lum_p.sum() - 1.0) < 1e-2


def test_non_finite_records(tracer, tex):
    """Records with NaN and infinite directions and crossing radii shade as the restatement
    shades them (finite images, no star light along a NaN direction)."""
    import torch

    v = workloads.c1_view(TERM_CONFIG)
    (h,) = tracer.trace([v])
    torch.cuda.synchronize()
    hits = hits_numpy(h.cpu()).copy()
    rng = np.random.default_rng(4)
    k = rng.choice(hits.size, 200, replace=False)
    hits["dir"][k[:80], 0] = np.nan
    hits["dir"][k[80:120], 1] = np.inf
    hits["cross_r"][k[120:160], 0] = np.nan
    hits["ncross"][k[120:160]] = 1
    hits["cross_phi"][k[160:], 0] = -np.inf
    hits["ncross"][k[160:]] = 1
    hd = torch.from_numpy(hits.view(np.uint8)).cuda()
    p = shade_params()
    (img,) = tracer.shade([v], [hd], p)
    torch.cuda.synchronize()
    img = img.cpu().numpy()
    ref = O.shade_view(v, hits, p, *tex)
    assert np.all(np.isfinite(img)) and np.all(np.isfinite(ref))
    _compare(img, ref, "non-finite records")


def test_shade_argument_errors(tracer):
    import torch

    v = make_view(TERM_CONFIG, width=8, height=8)
    h = torch.zeros(64 * 64, dtype=torch.uint8, device="cuda")
    o = torch.zeros((8, 8, 4), dtype=torch.float32, device="cuda")
    with pytest.raises(BhrError) as e:  # buffers must be 16-byte aligned
        tracer.shade([v], [h[4:]], outs=[o])
    assert e.value.code == -1
    bad = v.copy()
    bad.width = 0
    with pytest.raises(BhrError) as e:
        tracer.shade([bad], [h], outs=[o])
    assert e.value.code == -1
    (img,) = tracer.shade([v], [h], outs=[o])  # zeroed records: captured-like, black
    torch.cuda.synchronize()
    assert torch.all(img == 0)
