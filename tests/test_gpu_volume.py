"""The volumetric disk march on the GPU (bhr_trace_volumetric) against the FP64 and FP32 CPU
restatements: classification (escaped / captured / budget / opaque) outside the ill-conditioned
sets, the gathered colour and transmittance, the escape directions; its in-place shading;
argument errors."""
import numpy as np
import pytest

import oracle_lib as O
from blackholerender_gb300 import (DISK_THIN, DISK_VOLUMETRIC, SQRT27, STATUS_ESCAPED, STATUS_OPAQUE, TERM_CONFIG,
                                   TERM_CPU, TERM_SHADER, BhrError, Tracer, hits_numpy, make_view, shade_params)

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


def _run(tracer, v, p):
    import torch

    (h,), (c,) = tracer.trace_volumetric([v], p)
    torch.cuda.synchronize()
    return hits_numpy(h.cpu()).copy(), c.cpu().numpy()


CASES = [
    ("C1-like 256x144, Low, CONFIG", dict(term=TERM_CONFIG, width=256, height=144, preset=0,
                                          pose=(30.0, np.radians(85.0), 0.0)), dict()),
    ("160x90 Medium, shader rule, dense", dict(term=TERM_SHADER, width=160, height=90, preset=1,
                                               pose=(25.0, np.radians(75.0), 1.1)), dict(disk_density=4.0)),
    ("edge-on 128x72 High, Doppler", dict(term=TERM_CONFIG, width=128, height=72, preset=2,
                                          pose=(20.0, np.radians(88.0), 0.3), fov_deg=40.0),
     dict(doppler_strength=1.0, disk_time=33.0)),
]


@pytest.mark.parametrize("name,vk,pk", CASES, ids=[c[0] for c in CASES])
def test_volumetric_march_matches_the_oracle(tracer, tex, name, vk, pk):
    vk = dict(vk)
    v = make_view(vk.pop("term"), disk_mode=DISK_VOLUMETRIC, **vk)
    p = shade_params(**pk)
    g, gc = _run(tracer, v, p)
    r64, c64 = O.trace_volumetric(v, p, *tex, fp64=True)
    r32, c32 = O.trace_volumetric(v, p, *tex, fp64=False)
    T64 = c64[..., 3].reshape(-1)
    # ill-conditioned: the photon-sphere band, a budget decided on the last steps, a transmittance
    # within a factor 2 of the opacity threshold
    amb = ((np.abs(r64["b"] - SQRT27) < 1e-2) | (np.abs(r64["steps"].astype(int) - v.max_steps) <= 2)
           | ((T64 > 0.002) & (T64 < 0.008)))
    cls = (g["status"] != r64["status"]) & ~amb
    cls32 = (r32["status"] != r64["status"]) & ~amb
    same = (g["status"] == r64["status"]) & ~amb
    d = np.abs(gc - c64).reshape(-1, 4)[same]
    d32 = np.abs(c32 - c64).reshape(-1, 4)[same]
    sc = np.abs(c64).reshape(-1, 4)[same] + 1e-3
    e, e32 = d / sc, d32 / sc
    esc = same & (g["status"] == STATUS_ESCAPED) & (r32["status"] == STATUS_ESCAPED)
    ang = O.angle(g["dir"][esc], r64["dir"][esc])
    ang32 = O.angle(r32["dir"][esc], r64["dir"][esc])
    print(f"\n{name}: rays {len(g)}, opaque {int((r64['status'] == STATUS_OPAQUE).sum())}, ambiguous {int(amb.sum())}, "
          f"class mismatches {int(cls.sum())} (FP32 restatement {int(cls32.sum())}); |d rgbt|/(|ref|+1e-3) p50 "
          f"{np.median(e):.1e} p99 {np.percentile(e, 99):.1e} (FP32 restatement p99 {np.percentile(e32, 99):.1e}); "
          f"dir p99 {np.percentile(ang, 99):.1e} rad (FP32 restatement {np.percentile(ang32, 99):.1e}); steps differ on {np.mean(g['steps'][same] != r64['steps'][same]):.4f}")
    assert cls.sum() <= max(2, 3 * cls32.sum())
    assert np.percentile(e, 99) <= max(2e-3, 3 * np.percentile(e32, 99))
    assert np.percentile(ang, 99) <= max(2e-5, 3 * np.percentile(ang32, 99))
    assert np.mean(g["steps"][same] != r64["steps"][same]) < 0.01


def test_volumetric_shading_in_place(tracer, tex):
    import torch

    v = make_view(TERM_CONFIG, width=200, height=112, preset=0, pose=(30.0, np.radians(82.0), 2.0),
                  disk_mode=DISK_VOLUMETRIC)
    p = shade_params(star_density=2.0, doppler_strength=0.5)
    (h,), (c,) = tracer.trace_volumetric([v], p)
    torch.cuda.synchronize()
    hits = hits_numpy(h.cpu()).copy()
    rgbt = c.cpu().numpy().copy()
    tracer.shade([v], [h], p, [c])  # in place
    torch.cuda.synchronize()
    img = c.cpu().numpy()
    ref = O.shade_volumetric(v, hits, rgbt, p, *tex)
    d = np.abs(img - ref)
    bad = np.any(d > 1e-4 * np.abs(ref) + 1e-7, axis=-1)
    print(f"\nvolumetric shading: bad {int(bad.sum())} of {bad.size}, max |d| {d.max():.2e}")
    assert bad.mean() <= 2e-3 and d.max() < 1e-3 * max(1.0, float(np.abs(ref).max()))
    # the disk's own light is kept; opaque pixels carry no sky weight
    assert np.all(img[..., :3] >= rgbt[..., :3] - 1e-6)
    assert np.all(img.reshape(-1, 4)[hits["status"] == STATUS_OPAQUE, 3] == 0.0)


def test_volumetric_argument_errors(tracer):
    import torch

    v = make_view(TERM_CONFIG, width=8, height=8, disk_mode=DISK_VOLUMETRIC)
    h = torch.empty(64 * 64, dtype=torch.uint8, device="cuda")
    c = torch.empty((8, 8, 4), dtype=torch.float32, device="cuda")
    thin = v.copy()
    thin.disk_mode = DISK_THIN
    with pytest.raises(BhrError) as e:
        tracer.trace_volumetric([thin], hits=[h], rgbt=[c])
    assert e.value.code == -1
    cpu = v.copy()
    cpu.term_mode = TERM_CPU
    with pytest.raises(BhrError) as e:
        tracer.trace_volumetric([cpu], hits=[h], rgbt=[c])
    assert e.value.code == -5
    with pytest.raises(BhrError) as e:  # the thin-disk trace still refuses the volumetric disk
        tracer.trace([v], [h])
    assert e.value.code == -5
    hits, rgbt = tracer.trace_volumetric([v], hits=[h], rgbt=[c])  # usable after the errors
    torch.cuda.synchronize()
    assert torch.all((rgbt[0][..., 3] >= 0) & (rgbt[0][..., 3] <= 1))
