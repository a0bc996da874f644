"""Bodies on the GPU against the CPU restatements: the body-aware march (bhr_trace_bodies:
which rays stop on which body, the near-field and chord hit geometry, the records of the rays
that miss every body, against FP64 and FP32) and the shading of bodies (bhr_shade_bodies: all
nine planet looks, a star, an exploding photosphere, rings, translucency, halos)."""
import math

import numpy as np
import pytest

import oracle_lib as O
from blackholerender_gb300 import (BODY_HIT_DTYPE, DISK_NONE, DISK_THIN, DISK_VOLUMETRIC, SQRT27, STATUS_BODY,
                                   TERM_CONFIG, TERM_SHADER, BhrError, Tracer, hits_numpy, make_view, workloads)
from test_cpu_bodies import body

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tracer():
    with Tracer(0) as t:
        yield t


def _scene(v):
    cam = np.array(v.cam_pos, dtype=np.float64)
    rhat = cam / np.linalg.norm(cam)
    return [body(cam - 6.0 * rhat + np.array([0.5, 0.3, 0.0]), 0.6, cam),               # near field
            body(-40.0 * rhat, 3.0, cam, ring=(4.0, 7.0, 0.0, 1.0)),                       # behind the hole
            body(np.array([25.0, 2.0, -10.0]), 1.5, cam, kind=1.0),                        # off to the side
            body(cam + np.array([0.3, -0.2, 0.0]) - 0.02 * rhat, 0.004, cam)]              # tiny, close by


CASES = [("256x144 Low, thin disk, CONFIG", dict(term=TERM_CONFIG, width=256, height=144, preset=0,
                                                 pose=(30.0, math.radians(80.0), 0.4), disk_mode=DISK_THIN), True),
         ("160x90 Medium, no disk, shader rule", dict(term=TERM_SHADER, width=160, height=90, preset=1,
                                                      pose=(25.0, math.radians(60.0), 1.0), disk_mode=DISK_NONE), False)]


def _normals(bh, bodies, m):
    """Unit normals at the chord hits m: (ro + rd t - centre) / |.|"""
    c = np.array([bodies[k].pos_radius[:3] for k in bh["body"][m]], dtype=np.float64)
    p = bh["ro"][m].astype(np.float64) + bh["rd"][m].astype(np.float64) * bh["t"][m, None].astype(np.float64) - c
    return p / np.linalg.norm(p, axis=1, keepdims=True)


@pytest.mark.parametrize("name,vk,has_chord", CASES, ids=[c[0] for c in CASES])
def test_body_march_matches_the_oracle(tracer, name, vk, has_chord):
    import torch

    vk = dict(vk)
    v = make_view(vk.pop("term"), **vk)
    bodies = _scene(v)
    h, bhd = tracer.trace_bodies(v, bodies)
    torch.cuda.synchronize()
    g = hits_numpy(h.cpu())
    gb = bhd.cpu().numpy().view(np.uint8).reshape(-1).view(BODY_HIT_DTYPE)
    r64, b64 = O.trace_bodies(v, bodies, fp64=True)
    r32, b32 = O.trace_bodies(v, bodies, fp64=False)
    amb = (np.abs(r64["b"] - SQRT27) < 1e-2) | (np.abs(r64["steps"].astype(int) - v.max_steps) <= 2)
    mism = ((g["status"] != r64["status"]) | (gb["body"] != b64["body"])) & ~amb
    mism32 = ((r32["status"] != r64["status"]) | (b32["body"] != b64["body"])) & ~amb
    hit = (g["status"] == STATUS_BODY) & (r64["status"] == STATUS_BODY) & (gb["body"] == b64["body"])
    chord = hit & (b64["t"] > 0)
    near = hit & (b64["t"] == 0)
    dn = np.abs(gb["near_t"][near] - b64["near_t"][near]) / b64["near_t"][near]
    chord32 = chord & (r32["status"] == STATUS_BODY) & (b32["body"] == b64["body"]) & (b32["t"] > 0)
    na = O.angle(_normals(gb, bodies, chord32), _normals(b64, bodies, chord32)) if chord32.any() else np.zeros(1)
    na32 = O.angle(_normals(b32, bodies, chord32), _normals(b64, bodies, chord32)) if chord32.any() else np.zeros(1)
    print(f"\n{name}: body hits {int(hit.sum())} (near {int(near.sum())}, chord {int(chord.sum())}), status/body "
          f"mismatches {int(mism.sum())} (FP32 restatement {int(mism32.sum())}); chord-hit normal p99 "
          f"{np.percentile(na, 99):.1e} rad (FP32 restatement {np.percentile(na32, 99):.1e}), near t rel max "
          f"{dn.max() if dn.size else 0:.1e}")
    assert hit.sum() > 50 and near.sum() > 0 and (chord.sum() > 0) == has_chord
    assert mism.sum() <= max(3, 3 * mism32.sum())
    assert np.all(gb["near_mask"] == b64["near_mask"])
    assert (dn.max() if dn.size else 0) < 1e-4
    assert np.percentile(na, 99) <= max(1e-4, 3 * np.percentile(na32, 99))
    # the rays that miss every body: the same records as the plain march's parity bar
    miss = (r64["status"] != STATUS_BODY) & (g["status"] != STATUS_BODY) & ~amb
    esc = miss & (g["status"] == 1) & (r64["status"] == 1)
    ang = O.angle(g["dir"][esc], r64["dir"][esc])
    ang32 = O.angle(r32["dir"][esc], r64["dir"][esc])
    assert np.percentile(ang, 99) <= max(2e-5, 3 * np.percentile(ang32, 99))


def test_body_march_argument_errors(tracer):
    v = make_view(TERM_CONFIG, width=8, height=8, disk_mode=DISK_VOLUMETRIC)
    cam = np.array(v.cam_pos, dtype=np.float64)
    with pytest.raises(BhrError) as e:
        tracer.trace_bodies(v, [body(np.zeros(3) + 40, 1.0, cam)])
    assert e.value.code == -5
    v.disk_mode = DISK_THIN
    with pytest.raises(BhrError) as e:
        tracer.trace_bodies(v, [body(np.zeros(3) + 40, 1.0, cam)] * 33)
    assert e.value.code == -1
    with pytest.raises(BhrError) as e:
        tracer.trace_bodies(v, [body(np.zeros(3) + 40, 0.0, cam)])
    assert e.value.code == -1


def test_body_shading_matches_the_oracle(tracer):
    import torch

    from blackholerender_gb300 import shade_params

    v = make_view(TERM_CONFIG, width=320, height=180, preset=0, pose=(30.0, math.radians(70.0), 0.4), disk_mode=DISK_THIN)
    bodies = workloads.body_gallery(v)
    p = shade_params(time=37.0, doppler_strength=0.5)
    h, bhd = tracer.trace_bodies(v, bodies)
    img = tracer.shade_bodies(v, h, bhd, bodies, p)
    noise = tracer.noise_bake(7)
    torch.cuda.synchronize()
    g = hits_numpy(h.cpu())
    gb = bhd.cpu().numpy().view(np.uint8).reshape(-1).view(BODY_HIT_DTYPE)
    img = img.cpu().numpy()
    ref = O.shade_bodies(v, g, gb, bodies, p, noise.cpu().numpy().view(np.uint16), O.blackbody_lut())
    on = g["status"] == STATUS_BODY
    per_body = np.bincount(gb["body"][on], minlength=12)
    d = np.abs(img - ref)
    bad = np.any(d > 1e-4 * np.abs(ref) + 1e-6, axis=-1).reshape(-1)
    r = (d / np.maximum(np.abs(ref), 1e-6)).reshape(-1, 4)
    print(f"\nbody shading 320x180: body pixels {int(on.sum())}, per body {per_body.tolist()}; outside 1e-4: "
          f"{int(bad.sum())} ({int(bad[on].sum())} on bodies), rel p99 on bodies {np.percentile(r[on], 99):.1e}, "
          f"max |d| {d.max():.2e}")
    assert np.all(per_body > 30)
    assert np.all(np.isfinite(img))
    assert bad.mean() <= 2e-3 and bad[on].mean() <= 2e-3
    assert d.max() <= 1e-3 * max(1.0, float(np.abs(ref).max()))


def _vol_scene(term=TERM_CONFIG):
    """The volumetric disk with the planet below the disk plane (tests/test_cpu_bodies_volumetric)
    and the near-field, far-side and side bodies of the thin-disk cases."""
    from test_cpu_bodies_volumetric import scene

    v, below = scene(192, 108, term)
    return v, below + _scene(v)


@pytest.mark.parametrize("density,term", [(1.0, TERM_CONFIG), (6.0, TERM_CONFIG), (2.0, TERM_SHADER)],
                         ids=["density 1, CONFIG", "density 6, CONFIG", "density 2, shader rule"])
def test_volumetric_body_march_matches_the_oracle(tracer, density, term):
    import torch

    from blackholerender_gb300 import STATUS_OPAQUE, shade_params

    v, bodies = _vol_scene(term)
    p = shade_params(disk_density=density)
    h, bhd, rgbt = tracer.trace_bodies_volumetric(v, bodies, p)
    noise = tracer.noise_bake(7)
    torch.cuda.synchronize()
    g = hits_numpy(h.cpu())
    gb = bhd.cpu().numpy().view(np.uint8).reshape(-1).view(BODY_HIT_DTYPE)
    gc = rgbt.cpu().numpy().reshape(-1, 4)
    tex = (noise.cpu().numpy().view(np.uint16), O.blackbody_lut())
    r64, b64, c64 = O.trace_bodies_volumetric(v, bodies, p, *tex, fp64=True)
    r32, b32, c32 = O.trace_bodies_volumetric(v, bodies, p, *tex, fp64=False)
    T = c64[:, 3]
    # ill-conditioned: the photon-sphere band, a budget decided on the last steps, a transmittance
    # within a factor 2 of the opacity threshold
    amb = ((np.abs(r64["b"] - SQRT27) < 1e-2) | (np.abs(r64["steps"].astype(int) - v.max_steps) <= 2)
           | ((T > 0.002) & (T < 0.008)))
    mism = ((g["status"] != r64["status"]) | (gb["body"] != b64["body"])) & ~amb
    mism32 = ((r32["status"] != r64["status"]) | (b32["body"] != b64["body"])) & ~amb
    same = (g["status"] == r64["status"]) & (gb["body"] == b64["body"]) & ~amb
    e = (np.abs(gc - c64) / (np.abs(c64) + 1e-3))[same]
    same32 = same & (r32["status"] == r64["status"]) & (b32["body"] == b64["body"])
    e32 = (np.abs(c32 - c64) / (np.abs(c64) + 1e-3))[same32]
    hit = same & (g["status"] == STATUS_BODY)
    print(f"\nvolumetric + bodies, density {density}, rule {term}: body hits {int(hit.sum())} (through the slab "
          f"{int((hit & (T < 0.99)).sum())}), opaque {int((r64['status'] == STATUS_OPAQUE).sum())}, status/body "
          f"mismatches {int(mism.sum())} (FP32 restatement {int(mism32.sum())}); |d rgbt|/(|ref|+1e-3) p99 "
          f"{np.percentile(e, 99):.1e} (FP32 restatement {np.percentile(e32, 99):.1e})")
    assert hit.sum() > 100 and (hit & (T < 0.99)).sum() > 50
    assert mism.sum() <= max(3, 3 * mism32.sum())
    assert np.percentile(e, 99) <= max(2e-3, 3 * np.percentile(e32, 99))
    assert np.all(gb["near_mask"] == b64["near_mask"])
    esc = same & (g["status"] == 1) & (r32["status"] == 1)
    ang = O.angle(g["dir"][esc], r64["dir"][esc])
    ang32 = O.angle(r32["dir"][esc], r64["dir"][esc])
    assert np.percentile(ang, 99) <= max(2e-5, 3 * np.percentile(ang32, 99))


def test_volumetric_body_shading_in_place(tracer):
    import torch

    from blackholerender_gb300 import shade_params

    v, bodies = _vol_scene()
    p = shade_params(time=21.0, doppler_strength=0.5)
    h, bhd, rgbt = tracer.trace_bodies_volumetric(v, bodies, p)
    noise = tracer.noise_bake(7)
    torch.cuda.synchronize()
    g = hits_numpy(h.cpu()).copy()
    gb = bhd.cpu().numpy().view(np.uint8).reshape(-1).view(BODY_HIT_DTYPE).copy()
    march = rgbt.cpu().numpy().copy()
    img = tracer.shade_bodies(v, h, bhd, bodies, p, out=rgbt)  # in place
    torch.cuda.synchronize()
    img = img.cpu().numpy()
    ref = O.shade_bodies_volumetric(v, g, gb, bodies, march.reshape(-1, 4), p, noise.cpu().numpy().view(np.uint16),
                                    O.blackbody_lut())
    on = g["status"] == STATUS_BODY
    d = np.abs(img - ref)
    bad = np.any(d > 1e-4 * np.abs(ref) + 1e-6, axis=-1).reshape(-1)
    print(f"\nvolumetric body shading 192x108: body pixels {int(on.sum())}; outside 1e-4: {int(bad.sum())} "
          f"({int(bad[on].sum())} on bodies), max |d| {d.max():.2e}")
    assert on.sum() > 100 and np.all(np.isfinite(img))
    assert bad.mean() <= 2e-3 and bad[on].mean() <= 2e-3
    assert d.max() <= 1e-3 * max(1.0, float(np.abs(ref).max()))
    # the disk's light in front of a body is kept
    assert np.all(img.reshape(-1, 4)[on, :3] >= march.reshape(-1, 4)[on, :3] - 1e-6)


def test_volumetric_body_march_argument_errors(tracer):
    from blackholerender_gb300 import shade_params

    v, bodies = _vol_scene()
    thin = v.copy()
    thin.disk_mode = DISK_THIN
    with pytest.raises(BhrError) as e:
        tracer.trace_bodies_volumetric(thin, bodies, shade_params())
    assert e.value.code == -1
    with pytest.raises(BhrError) as e:  # the thin-disk entry point points to this one
        tracer.trace_bodies(v, bodies)
    assert e.value.code == -5 and "bhr_trace_bodies_volumetric" in str(e.value)
    flat = v.copy()
    flat.disk_thickness = 0.0
    with pytest.raises(BhrError) as e:
        tracer.trace_bodies_volumetric(flat, bodies, shade_params())
    assert e.value.code == -1
