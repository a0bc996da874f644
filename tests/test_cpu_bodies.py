"""The body-aware march in the CPU restatement (blackhole.frag:101-121,146-150,184-190,236-250):
raySphere's known answers, a body straight ahead settled by the near-field test, a body behind
the hole found through the lensed chords, and no bodies = the plain march bit for bit."""
from __future__ import annotations

import math

import numpy as np

import oracle_lib as O
from blackholerender_gb300 import (DISK_NONE, DISK_THIN, STATUS_BODY, STATUS_CAPTURED, STATUS_ESCAPED, TERM_CONFIG, Body,
                                   make_view)


def body(pos, radius, cam, kind=0.0, ring=(0.0, 0.0, 0.0, 1.0)):
    b = Body()
    b.pos_radius[:] = (*pos, radius)
    b.rel_pos[:] = (*(np.asarray(pos, dtype=np.float64) - np.asarray(cam, dtype=np.float64)), kind)
    b.look[:] = (0.0, 7.0, 0.0, 0.0)
    b.tint[:] = (1.0, 1.0, 1.0, 0.0)
    b.light[:] = (0.0, 1.0, 0.0, 1.0)
    b.light_color[:] = (1.0, 1.0, 1.0, 5772.0)
    b.axis[:] = (0.0, 1.0, 0.0, 0.0)
    b.ring[:] = ring
    return b


def _view(**kw):
    base = dict(width=96, height=54, preset=0, pose=(30.0, math.radians(80.0), 0.4), disk_mode=DISK_THIN)
    base.update(kw)
    return make_view(TERM_CONFIG, **base)


def test_no_bodies_is_the_plain_march():
    v = _view()
    h, bh = O.trace_bodies(v, [])
    ref = O.trace_view(v, fp64=True)
    assert np.array_equal(h.view(np.uint8), ref.view(np.uint8))
    assert np.all(bh["body"] == -1) and np.all(bh["near_idx"] == -1) and np.all(bh["near_mask"] == 0)


def test_body_straight_ahead_is_settled_by_the_near_field_test():
    v = _view()
    cam = np.array(v.cam_pos, dtype=np.float64)
    ahead = cam * (1.0 - 6.0 / np.linalg.norm(cam))  # 6 M from the camera, towards the hole
    b = body(ahead, 0.8, cam)
    h, bh = O.trace_bodies(v, [b])
    hit = h["status"] == STATUS_BODY
    assert hit.sum() > 20
    # settled by the straight ray: the near mask holds it, the near-field distance is 6 - 0.8 at the centre
    assert np.all(bh["near_mask"][hit] == 1) and np.all(bh["near_idx"][hit] == 0) and np.all(bh["body"][hit] == 0)
    c = (v.height // 2) * v.width + v.width // 2
    assert hit[c] and abs(bh["near_t"][c] - 5.2) < 0.05
    # the image disc of the body: its angular radius asin(0.8 / 6) seen through the pinhole
    rad_px = math.tan(math.asin(0.8 / 6.0)) / v.tan_half_fov * v.height / 2
    assert abs(hit.sum() - math.pi * rad_px ** 2) < 0.15 * math.pi * rad_px ** 2


def test_body_behind_the_hole_through_the_lensed_chords():
    v = _view(width=160, height=90)
    cam = np.array(v.cam_pos, dtype=np.float64)
    behind = -cam / np.linalg.norm(cam) * 40.0  # opposite side of the hole, 40 M out
    b = body(behind, 3.0, cam)
    h, bh = O.trace_bodies(v, [b])
    hit = h["status"] == STATUS_BODY
    assert hit.sum() > 10
    assert np.all(bh["near_mask"][hit] == 0) and np.all(bh["body"][hit] == 0)
    # chord hits: the hit point lies on the sphere
    p = bh["ro"][hit] + bh["rd"][hit] * bh["t"][hit][:, None]
    assert np.max(np.abs(np.linalg.norm(p - behind, axis=1) - 3.0)) < 1e-3
    assert np.all(np.abs(np.linalg.norm(bh["rd"][hit], axis=1) - 1.0) < 1e-6)
    # without the body those rays escape or are captured; the others are unchanged
    h0, _ = O.trace_bodies(v, [])
    assert np.all(np.isin(h0["status"][hit], [STATUS_ESCAPED, STATUS_CAPTURED, 3]))


def test_fp32_restatement_against_fp64():
    v = _view(width=128, height=72)
    cam = np.array(v.cam_pos, dtype=np.float64)
    bodies = [body(cam * (1.0 - 6.0 / np.linalg.norm(cam)) + np.array([0.5, 0.3, 0.0]), 0.6, cam),
              body(-cam / np.linalg.norm(cam) * 40.0, 3.0, cam), body(np.array([25.0, 2.0, -10.0]), 1.5, cam)]
    h64, b64 = O.trace_bodies(v, bodies, fp64=True)
    h32, b32 = O.trace_bodies(v, bodies, fp64=False)
    same = (h64["status"] == h32["status"]) & (b64["body"] == b32["body"])
    print(f"\nFP32 vs FP64: status and body agree on {same.mean():.5f} of {len(same)} rays, "
          f"{int((h64['status'] == STATUS_BODY).sum())} body hits")
    assert same.mean() > 0.998


# ---------------------------------------------------------------- shading of bodies


def _shade(v, bodies, **pk):
    from blackholerender_gb300 import shade_params

    h, bh = O.trace_bodies(v, bodies, fp64=False)
    p = shade_params(**pk)
    img = O.shade_bodies(v, h, bh, bodies, p, O.noise_bake(7), O.blackbody_lut())
    return h, bh, img


def _planet_ahead(v, look, radius=0.8, dist=6.0, light=(0.0, 1.0, 0.0), **kw):
    cam = np.array(v.cam_pos, dtype=np.float64)
    b = body(cam * (1.0 - dist / np.linalg.norm(cam)), radius, cam, **kw)
    b.look[0] = float(look)
    L = np.asarray(light, dtype=np.float64)
    b.light[:3] = L / np.linalg.norm(L)
    return b


def test_planet_lit_from_the_camera_side_and_dark_from_behind():
    v = _view(width=64, height=36, pose=(30.0, math.radians(20.0), 0.4), disk_mode=DISK_THIN)
    cam = np.array(v.cam_pos, dtype=np.float64)
    toward_cam = cam / np.linalg.norm(cam)
    _, _, lit = _shade(v, [_planet_ahead(v, 0, light=toward_cam)])
    h, bh, dark = _shade(v, [_planet_ahead(v, 0, light=-toward_cam)])
    on = h["status"] == STATUS_BODY
    lum_lit = lit.reshape(-1, 4)[on, :3].sum(1)
    lum_dark = dark.reshape(-1, 4)[on, :3].sum(1)
    assert on.sum() > 20 and np.all(np.isfinite(lit)) and np.all(lum_lit > 0)
    # lit side: wrap light up to albedo x irradiance; night side: the 1.5% ambient term only
    assert np.median(lum_lit) > 20 * np.median(lum_dark)
    # an opaque body hides the sky behind it: no sky-cube weight on its pixels
    assert np.all(lit.reshape(-1, 4)[on, 3] == 0.0)


def test_transparent_body_lets_the_sky_through():
    v = _view(width=64, height=36, pose=(30.0, math.radians(20.0), 0.4), disk_mode=DISK_THIN)
    b = _planet_ahead(v, 0, ring=(0.0, 0.0, 0.0, 0.5))  # opacity 0.5
    h, bh, img = _shade(v, [b])
    on = h["status"] == STATUS_BODY
    # the ray goes on straight from the body: half the sky-cube weight is left
    a = img.reshape(-1, 4)[on, 3]
    assert on.sum() > 20 and np.allclose(a, 0.5, atol=1e-6)


def test_star_halo_and_photosphere():
    v = _view(width=96, height=54, pose=(30.0, math.radians(20.0), 0.4), disk_mode=DISK_THIN)
    b = _planet_ahead(v, 0, radius=0.5, kind=1.0)
    b.light[3] = 3.0
    h, bh, img = _shade(v, [b])
    _, _, sky = _shade(v, [])
    on = h["status"] == STATUS_BODY
    lum = img[..., :3].sum(-1).reshape(-1)
    assert on.sum() > 20 and lum[on].min() > 0.5
    lum = lum - sky[..., :3].sum(-1).reshape(-1)  # the halo alone, off the disc
    # the glow outside the disc falls off with distance from the limb
    c = np.array([v.width / 2.0, v.height / 2.0])
    jj, ii = np.divmod(np.arange(lum.size), v.width)
    rr = np.hypot(ii + 0.5 - c[0], jj + 0.5 - c[1])
    rad = rr[on].max()
    ring1 = (~on) & (rr > rad + 1) & (rr < rad + 3)
    ring2 = (~on) & (rr > rad + 6) & (rr < rad + 9)
    assert lum[ring1].mean() > 1.5 * lum[ring2].mean() > 0.0


def test_every_look_shades_finite_and_distinct():
    v = _view(width=48, height=28, pose=(30.0, math.radians(20.0), 0.4), disk_mode=DISK_NONE)
    cam = np.array(v.cam_pos, dtype=np.float64)
    toward_cam = cam / np.linalg.norm(cam)
    means = []
    for look in range(9):
        b = _planet_ahead(v, look, light=toward_cam + np.array([0.3, 0.5, 0.0]))
        b.look[2] = 0.5 if look in (2, 4, 7) else 0.0  # atmospheres for the airy looks
        h, _, img = _shade(v, [b], time=12.0)
        on = h["status"] == STATUS_BODY
        px = img.reshape(-1, 4)[on, :3]
        assert on.sum() > 20 and np.all(np.isfinite(px)) and np.all(px >= 0.0)
        means.append(px.mean(0))
    means = np.array(means)
    # lava glows red; the ocean and the cold giant are bluer than the desert
    assert means[8, 0] > means[8, 2]
    assert means[2, 2] / means[2, 0] > means[1, 2] / means[1, 0]
    assert means[6, 2] / means[6, 0] > means[5, 2] / means[5, 0]
    assert len({tuple(np.round(m, 5)) for m in means}) == 9


def test_ring_in_front_of_the_sky():
    v = _view(width=96, height=54, pose=(30.0, math.radians(20.0), 0.4), disk_mode=DISK_NONE)
    b = _planet_ahead(v, 0, radius=0.4, ring=(0.6, 1.2, 0.0, 1.0))
    cam = np.array(v.cam_pos, dtype=np.float64)
    ax = cam / np.linalg.norm(cam)  # ring plane facing the camera: an annulus on screen
    b.axis[:3] = ax
    h, _, img = _shade(v, [b])
    _, _, bare = _shade(v, [_planet_ahead(v, 0, radius=0.4)])
    changed = np.any(np.abs(img - bare) > 1e-6, axis=-1).reshape(-1) & (h["status"] != STATUS_BODY)
    # the annulus between 0.6 and 1.2 M at 6 M: ring light, less sky weight. Only escaped rays
    # take the straight stretches (blackhole.frag:283-291): the part of the ring in front of the
    # hole's shadow is not drawn, as in the reference
    assert changed.sum() > 20
    assert np.all(img.reshape(-1, 4)[changed, 3] <= bare.reshape(-1, 4)[changed, 3] + 1e-6)


def test_sampled_pixels_equal_the_whole_view():
    """The restatement's sampled-pixel entry marches exactly the pixels the whole-view entry does."""
    from blackholerender_gb300 import workloads
    v = make_view(TERM_CONFIG, width=48, height=27, preset=2, pose=(30.0, math.radians(80.0), 0.4))
    bodies = workloads.body_gallery(v)
    h, bh = O.trace_bodies(v, bodies)
    idx = np.array([0, 11, 500, 1295, 648, 649])
    hs, bs = O.trace_bodies_pixels(v, bodies, idx)
    assert hs.tobytes() == h[idx].tobytes() and bs.tobytes() == bh[idx].tobytes()
