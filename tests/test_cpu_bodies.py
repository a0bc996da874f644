"""The body-aware march in the CPU restatement (blackhole.frag:101-121,146-150,184-190,236-250):
raySphere's known answers, a body straight ahead settled by the near-field test, a body behind
the hole found through the lensed chords, and no bodies = the plain march bit for bit."""
from __future__ import annotations

import math

import numpy as np

import oracle_lib as O
from blackholerender_gb300 import (DISK_THIN, STATUS_BODY, STATUS_CAPTURED, STATUS_ESCAPED, TERM_CONFIG, Body,
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
