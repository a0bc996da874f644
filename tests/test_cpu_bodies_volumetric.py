"""Bodies with the volumetric disk in the CPU restatement (blackhole.frag with BHS_BODIES 1 and
DISK_VOLUMETRIC: :101-121,146-150,169-190,217-250): no bodies = the volumetric march bit for bit,
a body behind the disk keeps the light gathered in front of it, a dense disk turns rays opaque
before they reach the body, the FP32 restatement against the FP64 one, and the shading."""
from __future__ import annotations

import math

import numpy as np
import pytest

import oracle_lib as O
from blackholerender_gb300 import (DISK_VOLUMETRIC, SQRT27, STATUS_BODY, STATUS_OPAQUE, TERM_CONFIG, make_view,
                                   shade_params)
from test_cpu_bodies import body


@pytest.fixture(scope="module")
def tex():
    return O.noise_bake(7), O.blackbody_lut()


def scene(width=128, height=72, term=TERM_CONFIG):
    """A camera 30 M out, 30 degrees above the disk, and a planet of radius 2 below the disk
    plane at radius 8 on the camera's side: every ray to it crosses the disk's slab first."""
    v = make_view(term, width=width, height=height, preset=0, pose=(30.0, math.radians(60.0), 0.4),
                  disk_mode=DISK_VOLUMETRIC)
    cam = np.array(v.cam_pos, dtype=np.float64)
    hor = np.array([cam[0], 0.0, cam[2]])
    hor /= np.linalg.norm(hor)
    return v, [body(8.0 * hor + np.array([0.0, -4.0, 0.0]), 2.0, cam)]


@pytest.mark.parametrize("density", [1.0, 4.0])
def test_no_bodies_is_the_volumetric_march(tex, density):
    v, _ = scene()
    p = shade_params(disk_density=density)
    h, bh, rgbt = O.trace_bodies_volumetric(v, [], p, *tex)
    h0, rgbt0 = O.trace_volumetric(v, p, *tex)
    assert np.array_equal(h.view(np.uint8), h0.view(np.uint8))
    assert np.array_equal(rgbt, rgbt0.reshape(-1, 4))
    assert np.all(bh["body"] == -1) and np.all(bh["near_mask"] == 0)


def test_body_behind_the_disk_keeps_the_light_in_front(tex):
    v, bodies = scene()
    h, bh, rgbt = O.trace_bodies_volumetric(v, bodies, shade_params(), *tex)
    hit = h["status"] == STATUS_BODY
    assert hit.sum() > 50 and np.all(bh["body"][hit] == 0)
    # every ray to the body crossed the slab: absorbed in part, lit by the disk
    assert np.all(rgbt[hit, 3] < 0.99) and np.all(rgbt[hit, 3] >= 0.004)
    assert np.all(rgbt[hit, :3].sum(-1) > 0)
    # an empty disk gathers nothing and stops the same rays on the body
    h0, bh0, rgbt0 = O.trace_bodies_volumetric(v, bodies, shade_params(disk_density=0.0), *tex)
    assert np.array_equal(h0["status"] == STATUS_BODY, hit)
    assert np.all(rgbt0[:, 3] == 1.0) and np.all(rgbt0[:, :3] == 0.0)


def test_a_dense_disk_hides_the_body(tex):
    v, bodies = scene()
    h1, _, _ = O.trace_bodies_volumetric(v, bodies, shade_params(), *tex)
    h, bh, rgbt = O.trace_bodies_volumetric(v, bodies, shade_params(disk_density=40.0), *tex)
    op = h["status"] == STATUS_OPAQUE
    hidden = (h1["status"] == STATUS_BODY) & op
    assert hidden.sum() > 10  # rays that reached the body through the light disk turn opaque in the dense one
    assert np.all(bh["body"][op] == -1) and np.all(rgbt[op, 3] < 0.004)


def test_fp32_restatement_against_fp64(tex):
    v, bodies = scene()
    p = shade_params(disk_density=4.0)
    r64, b64, c64 = O.trace_bodies_volumetric(v, bodies, p, *tex, fp64=True)
    r32, b32, c32 = O.trace_bodies_volumetric(v, bodies, p, *tex, fp64=False)
    T = c64[:, 3]
    amb = (np.abs(r64["b"] - SQRT27) < 1e-2) | ((T > 0.002) & (T < 0.008))
    cls = ((r32["status"] != r64["status"]) | (b32["body"] != b64["body"])) & ~amb
    assert cls.mean() < 2e-3
    same = (r32["status"] == r64["status"]) & ~amb
    e = (np.abs(c32 - c64) / (np.abs(c64) + 1e-3))[same]
    assert np.percentile(e, 99) < 2e-3


def test_sampled_pixels_equal_the_whole_view(tex):
    v, bodies = scene(64, 36)
    p = shade_params(disk_density=2.0)
    h, bh, rgbt = O.trace_bodies_volumetric(v, bodies, p, *tex, fp64=False)
    idx = np.random.default_rng(3).choice(v.width * v.height, 300, replace=False)
    hs, bs, cs = O.trace_bodies_volumetric(v, bodies, p, *tex, fp64=False, idx=idx)
    assert np.array_equal(hs.view(np.uint8), h[idx].view(np.uint8))
    assert np.array_equal(bs.view(np.uint8), bh[idx].view(np.uint8))
    assert np.array_equal(cs, rgbt[idx])


def test_shading_adds_the_body_behind_the_disk(tex):
    v, bodies = scene()
    p = shade_params(time=12.0)
    h, bh, rgbt = O.trace_bodies_volumetric(v, bodies, p, *tex)
    img = O.shade_bodies_volumetric(v, h, bh, bodies, rgbt, p, *tex).reshape(-1, 4)
    assert np.all(np.isfinite(img))
    hit = h["status"] == STATUS_BODY
    # the disk's light in front is kept and the lit planet adds to it; no sky behind the body
    assert np.all(img[hit, :3] >= rgbt[hit, :3] - 1e-6)
    assert np.mean(img[hit, :3].sum(-1) > rgbt[hit, :3].sum(-1) + 1e-4) > 0.5
    assert np.all(img[hit, 3] == 0.0)
    # without bodies the shading is the volumetric disk's own
    h0, bh0, rgbt0 = O.trace_bodies_volumetric(v, [], p, *tex)
    a = O.shade_bodies_volumetric(v, h0, bh0, [], rgbt0, p, *tex)
    b = O.shade_volumetric(v, h0, rgbt0.reshape(v.height, v.width, 4), p, *tex)
    assert np.array_equal(a, b)
