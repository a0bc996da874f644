"""Synthetic camera views of the benchmark configurations (the reference publishes no scene
files; every pose is drawn from a seeded std::mt19937_64 stream, restated here).

C1  256x144, FOV 60, r=30, inclination 85 deg, Low preset (200 steps), CONFIG termination
C2  1920x1080, FOV 60, High preset (450 steps), 16 poses from seed 0:
    r ~ U[15,60], inclination ~ U[60,90] deg, azimuth ~ U[0, 2 pi), draw order r, i, a
C3  3840x2160, FOV 40, Ultra preset (700 steps), r=20, inclination 88 deg, mixed precision
C4  64 views from seed 1, per view in draw order: pixel count log-uniform in
    [320*180, 3840*2160] at 16:9 (W = round(sqrt(N*16/9)), H = round(W*9/16)), FOV ~ U[30,90],
    r ~ log-U[6.5,200], inclination ~ U[0,90] deg, azimuth ~ U[0,2 pi), budget from
    {200,300,450,700} (preset Low..Ultra)
All use the thin disk r in [6,20] (H/r 0.035), escape at r>1000 and capture at r<2.0001.
A uniform draw is libstdc++'s: u = x * 2^-64 of one 64-bit engine output x (kept below 1).
Bodies: body_gallery places a fixed set of planets and stars in front of a view's camera.
"""
from __future__ import annotations

import math

from . import TERM_CONFIG, Body, View, make_view

_MASK = (1 << 64) - 1


class MT19937_64:
    """std::mt19937_64 (Matsumoto & Nishimura 2000, 64-bit parameters)."""

    def __init__(self, seed: int = 5489):
        self.mt = [0] * 312
        self.mt[0] = seed & _MASK
        for i in range(1, 312):
            self.mt[i] = (6364136223846793005 * (self.mt[i - 1] ^ (self.mt[i - 1] >> 62)) + i) & _MASK
        self.idx = 312

    def _twist(self):
        mt = self.mt
        for i in range(312):
            x = (mt[i] & 0xFFFFFFFF80000000) | (mt[(i + 1) % 312] & 0x7FFFFFFF)
            xa = x >> 1
            if x & 1:
                xa ^= 0xB5026F5AA96619E9
            mt[i] = mt[(i + 156) % 312] ^ xa
        self.idx = 0

    def __call__(self) -> int:
        if self.idx >= 312:
            self._twist()
        y = self.mt[self.idx]
        self.idx += 1
        y ^= (y >> 29) & 0x5555555555555555
        y ^= (y << 17) & 0x71D67FFFEDA60000
        y ^= (y << 37) & 0xFFF7EEE000000000
        y ^= y >> 43
        return y & _MASK

    def uniform(self, lo: float, hi: float) -> float:
        """std::uniform_real_distribution<double>(lo, hi) as libstdc++ draws it: one 64-bit
        output scaled by 2^-64 (generate_canonical, kept below 1), then u (hi - lo) + lo."""
        u = float(self()) / 18446744073709551616.0
        if u >= 1.0:
            u = math.nextafter(1.0, 0.0)
        return u * (hi - lo) + lo


PRESET_BY_BUDGET = {200: 0, 300: 1, 450: 2, 700: 3}


def c1_view(term_mode: int = TERM_CONFIG) -> View:
    return make_view(term_mode, width=256, height=144, fov_deg=60.0, preset=0,
                     pose=(30.0, math.radians(85.0), 0.0))


def c2_poses(seed: int = 0, n: int = 16):
    g = MT19937_64(seed)
    out = []
    for _ in range(n):
        r = g.uniform(15.0, 60.0)
        inc = g.uniform(math.radians(60.0), math.radians(90.0))
        az = g.uniform(0.0, 2.0 * math.pi)
        out.append((r, inc, az))
    return out


def c2_views(term_mode: int = TERM_CONFIG, width: int = 1920, height: int = 1080, seed: int = 0, n: int = 16):
    return [make_view(term_mode, width=width, height=height, fov_deg=60.0, preset=2, pose=p)
            for p in c2_poses(seed, n)]


def c3_view(term_mode: int = TERM_CONFIG, width: int = 3840, height: int = 2160) -> View:
    return make_view(term_mode, width=width, height=height, fov_deg=40.0, preset=3,
                     pose=(20.0, math.radians(88.0), 0.0))


def c4_specs(seed: int = 1, n: int = 64, scale: float = 1.0):
    """Per view of C4, in draw order: (width, height, fov_deg, preset, (r, inclination, azimuth)).
    `scale` < 1 shrinks every view's pixel count by that factor (test sizes)."""
    g = MT19937_64(seed)
    lo, hi = math.log(320 * 180), math.log(3840 * 2160)
    out = []
    for _ in range(n):
        npx = math.exp(g.uniform(lo, hi)) * scale
        w = max(16, round(math.sqrt(npx * 16.0 / 9.0)))
        h = max(9, round(w * 9.0 / 16.0))
        fov = g.uniform(30.0, 90.0)
        r = math.exp(g.uniform(math.log(6.5), math.log(200.0)))
        inc = g.uniform(0.0, math.radians(90.0))
        az = g.uniform(0.0, 2.0 * math.pi)
        budget = (200, 300, 450, 700)[min(3, int(g.uniform(0.0, 4.0)))]
        out.append((w, h, fov, PRESET_BY_BUDGET[budget], (r, inc, az)))
    return out


def c4_views(term_mode: int = TERM_CONFIG, seed: int = 1, n: int = 64, scale: float = 1.0):
    """`scale` < 1 shrinks every view's pixel count by that factor (test sizes)."""
    return [make_view(term_mode, width=w, height=h, fov_deg=fov, preset=preset, pose=pose)
            for w, h, fov, preset, pose in c4_specs(seed, n, scale)]


def body_gallery(view: View, n: int = 12, distance: float = 9.0, radius: float = 0.7) -> list[Body]:
    """n bodies on a grid 2.2 M apart, `distance` M in front of the view's camera: the nine
    planet looks in turn, a star and an exploding photosphere among them, the last one ringed
    and translucent. Light comes from behind the camera, up and to the right."""
    cam = [float(c) for c in view.cam_pos]
    B = [float(c) for c in view.cam_basis]
    right, up, back = B[0:3], B[3:6], B[6:9]
    lx = [back[k] + 0.4 * right[k] + 0.5 * up[k] for k in range(3)]
    ln = math.sqrt(sum(c * c for c in lx))
    out = []
    for k in range(n):
        gx, gy = k % 4, k // 4
        pos = [cam[c] - distance * back[c] + (gx - 1.5) * 2.2 * right[c] + (gy - 1.0) * 2.2 * up[c] for c in range(3)]
        b = Body()
        star = k % 12 in (9, 10)
        b.pos_radius[:] = (*pos, radius)
        b.rel_pos[:] = (*(pos[c] - cam[c] for c in range(3)), 1.0 if star else 0.0)
        b.look[:] = (float(k % 9), float(100 + k), 0.5 if k % 9 in (2, 4, 7) else 0.0, 0.3 * k)
        b.tint[:] = (1.0, 1.0, 1.0, 0.0)
        b.light[:] = (*(c / ln for c in lx), 1.5)
        b.light_color[:] = (1.0, 0.95, 0.9, 9000.0 if k % 12 == 10 else 5772.0)
        b.axis[:] = (0.0, 1.0, 0.0, 0.0)
        b.ring[:] = (0.0, 0.0, 0.0, 1.0)
        if k % 12 == 10:  # an exploding photosphere: turbulence, plumes per radius, its clock
            b.tint[3] = 0.8
            b.look[2] = 3.0
            b.ring[2] = 1.7
        if k % 12 == 11:  # rings, translucent
            b.ring[:] = (0.9 * radius / 0.7, 1.4 * radius / 0.7, 0.0, 0.6)
            b.axis[:3] = (0.2, 0.9, 0.3)
        out.append(b)
    return out
