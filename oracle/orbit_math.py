"""Closed-form orbit pieces of the surrogate, restated in numpy FP64 -- TEST INFRASTRUCTURE ONLY.

These are the oracle's versions of blackholerender_gb300/csrc/surrogate_math.cuh. For a photon
in Schwarzschild (G = c = M = 1) with impact parameter b, u = 1/r obeys the first integral of
the Binet equation u'' + u = 3u^2 (the orbit shape of x'' = -3 h^2 x / r^5,
shaders/geodesic.glsl:3-5 and src/physics/Geodesic.h:4-6):

    (du/dphi)^2 = P(u) = 2u^3 - u^2 + 1/b^2 = 2 (u - u1)(u - u2)(u - u3)

With b > sqrt(27) the roots are real, u1 < 0 < u2 < u3, and u2 is the turning point of an
ingoing ray. The polar angle swept between u = a and the turning point is the elliptic
integral

    I(a) = int_a^u2 du / sqrt(P(u)) = sqrt(2) sqrt(u2 - a) R_F(X, Y, Z),
    X = (a - u1)(u3 - u2),  Y = (u2 - u1)(u3 - u2),  Z = (u3 - a)(u2 - u1)

(Carlson's symmetric form, B. C. Carlson, "Numerical computation of real or complex elliptic
integrals", Numer. Algorithms 10 (1995); DLMF 19.29.4 with homogeneity). R_F is evaluated by
the duplication theorem followed by its fifth-order Taylor series; the surrogate's baseline
uses a single duplication step and learns the remainder.
"""
from __future__ import annotations

import numpy as np

SQRT27 = 27.0 ** 0.5


def roots(beta):
    """Roots u1 < u2 < u3 of 2u^3 - u^2 + 1/b^2 for b = sqrt(27)(1 + beta), beta > 0.

    Written around the double root u = 1/3 of the critical orbit: with u = 1/3 + w,
    P = w^2 (1 + 2w) - D, D = 1/27 - 1/b^2 = beta (2 + beta) / (27 (1 + beta)^2), so the two
    roots near 1/3 are found relative to 1/3 without cancellation (Newton from +-sqrt(D)).
    Away from it (beta >= 0.1) Newton from -sqrt(D) can step past w = -1/3, where the slope
    vanishes, onto the wrong root; there the roots come from the trigonometric solution of the
    cubic with a = asin(sqrt(27) / b) / 3: u2 = 2/3 sin(a) sin(2 pi/3 - a), u3 = 2/3 cos(a + pi/6)
    cos(a - pi/6), u3 - u2 = sin(pi/3 - 2a) / sqrt(3).
    """
    beta = np.asarray(beta, dtype=np.float64)
    D = beta * (2.0 + beta) / (27.0 * (1.0 + beta) ** 2)
    sd = np.sqrt(D)
    wp, wm = sd.copy(), -sd.copy()
    for _ in range(40):  # w^2 (1 + 2w) = D
        wp = wp - (wp * wp * (1 + 2 * wp) - D) / (2 * wp + 6 * wp * wp)
        wm = wm - (wm * wm * (1 + 2 * wm) - D) / (2 * wm + 6 * wm * wm)
    u2 = 1.0 / 3.0 + wm
    u3 = 1.0 / 3.0 + wp
    d32 = wp - wm
    a = np.arcsin(np.minimum(1.0 / (1.0 + np.maximum(beta, 1e-300)), 1.0)) / 3.0
    far = beta >= 0.1
    u2 = np.where(far, 2.0 / 3.0 * np.sin(a) * np.sin(2.0 * np.pi / 3.0 - a), u2)
    u3 = np.where(far, 2.0 / 3.0 * np.cos(a + np.pi / 6.0) * np.cos(a - np.pi / 6.0), u3)
    d32 = np.where(far, np.sin(np.pi / 3.0 - 2.0 * a) / np.sqrt(3.0), d32)
    u1 = 0.5 - u2 - u3  # roots of 2u^3 - u^2 + c sum to 1/2
    return u1, u2, u3, d32


def rf(x, y, z, ndup=None, tol=1e-16):
    """Carlson R_F by duplication (ndup steps, or until converged) + the Taylor series."""
    x, y, z = (np.asarray(v, dtype=np.float64).copy() for v in (x, y, z))
    n = 0
    while True:
        A = (x + y + z) / 3.0
        dev = np.max(np.abs(np.stack([x, y, z]) - A) / A)
        if (ndup is not None and n >= ndup) or (ndup is None and dev < tol ** (1 / 6)):
            break
        sx, sy, sz = np.sqrt(x), np.sqrt(y), np.sqrt(z)
        lam = sx * sy + sy * sz + sz * sx
        x, y, z = (x + lam) / 4.0, (y + lam) / 4.0, (z + lam) / 4.0
        n += 1
    A = (x + y + z) / 3.0
    X, Y = 1.0 - x / A, 1.0 - y / A
    Z = -(X + Y)
    E2 = X * Y - Z * Z
    E3 = X * Y * Z
    return (1.0 - E2 / 10.0 + E3 / 14.0 + E2 * E2 / 24.0 - 3.0 * E2 * E3 / 44.0) / np.sqrt(A)


def sweep_to_turn(a, beta, ndup=None):
    """I(a): polar angle between u = a and the turning point u2."""
    u1, u2, u3, d32 = roots(beta)
    a = np.asarray(a, dtype=np.float64)
    X = (a - u1) * d32
    Y = (u2 - u1) * d32
    Z = (u3 - a) * (u2 - u1)
    return np.sqrt(2.0) * np.sqrt(np.maximum(u2 - a, 0.0)) * rf(X, Y, Z, ndup)


BLEND_LO, BLEND_HI = 0.002, 0.02


def base_blend(beta):
    """Weight of the two-step closed form in the surrogate's baseline (surrogate_math.cuh
    base_blend): 1 below beta = 0.002, 0 above 0.02, smoothstep between."""
    x = np.clip((BLEND_HI - np.asarray(beta, dtype=np.float64)) / (BLEND_HI - BLEND_LO), 0.0, 1.0)
    return x * x * (3.0 - 2.0 * x)


def base_sweep(a, beta):
    """The baseline the network corrects: I(a) with one duplication step, blended with two steps
    near the photon sphere."""
    w = base_blend(beta)
    i1 = sweep_to_turn(a, beta, ndup=1)
    return i1 + w * (sweep_to_turn(a, beta, ndup=2) - i1)


def phi_of_u(u, uc, beta, leg, ndup=None):
    """Polar angle from the camera (u = uc, ingoing) to u on leg 0 (ingoing) or 1 (outgoing)."""
    Ic = sweep_to_turn(uc, beta, ndup)
    Iu = sweep_to_turn(u, beta, ndup)
    return np.where(np.asarray(leg) == 0, Ic - Iu, Ic + Iu)


def b_transform(b, eps=1e-3):
    """Monotone transform of b / sqrt(27): t = sign(beta) ln(1 + |beta| / eps)."""
    beta = np.asarray(b, dtype=np.float64) / SQRT27 - 1.0
    return np.sign(beta) * np.log1p(np.abs(beta) / eps)


def cap_orbit(beta):
    """Captured orbit (b < sqrt(27), beta < 0): the real root u1 < 0 of 2u^3 - u^2 + 1/b^2, A with
    A^2 = (p - u1)^2 + q^2 for the complex pair p +- iq, k^2 = (A + p - u1) / (2A), and K(k).
    Restates orbit::cap_orbit of blackholerender_gb300/csrc/surrogate_math.cuh in FP64."""
    beta = float(beta)
    c = 1.0 / (27.0 * (1.0 + beta) ** 2)
    u = -np.cbrt(c / 2.0)
    for _ in range(60):
        u -= (2 * u ** 3 - u ** 2 + c) / (6 * u ** 2 - 2 * u)
    p = 0.5 * (0.5 - u)
    A = np.sqrt(-c / (2 * u) - 2 * p * u + u * u)
    k2 = (A + p - u) / (2 * A)
    return u, A, k2, float(rf(0.0, 1.0 - k2, 1.0)), c


def cap_angle(u, uc, beta):
    """Polar angle swept by a captured orbit from u = uc (camera) to u: F(theta(u), k) - F(theta(uc), k),
    divided by sqrt(2A), with cos(theta) = (A - w) / (A + w), w = u - u1 (Byrd & Friedman 239.00)."""
    u1, A, k2, K, _ = cap_orbit(beta)

    def F(x):
        w = np.asarray(x, dtype=np.float64) - u1
        ct = (A - w) / (A + w)
        st = 2.0 * np.sqrt(A * w) / (A + w)
        f0 = st * rf(ct * ct, 1.0 - k2 * st * st, np.ones_like(ct))
        return np.where(ct < 0.0, 2.0 * K - f0, f0)

    return (F(u) - F(uc)) / np.sqrt(2.0 * A)


def exit_u_tol(b, tol, u_esc_min, u2):
    """Exit u of the tolerance escape (SHADER and CPU rules) in the limit of small steps
    (surrogate_math.cuh exit_u_tol): the outgoing leg's first u below 1 / rEscMin where
    0.75 b'^3 u^4 < tol, b' = b / sqrt(1 + 2 b^2 u^3), and never before the turning point u2.
    Solved here by bisection on the monotone estimate, independently of the kernel's iteration."""
    b = np.asarray(b, dtype=np.float64)

    def est(u):
        return 0.75 * (b / np.sqrt(1.0 + 2.0 * b * b * u ** 3)) ** 3 * u ** 4

    lo = np.zeros_like(b)
    hi = np.full_like(b, 1.0)
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        below = est(mid) < tol
        lo = np.where(below, mid, lo)
        hi = np.where(below, hi, mid)
    return np.minimum(np.minimum(lo, u_esc_min), u2)


def far_field_dir(x, v, h2):
    """farFieldDirection (shaders/geodesic.glsl:43-53, src/physics/Geodesic.h:65-75) on arrays of
    vectors (last axis), normalised."""
    vlen = np.linalg.norm(v, axis=-1, keepdims=True)
    vh = v / vlen
    r = np.linalg.norm(x, axis=-1, keepdims=True)
    p = np.sum(x * vh, axis=-1, keepdims=True)
    bvec = x - p * vh
    s = np.clip(p / r, 0.0, 1.0)
    r3 = r ** 3
    h2 = np.asarray(h2, dtype=np.float64)[..., None]
    dv = -(h2 / vlen) * (vh / r3 + bvec * ((2.0 + s) / (r3 * r * (1.0 + s) ** 2)))
    o = v + dv
    return o / np.linalg.norm(o, axis=-1, keepdims=True)


def exit_geometry(beta, rc, ue, residual=0.0, sweep=None):
    """The escaping orbit's answer in its orbital plane (e1 = the camera direction, e2 = the
    tangential direction of the initial velocity), as a view's exit table holds it: (psi, phi0,
    Ic), psi the angle of the escape direction from e1, phi0 the angle from the camera to the exit
    at u = ue (the closed form plus the network's residual there), Ic the angle from the camera to
    the turning point. The exit velocity follows the energy integral of x'' = -3 h^2 x / r^5,
    |v|^2 = 1 - 2 h^2 / rc^3 + 2 h^2 u^3 with |v| = 1 at the camera and h^2 = b^2 / (1 + 2 b^2 / rc^3);
    then farFieldDirection there."""
    sweep = base_sweep if sweep is None else sweep
    beta = np.asarray(beta, dtype=np.float64)
    ue = np.broadcast_to(np.asarray(ue, dtype=np.float64), beta.shape)
    b = SQRT27 * (1.0 + beta)
    u1, u2, u3, _ = roots(beta)
    Ic = sweep(1.0 / rc, beta)
    phi0 = Ic + sweep(ue, beta) + residual
    re = 1.0 / ue
    c, s = np.cos(phi0), np.sin(phi0)
    xe = np.stack([re * c, re * s, np.zeros_like(c)], -1)
    sP = np.sqrt(np.maximum(2.0 * (ue - u1) * (u2 - ue) * (u3 - ue), 0.0))
    T = np.stack([sP * re * re * c - re * s, sP * re * re * s + re * c, np.zeros_like(c)], -1)
    h2 = b * b / (1.0 + 2.0 * b * b / rc ** 3)
    vmag = np.sqrt(1.0 - 2.0 * h2 / rc ** 3 + 2.0 * h2 * ue ** 3)
    T = T * (vmag / np.linalg.norm(T, axis=-1))[..., None]
    d = far_field_dir(xe, T, h2)
    gam = np.arctan2(c * d[..., 1] - s * d[..., 0], c * d[..., 0] + s * d[..., 1])
    return phi0 + gam, phi0, Ic
