"""The surrogate's checkers without a GPU: the closed-form orbit restatement (oracle/orbit_math.py)
against independent numerics, the FP64 network reference (oracle/mlp_ref.py) against finite
differences, and the committed checkpoint read on the host."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT / "oracle"))

import mlp_ref  # noqa: E402
import orbit_math as om  # noqa: E402

from blackholerender_gb300.surrogate import DEFAULT_CHECKPOINT, read_checkpoint  # noqa: E402


@pytest.mark.parametrize("beta", [1e-3, 0.02, 0.3, 2.0, 10.0])
def test_roots_solve_the_cubic(beta):
    b = om.SQRT27 * (1.0 + beta)
    u1, u2, u3, d32 = om.roots(beta)
    ref = np.sort(np.roots([2.0, -1.0, 0.0, 1.0 / (b * b)]).real)
    assert np.allclose([u1, u2, u3], ref, rtol=1e-10, atol=1e-13)
    assert abs(d32 - (u3 - u2)) < 1e-12
    assert u1 < 0 < u2 < u3


def test_carlson_rf_against_scipy():
    sp = pytest.importorskip("scipy.special")
    rng = np.random.default_rng(1)
    x, y, z = rng.uniform(1e-3, 5.0, size=(3, 200))
    assert np.allclose(om.rf(x, y, z), sp.elliprf(x, y, z), rtol=1e-13)
    # truncated after one duplication step: the surrogate's baseline, accurate to ~1e-3 at worst here
    assert np.max(np.abs(om.rf(x, y, z, ndup=1) / sp.elliprf(x, y, z) - 1.0)) < 3e-2


@pytest.mark.parametrize("beta", [0.01, 0.2, 3.0])
def test_sweep_equals_quadrature(beta):
    integ = pytest.importorskip("scipy.integrate")
    b = om.SQRT27 * (1.0 + beta)
    u1, u2, u3, _ = om.roots(beta)
    for a in (0.0, 0.3 * u2, 0.9 * u2):
        # u = u2 - s^2 removes the turning-point singularity: du / sqrt(P) = 2 ds / sqrt(2 (u - u1)(u3 - u))
        def f(s):
            return 2.0 / np.sqrt(2.0 * (u2 - s * s - u1) * (u3 - u2 + s * s))

        val, _ = integ.quad(f, 0.0, np.sqrt(u2 - a), epsabs=1e-13, epsrel=1e-12, limit=200)
        assert abs(float(om.sweep_to_turn(a, beta)) - val) < 1e-9 * max(1.0, val), (a, val)
    # the whole deflection: 2 I(0) - pi approaches 4/b for large b (weak field)
    if beta > 1:
        defl = 2.0 * float(om.sweep_to_turn(0.0, beta)) - np.pi
        assert abs(defl - 4.0 / b) / (4.0 / b) < 0.2


def test_mlp_reference_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = rng.normal(scale=0.3, size=mlp_ref.NPARAMS)
    x = rng.uniform(-1, 1, size=(24, 3))
    y = rng.normal(size=24)
    lab = rng.integers(0, 3, size=24)
    samples = np.concatenate([x, y[:, None]], axis=1)
    w_c = 0.7

    def loss(q):
        s, _ = mlp_ref.loss_and_grad(q, samples, lab, w_c, quantize=False)
        n = len(samples)
        return s[0] / n + w_c * s[1] / n

    _, g = mlp_ref.loss_and_grad(p, samples, lab, w_c, quantize=False)
    for k in rng.choice(mlp_ref.NPARAMS, 60, replace=False):
        e = np.zeros_like(p)
        e[k] = 1e-6
        fd = (loss(p + e) - loss(p - e)) / 2e-6
        assert abs(fd - g[k]) <= 1e-6 + 1e-5 * abs(g[k]), (k, fd, g[k])


def test_committed_checkpoint_reads_on_the_host():
    ck = read_checkpoint(DEFAULT_CHECKPOINT)
    assert len(ck["params"]) == mlp_ref.NPARAMS and np.all(np.isfinite(ck["params"]))
    nm = ck["norm"]
    assert (nm["rc_lo"], nm["rc_hi"], nm["b_max"]) == (6.0, 200.0, 60.0)
    assert abs(nm["band"] - 2e-3) < 1e-9 and ck["adam_step"] > 0
    # the trained network's corrections stay small where it was trained (y is scaled by y_scale)
    rng = np.random.default_rng(0)
    q = np.stack([rng.uniform(-1, 1, 256), rng.uniform(0.2, 1.0, 256), rng.uniform(-1, 1, 256)], axis=1)
    out, _ = mlp_ref.forward(ck["params"].astype(np.float64), q)
    assert np.all(np.isfinite(out)) and np.max(np.abs(out[:, 0])) * nm["y_scale"] < 0.2


@pytest.mark.parametrize("beta", [-0.9, -0.3, -0.05, -2e-3, -4e-4])
def test_captured_orbit_angle_equals_quadrature(beta):
    integ = pytest.importorskip("scipy.integrate")
    u1, A, k2, K, c = om.cap_orbit(beta)
    assert abs(2 * u1 ** 3 - u1 ** 2 + c) < 1e-15 and u1 < 0
    uc = 1.0 / 30.0
    for u in (0.05, 0.17, 0.3, 1.0 / 2.0001):
        val, _ = integ.quad(lambda t: 1.0 / np.sqrt(2 * t ** 3 - t ** 2 + c), uc, u, epsabs=1e-13, epsrel=1e-12,
                            limit=500)
        assert abs(float(om.cap_angle(u, uc, beta)) - val) < 1e-10 * max(1.0, val), (u, val)


def test_blended_baseline_is_closer_near_the_photon_sphere():
    """Near b = sqrt(27) the one-step closed form misses by up to ~1e-1 rad; the blended baseline
    (two steps there) stays within ~1e-4 of the exact integral, and equals one step far away."""
    for beta, tol in ((5e-4, 2e-4), (2e-3, 2e-4), (0.1, 2e-2), (1.0, 5e-3)):
        exact = float(om.sweep_to_turn(0.0, beta))
        assert abs(float(om.base_sweep(0.0, beta)) - exact) < tol, beta
    assert om.base_blend(0.05) == 0.0 and om.base_blend(1e-3) == 1.0
    assert abs(float(om.sweep_to_turn(0.0, 5e-4, ndup=1)) - float(om.sweep_to_turn(0.0, 5e-4))) > 1e-2


def _table_setup():
    ck = read_checkpoint(DEFAULT_CHECKPOINT)
    nm = ck["norm"]
    P = ck["params"].astype(np.float64)

    def x2_of(beta):
        return np.sign(beta) * np.log1p(np.abs(beta) / nm["t_eps"]) * nm["t_scale"]

    def beta_of(x2):
        t = x2 / nm["t_scale"]
        return np.sign(t) * nm["t_eps"] * np.expm1(np.abs(t))

    def x1_of(rc):
        return 2 * (np.log(rc) - np.log(nm["rc_lo"])) / (np.log(nm["rc_hi"]) - np.log(nm["rc_lo"])) - 1

    band = nm["band"] / np.sqrt(27.0)
    esc = (x2_of(band), x2_of(nm["b_max"] / np.sqrt(27.0) - 1))
    cap = (x2_of(-1.0), x2_of(-band))
    return nm, P, x1_of, beta_of, esc, cap


@pytest.mark.parametrize("rcam", [15.0, 60.0])
def test_exit_table_resolution(rcam):
    """A captured ray reads its capture logit from its view's exit table: 2,048 points of x2 over
    the captured half, linear interpolation. With the FP64 network (no BF16 rounding) no capture
    logit changes sign against direct evaluation."""
    nm, P, x1_of, beta_of, esc, cap = _table_setup()
    x1 = x1_of(rcam)
    rng = np.random.default_rng(3)
    for side, (lo, hi) in (("captured", cap),):
        def f(x2):
            beta = beta_of(x2)
            sig = np.ones_like(beta)
            if side == "escaping":
                u1, u2, u3, d32 = om.roots(beta)
                sig = np.sqrt(np.maximum((u2 - nm["ue"]) / u2, 0.0))
            return mlp_ref.forward(P, np.stack([np.full_like(x2, x1), x2, sig], 1), quantize=False)[0]
        n = 2048
        g = np.linspace(lo, hi, n)
        T = f(g)
        xs = rng.uniform(lo, hi, 4000)
        D = f(xs)
        u = (xs - lo) / (hi - lo) * (n - 1)
        i = np.clip(np.floor(u).astype(int), 0, n - 2)
        t = (u - i)[:, None]
        I = T[i] + t * (T[i + 1] - T[i])
        assert np.all(np.sign(I[:, 1]) == np.sign(D[:, 1]))


@pytest.mark.parametrize("rcam", [15.0, 60.0])
def test_crossing_table_resolution(rcam):
    """The crossing queries of escaping orbits come from a per-view 256 x 64 table over (x2,
    sigma), bilinear: with the FP64 network within 2e-6 rad of direct evaluation at the 99th
    percentile and 5e-6 at most (measured 1.1e-6 and 2.6e-6), against the 1e-4 rad tolerance and the
    network's own ~3e-6 BF16 noise."""
    nm, P, x1_of, beta_of, esc, cap = _table_setup()
    x1 = x1_of(rcam)
    nx, ns = 256, 64
    gx, gs = np.linspace(esc[0], esc[1], nx), np.linspace(-1.0, 1.0, ns)
    X, S = np.meshgrid(gx, gs, indexing="ij")
    T = mlp_ref.forward(P, np.stack([np.full(X.size, x1), X.ravel(), S.ravel()], 1), quantize=False)[0][:, 0]
    T = T.reshape(nx, ns)
    rng = np.random.default_rng(4)
    xs, ss = rng.uniform(esc[0], esc[1], 4000), rng.uniform(-1, 1, 4000)
    D = mlp_ref.forward(P, np.stack([np.full(xs.size, x1), xs, ss], 1), quantize=False)[0][:, 0]
    u = (xs - esc[0]) / (esc[1] - esc[0]) * (nx - 1)
    v = (ss + 1) / 2 * (ns - 1)
    i, j = np.clip(np.floor(u).astype(int), 0, nx - 2), np.clip(np.floor(v).astype(int), 0, ns - 2)
    a, b = u - i, v - j
    I = ((1 - a) * (1 - b) * T[i, j] + a * (1 - b) * T[i + 1, j] + (1 - a) * b * T[i, j + 1]
         + a * b * T[i + 1, j + 1])
    err = np.abs(I - D) * nm["y_scale"]
    assert np.percentile(err, 99) < 2e-6 and err.max() < 5e-6, (np.percentile(err, 99), err.max())


def _cubic_table_lookup(T, lo, h, xs):
    """A view's cubic exit-table entries as the pass reads them: entry j holds points j .. j + 3,
    j = clamp(floor(u) - 1, 0, n - 4), Lagrange weights at u - j."""
    n = len(T)
    u = (xs - lo) / h
    m = np.clip(np.floor(u).astype(int), 0, n - 2)
    j = np.clip(m - 1, 0, n - 4)
    t = u - j
    a, b, c, d = t, t - 1, t - 2, t - 3
    L = np.stack([-b * c * d / 6, a * c * d / 2, -a * b * d / 2, a * b * c / 6], 1)
    return np.sum(L * np.stack([T[j], T[j + 1], T[j + 2], T[j + 3]], 1), 1)


@pytest.mark.parametrize("rcam,rule", [(15.0, "config"), (60.0, "config"), (15.0, "shader"), (45.0, "cpu")])
def test_escape_table_resolution(rcam, rule):
    """The surrogate pass reads an escaping ray's escape direction (psi), exit angle (phi0) and
    angle to the turning point (Ic) from its view's exit table: 2,048 points of x2 over the
    escaping half, cubic interpolation, the tolerance escape's two branches (exit at rEscMin, or
    where the estimate reaches esc_tol) tabulated apart, rays within ten spacings of the camera's
    tangential ray left to the plain march. With the FP64 network the table stays within 1e-6 rad
    of direct evaluation (1e-7 at the 99th percentile; measured 6e-7 and 3e-8), under the CONFIG rule's fixed exit and the
    SHADER and CPU rules' tolerance escape: far below the 1e-4 rad bar and the network's own noise."""
    nm, P, x1_of, beta_of, esc, cap = _table_setup()
    x1 = x1_of(rcam)
    tol, umin = {"config": (None, None), "shader": (0.01, 1 / 25.0), "cpu": (1e-4, 1 / 30.0)}[rule]

    def ue_branch(beta, branch):
        u2 = om.roots(beta)[1]
        if rule == "config":
            return np.full_like(beta, nm["ue"])
        if branch == 0:
            return np.minimum(umin, u2)
        return om.exit_u_tol(np.sqrt(27.0) * (1 + beta), tol, 1.0, u2)

    def f(x2, ue):
        beta = beta_of(x2)
        u2 = om.roots(beta)[1]
        sig = np.sqrt(np.maximum((u2 - ue) / u2, 0.0))
        y = mlp_ref.forward(P, np.stack([np.full_like(x2, x1), x2, sig], 1), quantize=False)[0][:, 0]
        return om.exit_geometry(beta, rcam, ue, y * nm["y_scale"])

    n = 2048
    lo, hi = esc
    h = (hi - lo) / (n - 1)
    g = lo + h * np.arange(n)
    tabs = [f(g, ue_branch(beta_of(g), r)) for r in (0, 1)]
    b_t = rcam / np.sqrt(1 - 2 / rcam)  # the camera's tangential ray
    x2_lim = np.log1p((b_t / np.sqrt(27.0) - 1) / nm["t_eps"]) * nm["t_scale"] - 10 * h
    xs = np.random.default_rng(5).uniform(lo, min(hi, x2_lim), 3000)
    bx = beta_of(xs)
    if rule == "config":
        ue = ue_branch(bx, 0)
        br = np.zeros(len(xs), dtype=int)
    else:
        ue = om.exit_u_tol(np.sqrt(27.0) * (1 + bx), tol, umin, om.roots(bx)[1])
        br = (ue < np.minimum(umin, om.roots(bx)[1])).astype(int)  # the exit moved out to u_tol
    direct = f(xs, ue)
    for q, name in enumerate(("psi", "phi0", "Ic")):
        got = np.where(br == 1, _cubic_table_lookup(tabs[1][q], lo, h, xs), _cubic_table_lookup(tabs[0][q], lo, h, xs))
        err = np.abs(got - direct[q])
        # worst next to the tangential ray's square-root end (6e-7 at ten spacings)
        assert err.max() < 1e-6 and np.percentile(err, 99) < 1e-7, (name, err.max(), np.percentile(err, 99))


def test_own_arctangent_within_its_bound():
    """The surrogate's per-ray angles use an own arctangent (surrogate_math.cuh atan_unit, a
    degree-7 polynomial in a^2 fitted to atan on [0, 1]): its coefficients are read from the header
    and its float32 evaluation, Horner as the kernel does, stays within 1e-7 rad of numpy's arctan
    over [0, 1], and refitting by the documented method gives the same coefficients."""
    import re
    from pathlib import Path

    text = (Path(__file__).resolve().parent.parent / "blackholerender_gb300" / "csrc" / "surrogate_math.cuh").read_text()
    body = text[text.index("float atan_unit(float a)"):]
    body = body[:body.index("return")]
    c = [float(v) for v in re.findall(r"(-?\d+\.\d+(?:e-?\d+)?)f", body)][::-1]  # Horner runs c7 .. c0
    assert len(c) == 8
    x = np.linspace(0, 1, 400001).astype(np.float32)
    s = (x * x).astype(np.float32)
    q = np.float32(c[7])
    for k in range(6, -1, -1):
        q = (q * s + np.float32(c[k])).astype(np.float32)
    r = (x + (x * s).astype(np.float32) * q).astype(np.float32)
    assert np.abs(r.astype(np.float64) - np.arctan(x.astype(np.float64))).max() < 1e-7
    # the fit: weighted least squares on 4000 Chebyshev nodes of [0, 1]
    n = 4000
    a = 0.5 * (1 - np.cos(np.pi * (np.arange(n) + 0.5) / n))
    ss = a * a
    w = a * ss
    A = np.vander(ss, 8, increasing=True)
    fit, *_ = np.linalg.lstsq(A * w[:, None], (np.arctan(a) - a) / (a * ss) * w, rcond=None)
    assert np.allclose(fit, c, rtol=1e-5, atol=1e-7)


@pytest.mark.parametrize("variant", ["learned", "closed_form"])
def test_crossing_inversion_converges_in_three_newton_steps(variant):
    """The pass inverts the orbit at each disk-plane crossing by three Newton steps in
    s = sqrt(u2 - u) on its variant's closed form (surrogate_math.cuh invert_sweep_v, first guess
    from the slope at the turning point). Restated here in FP64 over crossings of the disk's radii
    (0.97 r_in to 1.03 r_out for the [6, 20] disk) and beta from 4e-4 to 10.5: every crossing's u
    is within 2e-6 (relative) after three steps; the second step alone is not enough."""
    rng = np.random.default_rng(0)
    beta = np.exp(rng.uniform(np.log(4e-4), np.log(10.5), 20000))
    r = rng.uniform(6.0 * 0.97, 20.0 * 1.03, 20000)
    u1, u2, u3, d32 = om.roots(beta)
    u = np.minimum(1.0 / r, u2 * (1.0 - 1e-6))
    sweep = (lambda a: om.base_sweep(a, beta)) if variant == "learned" else (lambda a: om.sweep_to_turn(a, beta, ndup=3))
    target = sweep(u)
    x0 = (u2 - u1) * d32
    slope0 = np.sqrt(2.0) * om.rf(x0, x0, x0, ndup=1)
    smax = np.sqrt(u2)
    s = np.clip(target / slope0, 0.0, smax)
    errs = []
    for _ in range(3):
        uu = u2 - s * s
        s = np.clip(s - (sweep(uu) - target) * 0.5 * np.sqrt(2.0 * (uu - u1) * (u3 - uu)), 0.0, smax)
        errs.append(np.max(np.abs((u2 - s * s) - u) / u))
    assert errs[2] < 2e-6 and errs[1] > 1e-4, errs
