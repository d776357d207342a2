"""Pointwise derivative pieces of the adjoint, host builds (no GPU).

The tangent-linear form runs the forward numerics templates on dual numbers;
the reverse form is hand-written.  For every regime of the HLLC flux and
every limiter / sweep direction of the cell reconstruction, the reverse form
must be the exact transpose of the tangent form (dot-product identity
<J dx, y> = <dx, J^T y>), and the tangent form must agree with central
finite differences where the finite difference does not straddle a kink.
"""
import numpy as np
import pytest

import hydrofv_gb300 as h

GAMMA = 1.4
TOL = 1e-6

# (left, right) states (rho, u_normal, u_tangential, p) and the expected
# regime: PVRS 1, two-rarefaction 2, two-shock 3, vacuum 0 (code & 0x100).
HLLC_CASES = {
    "pvrs_right_star": ([1.0, 0.1, 0.2, 1.0], [1.1, 0.05, -0.1, 1.2], 1),
    "pvrs_left_star": ([1.2, 0.3, 0.2, 1.3], [1.0, 0.25, -0.1, 1.1], 1),
    "two_rarefaction": ([1.0, -0.5, 0.3, 1.0], [1.0, 0.6, -0.2, 1.0], 2),
    "two_shock": ([1.0, 2.0, 0.1, 1.0], [1.3, -1.5, 0.3, 1.1], 3),
    "supersonic_right": ([1.0, 5.0, 0.1, 1.0], [0.8, 4.0, 0.1, 0.9], None),
    "supersonic_left": ([1.0, -5.0, 0.1, 1.0], [0.8, -4.0, 0.1, 0.9], None),
    "strong_shock": ([1.0, 0.0, 0.1, 1000.0], [1.0, 0.0, 0.3, 0.01], None),
    "vacuum_fan": ([1.0, -1.5, 0.1, 1.0], [1.0, 10.0, 0.3, 1.0], 0),
}


@pytest.mark.parametrize("name", sorted(HLLC_CASES))
def test_hllc_reverse_is_transpose_of_tangent(name):
    L, R, regime = (np.array(x) if isinstance(x, list) else x for x in HLLC_CASES[name])
    rng = np.random.default_rng(sum(name.encode()))
    _, _, _, code = h.ad_hllc_vjp(GAMMA, TOL, L, R, np.ones(4))
    if regime == 0:
        assert code & 0x100
    elif regime is not None:
        assert not code & 0x100 and (code & 3) == regime
    for _ in range(16):
        dL, dR, Fb = rng.normal(size=(3, 4))
        F, dF, rc = h.ad_hllc_jvp(GAMMA, TOL, L, R, dL, dR)
        Lb, Rb, rc2, _ = h.ad_hllc_vjp(GAMMA, TOL, L, R, Fb)
        assert rc == 0 and rc2 == 0
        lhs = dF @ Fb
        rhs = dL @ Lb + dR @ Rb
        assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), np.abs(dF).max() * np.abs(Fb).max())


@pytest.mark.parametrize("name", sorted(HLLC_CASES))
def test_hllc_tangent_matches_finite_differences(name):
    L, R, _ = (np.array(x) if isinstance(x, list) else x for x in HLLC_CASES[name])
    rng = np.random.default_rng(7)
    eps = 1e-6
    for _ in range(8):
        dL, dR = rng.normal(size=(2, 4))
        _, dF, _ = h.ad_hllc_jvp(GAMMA, TOL, L, R, dL, dR)
        Fp, _, _ = h.ad_hllc_jvp(GAMMA, TOL, L + eps * dL, R + eps * dR, dL, dR)
        Fm, _, _ = h.ad_hllc_jvp(GAMMA, TOL, L - eps * dL, R - eps * dR, dL, dR)
        fd = (Fp - Fm) / (2 * eps)
        assert np.abs(fd - dF).max() <= 1e-6 * np.abs(dF).max()


@pytest.mark.parametrize("limiter", [1, 2, 3], ids=["minmod", "van_leer", "mc"])
@pytest.mark.parametrize("direction", [0, 1], ids=["x", "y"])
def test_recon_reverse_is_transpose_of_tangent(limiter, direction):
    rng = np.random.default_rng(100 * limiter + direction)
    base = np.array([1.0, 0.1, 0.2, 1.0])
    for _ in range(200):
        wm, w0, wp = base + 0.1 * rng.normal(size=(3, 4))
        dwm, dw0, dwp, lob, hib = rng.normal(size=(5, 4))
        lo, hi, dlo, dhi = h.ad_recon_jvp(limiter, direction, GAMMA, 0.3, wm, w0, wp, dwm, dw0, dwp)
        wmb, w0b, wpb = h.ad_recon_vjp(limiter, direction, GAMMA, 0.3, wm, w0, wp, lob, hib)
        lhs = dlo @ lob + dhi @ hib
        rhs = dwm @ wmb + dw0 @ w0b + dwp @ wpb
        assert abs(lhs - rhs) <= 1e-12 * max(1.0, abs(lhs))


@pytest.mark.parametrize("limiter", [1, 2, 3], ids=["minmod", "van_leer", "mc"])
@pytest.mark.parametrize("direction", [0, 1], ids=["x", "y"])
def test_recon_tangent_matches_finite_differences(limiter, direction):
    rng = np.random.default_rng(200 + 10 * limiter + direction)
    base = np.array([1.0, 0.1, 0.2, 1.0])
    eps = 1e-7
    for _ in range(100):
        wm, w0, wp = base + 0.1 * rng.normal(size=(3, 4))
        dwm, dw0, dwp = rng.normal(size=(3, 4))
        _, _, dlo, dhi = h.ad_recon_jvp(limiter, direction, GAMMA, 0.3, wm, w0, wp, dwm, dw0, dwp)
        lp, hp, _, _ = h.ad_recon_jvp(limiter, direction, GAMMA, 0.3, wm + eps * dwm, w0 + eps * dw0,
                                      wp + eps * dwp, dwm, dw0, dwp)
        lm, hm, _, _ = h.ad_recon_jvp(limiter, direction, GAMMA, 0.3, wm - eps * dwm, w0 - eps * dw0,
                                      wp - eps * dwp, dwm, dw0, dwp)
        fd = np.concatenate([lp - lm, hp - hm]) / (2 * eps)
        an = np.concatenate([dlo, dhi])
        assert np.abs(fd - an).max() <= 1e-6 * np.abs(an).max()


def test_recon_primal_is_forward_reconstruction():
    """The tangent form's values are the forward reconstruction: a flat
    state reconstructs to itself with zero slopes."""
    w = np.array([1.0, 0.3, -0.2, 2.0])
    lo, hi, dlo, dhi = h.ad_recon_jvp(3, 0, GAMMA, 0.3, w, w, w, np.zeros(4), np.zeros(4), np.zeros(4))
    assert np.array_equal(lo, w) and np.array_equal(hi, w)
    assert not dlo.any() and not dhi.any()


@pytest.mark.parametrize("name", sorted(HLLC_CASES))
def test_hllc_forced_with_own_code_is_the_flux(name):
    L, R, _ = (np.array(x) if isinstance(x, list) else x for x in HLLC_CASES[name])
    _, _, _, code = h.ad_hllc_vjp(GAMMA, TOL, L, R, np.ones(4))
    F, _, _ = h.ad_hllc_jvp(GAMMA, TOL, L, R, np.zeros(4), np.zeros(4))
    Ff = h.ad_hllc_forced(GAMMA, TOL, L, R, code)
    assert np.array_equal(F, Ff, equal_nan=True)


@pytest.mark.parametrize("limiter", [1, 2, 3], ids=["minmod", "van_leer", "mc"])
@pytest.mark.parametrize("direction", [0, 1], ids=["x", "y"])
def test_recon_forced_with_own_code_is_the_reconstruction(limiter, direction):
    rng = np.random.default_rng(300 + 10 * limiter + direction)
    base = np.array([1.0, 0.1, 0.2, 1.0])
    for _ in range(200):
        wm, w0, wp = base + 0.1 * rng.normal(size=(3, 4))
        lo, hi, _, _ = h.ad_recon_jvp(limiter, direction, GAMMA, 0.3, wm, w0, wp, *np.zeros((3, 4)))
        _, _, code = h.ad_recon_forced(limiter, direction, GAMMA, 0.3, wm, w0, wp, 0)
        lf, hf, _ = h.ad_recon_forced(limiter, direction, GAMMA, 0.3, wm, w0, wp, code)
        assert np.array_equal(lo, lf) and np.array_equal(hi, hf)
