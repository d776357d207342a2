"""Discrete adjoint, tangent-linear model and frozen-dt replay on the GPU.

The checks, per boundary set and limiter:
  * the replay and the tangent-linear model's primal reproduce the forward
    pass (production step kernel) bit for bit, and the segment
    recomputation reproduces every checkpoint and dt bit for bit;
  * dot-product test: <seed, TLM(dw0)> == <VJP(seed), dw0> (the hand-written
    reverse sweep is the transpose of the dual-number tangent model);
  * central finite differences of J = sum_{x > 0.5} rho^2 dx dy through the
    frozen-dt replay agree with <dJ/dW0, dw0> on directions whose replays
    took the forward pass's branches (equal branch signatures);
  * the gradient does not depend on the checkpoint interval.
"""
import math

import numpy as np
import pytest

import hydrofv_gb300 as h
from hydrofv_gb300.problems import (Problem2D, apply_bc_2d, mid_points, primitive_to_conserved_2d,
                                    shear_layer)

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _device(gpu_available):
    """Every test here needs the GPU: skip cleanly where none is visible."""
    return gpu_available


def smooth_problem(nx, ny, bc, limiter, seed=0, g=2, gamma=1.4):
    """Smooth periodic-friendly fields built from a few Fourier modes with
    irrational phases (no exact slope ties)."""
    rng = np.random.default_rng(seed)
    x = mid_points(0.0, 1.0, nx, g)
    y = mid_points(0.0, 1.0, ny, g)
    X, Y = np.meshgrid(x, y)
    W = np.zeros((4, ny + 2 * g, nx + 2 * g))
    base = [1.0, 0.2, -0.1, 1.0]
    amp = [0.2, 0.3, 0.3, 0.2]
    for f in range(4):
        W[f] = base[f]
        for _ in range(3):
            kx, ky = rng.integers(1, 3, size=2)
            ph = rng.uniform(0, 1, size=2) + 0.1234567
            W[f] += amp[f] / 3 * np.sin(2 * math.pi * (kx * X + ph[0])) * np.cos(2 * math.pi * (ky * Y + ph[1]))
    apply_bc_2d(W, g, nx, ny, bc)
    dx = 1.0 / (nx + 2 * g)
    dy = 1.0 / (ny + 2 * g)
    U = primitive_to_conserved_2d(W, gamma, dx * dy)
    return Problem2D(nx, ny, g, 0.0, 1.0, 0.0, 1.0, gamma, W, U, tuple(bc), "muscl_hancock_2d",
                     "riemann_solver_hllc", limiter, cfl=0.6, tf=1e300, max_steps=-1,
                     name=f"smooth_{nx}x{ny}")


def interior(p):
    m = np.zeros((p.ny + 2 * p.g, p.nx + 2 * p.g), dtype=bool)
    m[p.g:p.g + p.ny, p.g:p.g + p.nx] = True
    return m


def objective(p, W):
    """J = sum over interior cells with x > 0.5 of rho^2 dx dy, and dJ/dW."""
    x = mid_points(p.x_min, p.x_max, p.nx, p.g)
    mask = interior(p) & (x[None, :] > 0.5)
    dxdy = (1.0 / (p.nx + 2 * p.g)) * (1.0 / (p.ny + 2 * p.g))
    rho = W[0]
    J = math.fsum((rho[mask] ** 2).ravel()) * dxdy
    seed = np.zeros_like(W)
    seed[0][mask] = 2.0 * rho[mask] * dxdy
    return J, seed


def smooth_direction(p, rng, fields=(0, 3)):
    """A smooth random direction on the interior (relative to the field scale)."""
    x = mid_points(0.0, 1.0, p.nx, p.g)
    y = mid_points(0.0, 1.0, p.ny, p.g)
    X, Y = np.meshgrid(x, y)
    d = np.zeros((4,) + X.shape)
    for f in fields:
        for _ in range(3):
            kx, ky = rng.integers(1, 4, size=2)
            ph = rng.uniform(0, 1, size=2)
            d[f] += rng.normal() * np.sin(2 * math.pi * (kx * X + ph[0])) * np.sin(2 * math.pi * (ky * Y + ph[1]))
        d[f] *= np.abs(p.W[f]).max()
    d[:, ~interior(p)] = 0.0
    return d


def dot(a, b, p):
    m = interior(p)
    return math.fsum((a[:, m] * b[:, m]).ravel())


CASES = [
    (("periodic",) * 4, "monotonized_central"),
    (("reflective",) * 4, "minmod"),
    (("transmissive",) * 4, "van_leer"),
    (("reflective", "transmissive", "periodic", "periodic"), "monotonized_central"),
]


@pytest.mark.parametrize("bc,limiter", CASES, ids=["periodic-mc", "reflective-minmod",
                                                    "transmissive-vanleer", "mixed-mc"])
def test_replay_and_tangent_primal_match_forward(bc, limiter):
    p = smooth_problem(40, 36, bc, limiter, seed=1)
    with h.Adjoint2D(p, steps=25, checkpoint_every=6) as ad:
        WN = ad.forward()
        Wr, sig = ad.replay(p.W)
        assert np.array_equal(Wr, WN)
        assert sig.all()
        Wt, _ = ad.tangent(np.zeros_like(p.W))
        assert np.array_equal(Wt, WN)
        dt = ad.dt()
        assert (dt > 0).all() and len(dt) == 25


@pytest.mark.parametrize("bc,limiter", CASES, ids=["periodic-mc", "reflective-minmod",
                                                    "transmissive-vanleer", "mixed-mc"])
def test_dot_product_tangent_vs_adjoint(bc, limiter):
    p = smooth_problem(40, 36, bc, limiter, seed=2)
    rng = np.random.default_rng(3)
    with h.Adjoint2D(p, steps=25, checkpoint_every=6) as ad:
        ad.forward()
        for _ in range(3):
            seed = rng.normal(size=p.W.shape)
            dw0 = rng.normal(size=p.W.shape) * np.array([1.0, 0.3, 0.3, 1.0])[:, None, None]
            grad = ad.backward(seed)
            st = ad.stats()
            assert st["recompute_mismatches"] == 0
            _, dwN = ad.tangent(dw0)
            lhs = dot(seed, dwN, p)
            rhs = dot(grad, dw0, p)
            assert abs(lhs - rhs) <= 1e-11 * max(abs(lhs), 1e-300), (lhs, rhs)
            assert not grad[:, ~interior(p)].any()


@pytest.mark.parametrize("bc,limiter", CASES, ids=["periodic-mc", "reflective-minmod",
                                                    "transmissive-vanleer", "mixed-mc"])
def test_tape_and_recomputation_give_the_same_gradient(bc, limiter):
    """The reverse sweep reading the recomputation's tape and the one
    re-evaluating the reconstruction and the guesses agree bit for bit."""
    p = smooth_problem(40, 36, bc, limiter, seed=7)
    rng = np.random.default_rng(10)
    with h.Adjoint2D(p, steps=25, checkpoint_every=6) as ad:
        ad.forward()
        seed = rng.normal(size=p.W.shape)
        g_tape = ad.backward(seed)
        ad.set_tape(False)
        g_plain = ad.backward(seed)
        ad.set_tape(True)
        g_again = ad.backward(seed)
    assert np.array_equal(g_tape, g_plain) and np.array_equal(g_tape, g_again)


def test_gradient_independent_of_checkpoint_interval():
    p = smooth_problem(32, 32, ("periodic",) * 4, "monotonized_central", seed=4)
    grads = []
    for K in (1, 5, 20):
        with h.Adjoint2D(p, steps=20, checkpoint_every=K) as ad:
            WN = ad.forward()
            _, seed = objective(p, WN)
            grads.append(ad.backward(seed))
            assert ad.stats()["checkpoints"] == -(-20 // K)
    assert np.array_equal(grads[0], grads[1]) and np.array_equal(grads[0], grads[2])


@pytest.mark.parametrize("bc,limiter", CASES, ids=["periodic-mc", "reflective-minmod",
                                                    "transmissive-vanleer", "mixed-mc"])
def test_gradient_matches_central_differences(bc, limiter):
    """FD of the branch-frozen replay (the map the adjoint differentiates)
    on every direction; FD of the free replay on the directions whose
    replays kept the forward pass's branches."""
    p = smooth_problem(48, 48, bc, limiter, seed=5)
    rng = np.random.default_rng(6)
    with h.Adjoint2D(p, steps=30, checkpoint_every=8) as ad:
        WN = ad.forward()
        assert np.array_equal(ad.replay_frozen(p.W), WN)
        _, base_sig = ad.replay(p.W)
        _, seed = objective(p, WN)
        grad = ad.backward(seed)
        for _ in range(6):
            d = smooth_direction(p, rng)
            an = dot(grad, d, p)
            eps = 1e-6
            fd = (objective(p, ad.replay_frozen(p.W + eps * d))[0]
                  - objective(p, ad.replay_frozen(p.W - eps * d))[0]) / (2 * eps)
            assert abs(fd - an) <= 1e-6 * abs(an), (fd, an)
            eps = 1e-7
            Wp, sp = ad.replay(p.W + eps * d)
            Wm, sm = ad.replay(p.W - eps * d)
            if np.array_equal(sp, base_sig) and np.array_equal(sm, base_sig):
                fd = (objective(p, Wp)[0] - objective(p, Wm)[0]) / (2 * eps)
                assert abs(fd - an) <= 1e-6 * abs(an), (fd, an)


def test_shear_layer_dot_product_small():
    """The shear layer of the adjoint benchmark (MC, periodic, gamma 5/3) at 128^2."""
    p = shear_layer(128, steps=40)
    rng = np.random.default_rng(8)
    with h.Adjoint2D(p, steps=40, checkpoint_every=10) as ad:
        WN = ad.forward()
        _, seed = objective(p, WN)
        grad = ad.backward(seed)
        assert ad.stats()["recompute_mismatches"] == 0
        d = np.zeros_like(p.W)
        d[0] = rng.normal(size=d[0].shape)
        d[3] = rng.normal(size=d[3].shape)
        d[:, ~interior(p)] = 0.0
        _, dwN = ad.tangent(d)
        lhs = dot(seed, dwN, p)
        rhs = dot(grad, d, p)
        assert abs(lhs - rhs) <= 1e-11 * abs(lhs)


def test_shear_layer_frozen_central_differences():
    """Gradient w.r.t. initial rho and p of the shear layer (MC, periodic):
    central differences of the branch-frozen map, random directions."""
    p = shear_layer(128, steps=40)
    rng = np.random.default_rng(9)
    with h.Adjoint2D(p, steps=40, checkpoint_every=10) as ad:
        WN = ad.forward()
        _, seed = objective(p, WN)
        grad = ad.backward(seed)
        eps = 1e-6
        for _ in range(4):
            d = np.zeros_like(p.W)
            d[0] = rng.normal(size=d[0].shape) * np.abs(p.W[0])
            d[3] = rng.normal(size=d[3].shape) * np.abs(p.W[3])
            d[:, ~interior(p)] = 0.0
            an = dot(grad, d, p)
            fd = (objective(p, ad.replay_frozen(p.W + eps * d))[0]
                  - objective(p, ad.replay_frozen(p.W - eps * d))[0]) / (2 * eps)
            assert abs(fd - an) <= 1e-6 * abs(an), (fd, an)


def test_noisy_shear_layer_frozen_central_differences():
    """The shear layer with seeded relative noise 1e-3 on rho and p, so no
    limiter of those fields sits at its a = b = 0 kink: central differences
    of the branch-frozen map agree with the gradient to 1e-6, and so do the
    free replay's differences on any direction whose perturbed replays kept
    every branch of the forward pass.  (Directions that cross a Riemann
    regime switch -- the PVRS / two-rarefaction / two-shock choice of the
    star-pressure guess, which changes the HLLC wave speeds discontinuously
    -- cannot agree at any eps: the free map jumps there.)"""
    p = shear_layer(128, steps=40, rho_p_noise=1e-3)
    rng = np.random.default_rng(10)
    with h.Adjoint2D(p, steps=40, checkpoint_every=10) as ad:
        WN = ad.forward()
        _, seed = objective(p, WN)
        grad = ad.backward(seed)
        _, base_sig = ad.replay(p.W)
        eps = 1e-6
        for _ in range(4):
            d = np.zeros_like(p.W)
            d[0] = rng.normal(size=d[0].shape) * np.abs(p.W[0])
            d[3] = rng.normal(size=d[3].shape) * np.abs(p.W[3])
            d[:, ~interior(p)] = 0.0
            an = dot(grad, d, p)
            fd = (objective(p, ad.replay_frozen(p.W + eps * d))[0]
                  - objective(p, ad.replay_frozen(p.W - eps * d))[0]) / (2 * eps)
            assert abs(fd - an) <= 1e-6 * abs(an), (fd, an)
            Wp, sp = ad.replay(p.W + eps * d)
            Wm, sm = ad.replay(p.W - eps * d)
            if np.array_equal(sp, base_sig) and np.array_equal(sm, base_sig):
                fd = (objective(p, Wp)[0] - objective(p, Wm)[0]) / (2 * eps)
                assert abs(fd - an) <= 1e-6 * abs(an), (fd, an)
