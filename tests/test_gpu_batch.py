"""Batched ensembles: many independent grids, one launch per step.

Each instance keeps its own dt; results must equal the single-grid path on
the same instance (FP64: bit for bit, the same item code runs; FP32: to
FP32 rounding), and the oracle on a sample.
"""
import numpy as np
import pytest

import hydrofv_gb300 as H
from hydrofv_gb300.problems import four_quadrant_ensemble, random_problem_2d, shear_layer

pytestmark = pytest.mark.gpu


def single(p, precision=H.PRECISION_FP64):
    return H.run_2d(p.nx, p.ny, p.g, (p.x_min, p.x_max, p.y_min, p.y_max), p.gamma, p.W, p.U,
                    bc=p.bc, slope_limiter=p.slope_limiter, cfl=p.cfl, tf=p.tf,
                    max_steps=p.max_steps, options=H.default_options(precision=precision))


def mixed_batch(steps):
    """Uneven grids and boundaries; one integrator / limiter / CFL for the batch."""
    probs = [shear_layer(n, steps=steps) for n in (40, 130, 64)]
    for k, (nx, ny) in enumerate([(200, 37), (9, 140), (127, 126)]):
        probs.append(random_problem_2d(nx, ny, 30 + k, ("reflective", "transmissive", "none", "reflective"),
                                       "monotonized_central", steps, smooth=True))
    for p in probs:
        p.cfl = 0.6
    return probs


def test_batch_equals_single_grid_fp64(gpu_available):
    probs = mixed_batch(25)
    with H.Batch2D(probs) as b:
        st, ms = b.advance(25)
        outs = b.download()
    for p, (W, U), s in zip(probs, outs, st):
        r = single(p)
        assert r.code == 0, r.message
        assert s[0] == r.num_steps == 25
        assert s[1] == r.t and s[2] == r.dt          # per-instance dt, same bits
        assert np.array_equal(U, r.U, equal_nan=True)
        assert np.array_equal(W, r.W, equal_nan=True)


def test_batch_fp32_close_to_single_fp32(gpu_available):
    probs = mixed_batch(20)
    with H.Batch2D(probs, options=H.default_options(precision=H.PRECISION_FP32)) as b:
        b.advance(20)
        outs = b.download()
    for p, (W, U) in zip(probs, outs):
        r = single(p, H.PRECISION_FP32)
        g = p.g
        l1 = np.abs(U - r.U)[:, g:-g, g:-g].sum(axis=(1, 2)) / np.abs(r.U)[:, g:-g, g:-g].sum(axis=(1, 2))
        assert np.all(l1 <= 1e-5), l1


def test_batch_restart_and_split_advance(gpu_available):
    probs = four_quadrant_ensemble(count=10, steps=30, side_range=(40, 200))
    with H.Batch2D(probs) as b:
        b.advance(30)
        first = b.download()
        b.restart()
        b.advance(12)
        b.advance(18)
        second = b.download()
    for (W1, U1), (W2, U2) in zip(first, second):
        assert np.array_equal(U1, U2, equal_nan=True) and np.array_equal(W1, W2, equal_nan=True)


def test_batch_against_oracle_sample(gpu_available, oracle_mod):
    probs = four_quadrant_ensemble(count=8, steps=40, side_range=(32, 160))
    with H.Batch2D(probs) as b:
        b.advance(40)
        outs = b.download()
    orc = oracle_mod.load("oracle")
    for k in (0, 3, 7):
        ref = orc.run_2d(probs[k])
        assert ref.rc == 0
        l1 = oracle_mod.rel_l1(outs[k][1], ref.U, probs[k].g)
        assert np.all(l1 <= 1e-12), l1


def test_autotune_changes_schedule_not_results(gpu_available):
    """The autotuner only picks work-item shapes and grid sizes."""
    p = shear_layer(300, steps=12)
    ref = single(p)
    r = H.run_2d(p.nx, p.ny, p.g, (0, 1, 0, 1), p.gamma, p.W, p.U, bc=p.bc,
                 slope_limiter=p.slope_limiter, cfl=p.cfl, tf=p.tf, max_steps=p.max_steps,
                 options=H.default_options(autotune=1))
    assert r.code == 0, r.message
    assert np.array_equal(r.U, ref.U, equal_nan=True)
    probs = four_quadrant_ensemble(count=6, steps=10, side_range=(40, 300))
    outs = []
    for tune in (0, 1):
        with H.Batch2D(probs, options=H.default_options(autotune=tune)) as b:
            b.advance(10)
            outs.append(b.download())
    for (W0, U0), (W1, U1) in zip(*outs):
        assert np.array_equal(U0, U1, equal_nan=True)
