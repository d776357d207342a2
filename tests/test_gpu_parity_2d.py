"""GPU parity of the 2D MUSCL-Hancock + HLLC step against the CPU oracle.

The FP64 drop-in must agree with the reference algorithm to <= 1e-12
relative L1 per conserved field (interior cells) after the stated number of
steps; the tests also report the maximum absolute difference and check the
ghost layers, the status (num_steps, t, dt) and the full padded W.
"""
import numpy as np
import pytest

import hydrofv_gb300 as H

pytestmark = pytest.mark.gpu

REL_L1_TOL = 1e-12


def run_gpu(p, **kw):
    return H.run_2d(p.nx, p.ny, p.g, (p.x_min, p.x_max, p.y_min, p.y_max), p.gamma, p.W, p.U,
                    bc=p.bc, integrator=p.integrator, riemann_solver=p.riemann_solver,
                    slope_limiter=p.slope_limiter, cfl=p.cfl, tf=p.tf, max_steps=p.max_steps, **kw)


def assert_parity(p, gpu, ref, tol=REL_L1_TOL):
    import oracle as O
    assert gpu.code == 0, gpu.message
    assert ref.rc == 0, ref.message
    assert gpu.num_steps == ref.num_steps
    assert abs(gpu.t - ref.t) <= 1e-13 * max(1.0, abs(ref.t))
    assert abs(gpu.dt - ref.dt) <= 1e-12 * abs(ref.dt)
    l1 = O.rel_l1(gpu.U, ref.U, p.g)
    assert np.all(l1 <= tol), f"relative L1 per field {l1}"
    l1w = O.rel_l1(gpu.W, ref.W, p.g)
    assert np.all(l1w <= tol), f"relative L1 of W {l1w}"
    # every padded cell (ghost layers included, corners NaN-aware)
    both_nan = np.isnan(gpu.U) & np.isnan(ref.U)
    assert np.allclose(gpu.U[~both_nan], ref.U[~both_nan], rtol=1e-9, atol=1e-13)
    both_nan = np.isnan(gpu.W) & np.isnan(ref.W)
    assert np.allclose(gpu.W[~both_nan], ref.W[~both_nan], rtol=1e-9, atol=1e-13)
    return l1


@pytest.mark.parametrize("limiter", ["minmod", "van_leer", "monotonized_central"])
def test_shear_layer_small(gpu_available, oracle_mod, limiter):
    O = oracle_mod
    p = O.shear_layer(64, steps=40, limiter=limiter)
    ref = O.load("oracle").run_2d(p)
    gpu = run_gpu(p)
    assert_parity(p, gpu, ref)


@pytest.mark.parametrize("bc", [("none",) * 4, ("reflective",) * 4, ("transmissive",) * 4,
                                ("reflective", "transmissive", "periodic", "periodic"),
                                ("transmissive", "none", "reflective", "transmissive")])
@pytest.mark.parametrize("shape", [(19, 13), (130, 7), (3, 260)])
def test_boundaries_and_ragged_shapes(gpu_available, oracle_mod, bc, shape):
    O = oracle_mod
    nx, ny = shape
    p = O.random_problem_2d(nx, ny, 11, bc, "monotonized_central", 12, smooth=True)
    ref = O.load("oracle").run_2d(p)
    gpu = run_gpu(p)
    assert_parity(p, gpu, ref)


def test_point_blast_van_leer(gpu_available, oracle_mod):
    O = oracle_mod
    p = O.point_blast(96, steps=60)
    ref = O.load("oracle").run_2d(p)
    gpu = run_gpu(p)
    assert_parity(p, gpu, ref)


def test_run_to_tf(gpu_available, oracle_mod):
    """No step limit: the loop stops on t >= tf with the last dt clipped."""
    O = oracle_mod
    p = O.four_quadrant(40, np.random.default_rng(3), steps=-1)
    p.max_steps = -1
    p.tf = 0.05
    ref = O.load("oracle").run_2d(p)
    gpu = run_gpu(p)
    assert ref.t == pytest.approx(0.05)
    assert_parity(p, gpu, ref)
