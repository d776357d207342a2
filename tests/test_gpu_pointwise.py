"""Device builds of the exported pointwise numerics against the reference's
known answers (tests/golden/pointwise.npz, made by make_golden.py from the
compiled reference).

The step kernels call these functions (numerics.cuh) compiled for the GPU,
where division, square root and pow run as the integer-pipe forms of
fp64_int.cuh and pow_int.cuh.  The states cover vacuum generation, zero
densities, the two-rarefaction (TRRS, pow) and two-shock (TSRS) guesses, and
sampling of the exact solution on both sides of every wave.  Division and
square root are correctly rounded on both sides, so the only permitted
difference is pow: the device pow is correctly rounded while glibc's is off
by an ulp in ~0.1% of cases, which moves a TRRS guess, and through it a
flux, by a few ulp.  The exact solver iterates Newton on p* to a relative
tolerance of 1e-6, so an ulp in an iterate may end the iteration one step
earlier or later; its outputs are held to 1e-12.
"""
import os

import numpy as np
import pytest

import hydrofv_gb300 as H

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(GOLDEN, "pointwise.npz"))


def _compare(got, ref, rtol):
    """(fraction bit-identical, worst relative difference); NaNs must agree."""
    got, ref = np.atleast_2d(got), np.atleast_2d(ref)
    nan_g, nan_r = np.isnan(got), np.isnan(ref)
    assert np.array_equal(nan_g, nan_r), np.argwhere(nan_g != nan_r)[:5]
    same = (got.view(np.uint64) == ref.view(np.uint64)) | nan_g
    ok = ~nan_r
    err = np.zeros_like(got)
    err[ok] = np.abs(got[ok] - ref[ok]) / np.maximum(np.abs(ref[ok]), 1e-300)
    worst = float(err.max()) if err.size else 0.0
    assert worst <= rtol, (worst, np.unravel_index(np.argmax(err), err.shape))
    return float(same.all(axis=1).mean()), worst


def test_hllc_2d_device_against_reference(gpu_available, golden):
    g = golden
    F, rc = H.gpu_pointwise_eval("hllc_2d", g["gamma"], g["L"], g["R"])
    assert np.array_equal(rc == 0, g["hllc_rc"] == 0)
    good = rc == 0
    frac, worst = _compare(F[good], g["hllc"][good], 1e-14)
    assert frac >= 0.99, frac


def test_hllc_1d_device_against_reference(gpu_available, golden):
    g = golden
    m = len(g["speeds"])
    F, rc = H.gpu_pointwise_eval("hllc_1d", g["gamma"][:m], g["L"][:m], g["R"][:m])
    assert np.array_equal(rc == 0, g["hllc_1d_rc"] == 0)
    frac, worst = _compare(F, g["hllc_1d"], 1e-14)
    assert frac >= 0.99, frac


def test_guess_p_device_against_reference(gpu_available, golden):
    g = golden
    L, R, gam = g["L"], g["R"], g["gamma"]
    a = np.stack([np.sqrt(gam * L[:, 3] / np.maximum(L[:, 0], 1e-30)),
                  np.sqrt(gam * R[:, 3] / np.maximum(R[:, 0], 1e-30))], axis=1)
    p, rc = H.gpu_pointwise_eval("guess_p", gam, L, R, aux=a)
    frac, worst = _compare(p[:, None], g["guess_p"][:, None], 1e-14)
    assert frac >= 0.99, frac


@pytest.mark.parametrize("name,key", [("exact_flux_1d", "exact"), ("exact_1d", "exact_state")])
def test_exact_solver_device_against_reference(gpu_available, golden, name, key):
    g = golden
    m = len(g["speeds"])
    out, rc = H.gpu_pointwise_eval(name, g["gamma"][:m], g["L"][:m], g["R"][:m], aux=g["speeds"])
    assert np.array_equal(rc == 0, g[key + "_rc"] == 0)
    frac, worst = _compare(out, g[key], 1e-12)
    assert frac >= 0.95, frac


@pytest.mark.parametrize("name,key", [("exact_flux_1d", "exact"), ("exact_1d", "exact_state")])
def test_quad_exact_solver_is_the_single_lane_solver(gpu_available, golden, name, key):
    """The 1D kernel's four-lane exact solver (quad_exact.cuh) against the
    one-thread device build of exact_solve_1d on every golden state pair
    (vacuum generation, TRRS, TSRS, fans, shocks, both sides of every wave):
    the same bits, and the reference's answers within the exact tolerance."""
    g = golden
    m = len(g["speeds"])
    one, rc1 = H.gpu_pointwise_eval(name, g["gamma"][:m], g["L"][:m], g["R"][:m], aux=g["speeds"])
    four, rc4 = H.gpu_pointwise_eval(name + "_quad", g["gamma"][:m], g["L"][:m], g["R"][:m], aux=g["speeds"])
    assert np.array_equal(rc1, rc4)
    assert np.array_equal(one.view(np.uint64), four.view(np.uint64))
    assert np.array_equal(rc4 == 0, g[key + "_rc"] == 0)
    _compare(four, g[key], 1e-12)


def test_pointwise_rejects_unknown_op(gpu_available):
    lib = H.library()
    one = np.ones(4)
    out = np.zeros(4)
    rc = np.zeros(1, dtype=np.int32)
    import ctypes as C
    dp = C.POINTER(C.c_double)
    code = lib.hydro_gpu_pointwise_eval(0, 9, 1, one.ctypes.data_as(dp), 1e-6, one.ctypes.data_as(dp),
                                        one.ctypes.data_as(dp), one.ctypes.data_as(dp),
                                        out.ctypes.data_as(dp), rc.ctypes.data_as(C.POINTER(C.c_int)))
    assert code != 0
