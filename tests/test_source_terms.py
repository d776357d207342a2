"""The exported source-term functions on the host (CPU only).

add_geometry_source_term (src/source_term.c:45-183) and
add_gravity_source_term_2d (src/source_term.c:185-259) are part of the
reference's numerics API; a program may call them between its own steps.
The library's host builds (csrc/gpu/source_term_host.cu, compiled from the
same templates as the step kernels) are called through the C ABI on
non-trivial states -- the Sedov blasts on cylindrical and spherical grids
and the Rayleigh-Taylor problem after some steps (the reference's outputs,
tests/golden/) -- and compared bit for bit with the oracle and, where it was
built, with the reference itself.
"""
import ctypes as C
import os

import numpy as np
import pytest

import hydrofv_gb300 as H

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def bits_equal(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint64), np.ascontiguousarray(b).view(np.uint64))


def backends(O):
    out = [O.load("oracle")]
    if O.reference_available():
        out.append(O.load("ref_serial"))
    return out


def library_call(fn_name, coord_sys, nx, ny, g, bounds, gamma, bc, W, U, dt, gravity=0.0):
    """Set up a System with system_init, copy W and U in, finalize the
    boundary parameters and call the exported function; (code, W, U)."""
    lib = H.library()
    h = H._SystemHandle(lib, coord_sys, nx, ny, g, bounds, gamma)
    try:
        h.s.gravity = gravity
        wn, un = (H.W2, H.U2) if ny > 0 else (H.W1, H.U1)
        for dst, src in zip(h.fields(wn), W):
            dst[:] = src.reshape(-1)
        for dst, src in zip(h.fields(un), U):
            dst[:] = src.reshape(-1)
        keep = []
        bcp, _ = H._params(lib, bc, "godunov_first_order_1d", "riemann_solver_exact", "minmod", 0.5, keep)
        code, msg = H._consume(lib, lib.finalize_boundary_condition_param(C.byref(h.s), C.byref(bcp)))
        assert code == 0, msg
        code, msg = H._consume(lib, getattr(lib, fn_name)(C.byref(bcp), C.byref(h.s), dt))
        Wo = np.stack([f.copy() for f in h.fields(wn)]).reshape(W.shape)
        Uo = np.stack([f.copy() for f in h.fields(un)]).reshape(U.shape)
        return code, msg, Wo, Uo
    finally:
        h.close()


@pytest.mark.parametrize("coord", ["cylindrical_1d", "spherical_1d"])
@pytest.mark.parametrize("dt", [1e-3, 0.0137])
def test_geometry_source_matches_oracle_and_reference(hydro_lib, oracle_mod, coord, dt):
    O = oracle_mod
    p = O.sedov_1d(64, coord_sys=coord)
    gold = np.load(os.path.join(GOLDEN, f"sedov_60_{coord}_muscl_hllc_mc.npz"))
    W, U = gold["W"].copy(), gold["U"].copy()
    assert np.abs(W[1]).max() > 0.1   # a moving state, not the initial one
    code, msg, Wl, Ul = library_call("add_geometry_source_term", coord, p.nx, 0, p.g,
                                     (p.x_min, p.x_max), p.gamma, list(p.bc) + [None, None], W, U, dt)
    assert code == 0, msg
    assert not bits_equal(Ul, U)
    for b in backends(O):
        rc, Wb, Ub = b.geometry_source_1d(p, W, U, dt)
        assert rc == 0
        assert bits_equal(Ul, Ub) and bits_equal(Wl, Wb), b.prefix


@pytest.mark.parametrize("dt", [2e-3, 0.011])
def test_gravity_source_matches_oracle_and_reference(hydro_lib, oracle_mod, dt):
    O = oracle_mod
    p = O.rayleigh_taylor(24, 40, g=3, steps=30)
    gold = np.load(os.path.join(GOLDEN, "rayleigh_taylor_24x40_g3_30.npz"))
    W, U = gold["W"].copy(), gold["U"].copy()
    code, msg, Wl, Ul = library_call("add_gravity_source_term_2d", "cartesian_2d", p.nx, p.ny, p.g,
                                     (p.x_min, p.x_max, p.y_min, p.y_max), p.gamma, p.bc, W, U, dt,
                                     gravity=p.gravity)
    assert code == 0, msg
    assert not bits_equal(Ul, U)
    for b in backends(O):
        rc, Wb, Ub = b.gravity_source_2d(p, W, U, dt)
        assert rc == 0
        both_nan = np.isnan(Wl) & np.isnan(Wb)
        assert bits_equal(Ul, Ub), b.prefix
        assert bits_equal(np.where(both_nan, 0.0, Wl), np.where(both_nan, 0.0, Wb)), b.prefix


def test_zero_gravity_leaves_the_state_alone(hydro_lib, oracle_mod):
    """gravity == 0 returns at once, without the conversion or the ghost
    fill (src/source_term.c:195-198)."""
    O = oracle_mod
    p = O.rayleigh_taylor(24, 40, g=3, steps=30)
    W = p.W.copy()
    W[:, 0, :] = 123.0    # a ghost row the boundary routine would overwrite
    code, msg, Wl, Ul = library_call("add_gravity_source_term_2d", "cartesian_2d", p.nx, p.ny, p.g,
                                     (p.x_min, p.x_max, p.y_min, p.y_max), p.gamma, p.bc, W, p.U, 0.01,
                                     gravity=0.0)
    assert code == 0, msg
    assert bits_equal(Wl, W) and bits_equal(Ul, p.U)


def test_geometry_source_rejects_cartesian_grids(hydro_lib, oracle_mod):
    O = oracle_mod
    p = O.sod_1d(32)
    code, msg, _, _ = library_call("add_geometry_source_term", "cartesian_1d", p.nx, 0, p.g,
                                   (p.x_min, p.x_max), p.gamma, list(p.bc) + [None, None], p.W, p.U, 1e-3)
    assert code == 2   # VALUE_ERROR
    assert "Wrong coordinate system, expected cylindrical 1D or spherical 1D." in msg
