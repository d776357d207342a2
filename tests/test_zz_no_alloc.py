"""The allocation-free entry point against the regular one.

hydro_gpu_muscl_hancock_2d_noalloc serves callers that must not allocate
while they step (device memory owned by another allocator, or loops that
cannot take cudaFree's device-wide synchronisation): its device state lives
in a static array shared by every call.  This test drives it through the C
ABI on consecutive calls with different grids -- so a call starts from
whatever the previous one left in the array -- and checks each result
against hydro_gpu_launch_simulation on the same input, with the tolerance
the other parity tests use, over both limiters' code paths and the
boundary kinds the entry point parses itself (including periodic sides).
A run that ends in a device error (an unstable CFL number) must return the
same code, message, status and state as the regular entry point.  Around
repeated calls the device's free memory must not move: the entry point
allocates nothing.  It also checks that an oversized grid is refused with a
clear error.

Collected last on purpose (file name), so a run that stops at the first
failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import hydrofv_gb300 as H
from hydrofv_gb300.problems import random_problem_2d, shear_layer

pytestmark = pytest.mark.gpu

REL_L1_TOL = 1e-12
MAX_CELLS = 32768  # HYDRO_GPU_NOALLOC_MAX_CELLS


def _bind():
    lib = H.library()
    fn = lib.hydro_gpu_muscl_hancock_2d_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(H.BoundaryConditionParam), C.POINTER(H.System),
                   C.POINTER(H.IntegratorParam), C.c_double, C.c_int64,
                   C.POINTER(H.SimulationStatus), C.c_char_p, C.c_int]
    return lib, fn


def run_noalloc(p):
    lib, fn = _bind()
    h = H._SystemHandle(lib, "cartesian_2d", p.nx, p.ny, p.g,
                        (p.x_min, p.x_max, p.y_min, p.y_max), p.gamma)
    try:
        for dst, src in zip(h.fields(H.W2), p.W):
            dst[:] = src.reshape(-1)
        for dst, src in zip(h.fields(H.U2), p.U):
            dst[:] = src.reshape(-1)
        keep = []
        bcp, ip = H._params(lib, p.bc, p.integrator, p.riemann_solver, p.slope_limiter, p.cfl, keep)
        st = H.SimulationStatus(0, 0.0, 0.0)
        err = C.create_string_buffer(512)
        rc = fn(C.byref(bcp), C.byref(h.s), C.byref(ip), p.tf, p.max_steps, C.byref(st),
                err, len(err))
        W = np.stack([f.copy() for f in h.fields(H.W2)]).reshape((4,) + h.shape)
        U = np.stack([f.copy() for f in h.fields(H.U2)]).reshape((4,) + h.shape)
        return rc, err.value.decode(), W, U, st
    finally:
        h.close()


def device_free_bytes():
    """Free device memory as the driver reports it, for the context that the
    library's calls made current on this thread."""
    cuda = C.CDLL("libcuda.so.1")
    free, total = C.c_size_t(0), C.c_size_t(0)
    rc = cuda.cuMemGetInfo_v2(C.byref(free), C.byref(total))
    assert rc == 0, f"cuMemGetInfo_v2 returned {rc}"
    return free.value


def run_regular(p):
    return H.run_2d(p.nx, p.ny, p.g, (p.x_min, p.x_max, p.y_min, p.y_max), p.gamma, p.W, p.U,
                    bc=p.bc, integrator=p.integrator, riemann_solver=p.riemann_solver,
                    slope_limiter=p.slope_limiter, cfl=p.cfl, tf=p.tf, max_steps=p.max_steps)


def rel_l1(a, b, g):
    ia, ib = a[:, g:-g, g:-g], b[:, g:-g, g:-g]
    return np.abs(ia - ib).sum(axis=(1, 2)) / np.abs(ib).sum(axis=(1, 2))


def consecutive_problems():
    return [
        shear_layer(96, steps=30),
        random_problem_2d(150, 100, 5, ("reflective", "transmissive", "none", "reflective"),
                          "van_leer", 25, smooth=True),
        random_problem_2d(120, 90, 3, ("periodic",) * 4, "minmod", 20, smooth=True),
        shear_layer(96, steps=30),
    ]


def test_noalloc_matches_regular_entry_point_on_consecutive_calls(gpu_available):
    problems = consecutive_problems()
    for p in problems:
        assert (p.nx + 2 * p.g) * (p.ny + 2 * p.g) <= MAX_CELLS
        rc, msg, W, U, st = run_noalloc(p)
        ref = run_regular(p)
        assert rc == 0, msg
        assert ref.code == 0, ref.message
        assert st.num_steps == ref.num_steps == p.max_steps
        assert st.t == pytest.approx(ref.t, rel=1e-13)
        assert np.all(rel_l1(U, ref.U, p.g) <= REL_L1_TOL)
        assert np.all(rel_l1(W, ref.W, p.g) <= REL_L1_TOL)


def test_noalloc_rejects_grids_above_the_limit(gpu_available):
    p = random_problem_2d(200, 200, 1, ("periodic",) * 4, "minmod", 2)
    assert (p.nx + 2 * p.g) * (p.ny + 2 * p.g) > MAX_CELLS
    rc, msg, W, U, st = run_noalloc(p)
    assert rc == 2  # VALUE_ERROR
    assert "exceeds the no-allocation limit" in msg
    assert st.num_steps == 0


def test_noalloc_device_error_matches_regular_entry_point(gpu_available):
    """An unstable CFL number drives the point blast into HLLC's invalid wave
    speed at step 21: the code, the reference's message, the status and the
    state at the start of the failing step agree with the regular entry
    point, and a following call on the same array runs cleanly."""
    from hydrofv_gb300.problems import point_blast
    p = point_blast(32, steps=80)
    p.cfl = 2.0
    rc, msg, W, U, st = run_noalloc(p)
    ref = run_regular(p)
    assert ref.code == 2 and rc == 2, (ref.code, rc, msg)
    assert "Invalid wave speed for the HLLC riemann solver. Possible fix: use a smaller CFL." in msg
    assert st.num_steps == ref.num_steps == 21
    assert st.t == ref.t and st.dt == ref.dt
    assert np.all(rel_l1(U, ref.U, p.g) <= REL_L1_TOL)
    assert np.all(rel_l1(W, ref.W, p.g) <= REL_L1_TOL)
    q = shear_layer(64, steps=10)
    rc, msg, W, U, st = run_noalloc(q)
    ref = run_regular(q)
    assert rc == 0 and st.num_steps == ref.num_steps == 10, msg
    assert np.all(rel_l1(U, ref.U, q.g) <= REL_L1_TOL)


def test_noalloc_calls_leave_device_memory_unchanged(gpu_available):
    """A first round of calls creates the CUDA context and loads every kernel
    the later calls launch (module loading is lazy and takes device memory
    on a kernel's first launch); after that, repeated calls must not change
    the device's free memory."""
    problems = consecutive_problems()
    for p in problems:
        assert run_noalloc(p)[0] == 0
    before = device_free_bytes()
    for _ in range(2):
        for p in problems:
            assert run_noalloc(p)[0] == 0
    assert device_free_bytes() == before
