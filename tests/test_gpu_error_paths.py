"""Device error paths of the drop-in, driven through launch_simulation.

Every fault is planted on the host, in the initial state or the parameters a
caller passes, and the kernels meet it in the ordinary course of a step:

* an unstable CFL number, which drives the 2D MUSCL-Hancock and Godunov
  schemes into states where HLLC has no valid wave speed: "Invalid wave
  speed for the HLLC riemann solver. Possible fix: use a smaller CFL."
  (src/riemann_solver_hllc.c:372-375), raised some steps into the run;
* dt == 0 (src/integrator_muscl_hancock.c:545-549,
  src/integrator_godunov_first_order.c:141-145): the smallest positive CFL
  number (it passes the "CFL number must be positive" check,
  src/integrator.c:88-91), and an infinite velocity, whose signal speed
  makes cfl / (S_x/dx + S_y/dy) zero;
* the exact solver's bisection that cannot converge
  (src/riemann_solver_exact.c:745-754): pressures near 1e12, where
  neighbouring doubles are further apart than the absolute tolerance 1e-6,
  so the bracket never closes; also NaN and negative pressures, and an
  unstable CFL number in the Godunov 1D scheme;
* the exact solver's bracket search that finds no sign change
  (src/riemann_solver_exact.c:702-707): states near the top of the double
  range, where ten times the pressure guess overflows.

For each case the error code, the reference's message, the status
(num_steps, t, dt of the failing step) and the returned arrays are
compared with the oracle.  The arrays are the state at the start of the
failing step, i.e. the oracle's state after num_steps completed steps: the
reference leaves a partial update there (the faces solved before the
failing one), which this library does not reproduce.
"""
import os
import shutil
import subprocess
import warnings

import numpy as np
import pytest

import hydrofv_gb300 as H

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
VALUE_ERROR = 2
FAILURE = 1
HLLC_MSG = "Invalid wave speed for the HLLC riemann solver. Possible fix: use a smaller CFL."
DT_MSG = "dt is zero."
BISECTION_MSG = "Bisection method did not converge after 5001 iterations for exact riemann solver."
BRACKET_MSG = "Failed to bracket the root for bisection method."
REL_L1_TOL = 1e-12


def run2(p):
    return H.run_2d(p.nx, p.ny, p.g, (p.x_min, p.x_max, p.y_min, p.y_max), p.gamma, p.W, p.U,
                    bc=p.bc, integrator=p.integrator, riemann_solver=p.riemann_solver,
                    slope_limiter=p.slope_limiter, cfl=p.cfl, tf=p.tf, max_steps=p.max_steps)


def run1(p):
    return H.run_1d(p.nx, p.g, (p.x_min, p.x_max), p.gamma, p.W, p.U, bc=p.bc,
                    integrator=p.integrator, riemann_solver=p.riemann_solver,
                    slope_limiter=p.slope_limiter, cfl=p.cfl, tf=p.tf, max_steps=p.max_steps,
                    coord_sys=p.coord_sys)


def same_bits(a, b):
    """Equal arrays, NaN in the same places."""
    return np.array_equal(a, b, equal_nan=True)


def assert_close_2d(O, got, want, g):
    """Interior cells: NaN and infinities in the same places with the same
    values, and at most REL_L1_TOL relative L1 per field over the finite
    ones (an unstable run can carry NaN before HLLC meets it)."""
    fin = np.isfinite(want)
    assert np.array_equal(fin, np.isfinite(got))
    assert np.array_equal(got[~fin], want[~fin], equal_nan=True)
    l1 = O.rel_l1(np.where(fin, got, 0.0), np.where(fin, want, 0.0), g)
    assert np.all(l1 <= REL_L1_TOL), l1


def sod(O, n, steps):
    """The Sod tube stopped after a fixed number of steps (not at t = 0.2)."""
    p = O.sod_1d(n)
    p.max_steps = steps
    p.tf = 1e300
    return p


def check_error(O, p, gpu, code, message, two_d):
    """The GPU run failed like the oracle's: code, message, status, and the
    state at the start of the failing step."""
    orc = O.load("oracle")
    ref = orc.run_2d(p) if two_d else orc.run_1d(p)
    assert ref.rc == code and ref.message == message, (ref.rc, ref.message)
    assert gpu.code == code, (gpu.code, gpu.message)
    assert message in gpu.message, gpu.message
    assert gpu.num_steps == ref.num_steps
    assert gpu.t == ref.t
    assert gpu.dt == ref.dt
    # the oracle's state after the completed steps
    q = p.copy()
    q.max_steps = ref.num_steps
    done = orc.run_2d(q) if two_d else orc.run_1d(q)
    assert done.rc == 0 and done.num_steps == ref.num_steps
    if two_d:
        assert_close_2d(O, gpu.U, done.U, p.g)
        assert_close_2d(O, gpu.W, done.W, p.g)
    else:
        assert same_bits(gpu.U, done.U)
        assert same_bits(gpu.W, done.W)
    return ref


def conserved_1d(O, p):
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        return O.primitive_to_conserved_1d(p.W, p.gamma, (p.x_max - p.x_min) / (p.nx + 2 * p.g))


def conserved_2d(O, p):
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        return O.primitive_to_conserved_2d(p.W, p.gamma, ((p.x_max - p.x_min) / (p.nx + 2 * p.g))
                                           * ((p.y_max - p.y_min) / (p.ny + 2 * p.g)))


@pytest.mark.parametrize("case,integrator,cfl,fail_step", [
    ("point_blast", "muscl_hancock_2d", 2.0, 21),
    ("point_blast", "muscl_hancock_2d", 3.0, 13),
    ("shear_layer", "muscl_hancock_2d", 2.0, 24),
    ("point_blast", "godunov_first_order_2d", 2.0, 60),
])
def test_unstable_cfl_raises_hllc_wave_speed_error(gpu_available, oracle_mod, case, integrator, cfl,
                                                   fail_step):
    O = oracle_mod
    p = (O.point_blast if case == "point_blast" else O.shear_layer)(32, steps=80)
    p.integrator = integrator
    p.cfl = cfl
    gpu = run2(p)
    ref = check_error(O, p, gpu, VALUE_ERROR, HLLC_MSG, two_d=True)
    assert ref.num_steps == fail_step


@pytest.mark.parametrize("integrator", ["muscl_hancock_2d", "godunov_first_order_2d"])
@pytest.mark.parametrize("plant", ["smallest_cfl", "infinite_velocity"])
def test_zero_time_step_2d(gpu_available, oracle_mod, integrator, plant):
    O = oracle_mod
    p = O.point_blast(32, steps=20)
    p.integrator = integrator
    if plant == "smallest_cfl":
        p.cfl = 5e-324
    else:
        p.W[1, 10, 12] = np.inf
        p.U = conserved_2d(O, p)
    gpu = run2(p)
    check_error(O, p, gpu, VALUE_ERROR, DT_MSG, two_d=True)
    assert gpu.num_steps == 0 and gpu.dt == 0.0
    # nothing stepped: the caller's arrays come back as they went in
    assert same_bits(gpu.W, p.W) and same_bits(gpu.U, p.U)


@pytest.mark.parametrize("integrator,solver", [("godunov_first_order_1d", "riemann_solver_exact"),
                                               ("muscl_hancock_1d", "riemann_solver_hllc")])
def test_zero_time_step_1d(gpu_available, oracle_mod, integrator, solver):
    O = oracle_mod
    p = sod(O, 100, 20)
    p.integrator, p.riemann_solver = integrator, solver
    p.cfl = 5e-324
    gpu = run1(p)
    check_error(O, p, gpu, VALUE_ERROR, DT_MSG, two_d=False)
    assert gpu.num_steps == 0
    assert same_bits(gpu.W, p.W) and same_bits(gpu.U, p.U)


@pytest.mark.parametrize("plant,fail_step", [
    ("pressure_scale_1e12", 1),
    ("nan_pressure", 0),
    ("negative_pressure", 0),
    ("cfl_1.5", 20),
    ("cfl_3", 13),
])
def test_exact_solver_bisection_does_not_converge(gpu_available, oracle_mod, plant, fail_step):
    O = oracle_mod
    p = sod(O, 100, 200)
    if plant == "pressure_scale_1e12":
        p.W[2] *= 1e12
    elif plant == "nan_pressure":
        p.W[2, 30] = np.nan
    elif plant == "negative_pressure":
        p.W[2, 30] = -1.0
    else:
        p.cfl = float(plant.split("_")[1])
    p.U = conserved_1d(O, p)
    gpu = run1(p)
    ref = check_error(O, p, gpu, FAILURE, BISECTION_MSG, two_d=False)
    assert ref.num_steps == fail_step


def test_exact_solver_bracket_search_fails(gpu_available, oracle_mod):
    """A collision near the top of the double range: the pressure guess is
    below the root and ten times it overflows, so the bracket search of
    [0, 10 p_guess] finds no sign change.  The energies of these states
    overflow to infinity; the fluxes are computed from W, as in the
    reference's first step."""
    O = oracle_mod
    L = (2.4713952001496793, -6.135057360918247e+154, 4.680966664334494e+296)
    R = (0.29708479651481207, -1.2428437714217527e+155, 1.3194467671491075e+302)
    assert O.load("oracle").exact_status(1.4, L, R)[0] == 1
    p = sod(O, 64, 10)
    left = np.arange(p.W.shape[1]) < p.W.shape[1] // 2
    for q in range(3):
        p.W[q] = np.where(left, L[q], R[q])
    p.U = conserved_1d(O, p)
    gpu = run1(p)
    check_error(O, p, gpu, FAILURE, BRACKET_MSG, two_d=False)
    assert gpu.num_steps == 0


def test_muscl_1d_steps_over_failed_faces_like_the_oracle(gpu_available, oracle_mod):
    """MUSCL-Hancock 1D does not stop on a failed Riemann solve: the
    reference overwrites the flux loop's status with the boundary routine's
    (src/integrator_muscl_hancock.c:249-295, :310) and updates with the
    failed face's uninitialised flux.  Here (and in the oracle) a failed
    face contributes no flux; at CFL 1.5 the Sod tube meets negative
    pressures from step 18 on and still runs its 80 steps."""
    O = oracle_mod
    p = sod(O, 100, 80)
    p.cfl = 1.5
    p.integrator, p.riemann_solver = "muscl_hancock_1d", "riemann_solver_hllc"
    gpu = run1(p)
    ref = O.load("oracle").run_1d(p)
    assert ref.rc == 0 and gpu.code == 0, gpu.message
    assert gpu.num_steps == ref.num_steps == 80
    assert gpu.t == ref.t and gpu.dt == ref.dt
    assert same_bits(gpu.U, ref.U) and same_bits(gpu.W, ref.W)


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc not available")
def test_c_program_gets_the_error_through_launch_simulation(gpu_available, oracle_mod, tmp_path):
    """tests/c_programs/sod_tube.c with its pressures scaled by 1e12: the
    program's launch_simulation returns FAILURE with the reference's message
    in the traceback, and the System arrays hold the state after the
    completed step."""
    O = oracle_mod
    libdir = os.path.dirname(H.LIB_PATH)
    exe = str(tmp_path / "sod_tube")
    build = subprocess.run(["gcc", "-std=gnu99", "-O2", "-I", os.path.join(ROOT, "include"), "-o", exe,
                            os.path.join(HERE, "c_programs", "sod_tube.c"), "-L", libdir,
                            "-l:" + os.path.basename(H.LIB_PATH), "-lm", "-Wl,-rpath," + libdir],
                           stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert build.returncode == 0, build.stdout
    out = str(tmp_path / "state.bin")
    run = subprocess.run([exe, out, "1e12"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                         timeout=300)
    assert run.returncode == 3, run.stdout[-3000:]
    assert BISECTION_MSG in run.stdout

    p = O.sod_1d(1000)
    p.W[2] *= 1e12
    p.U = conserved_1d(O, p)
    ref = O.load("oracle").run_1d(p)
    assert ref.rc == FAILURE and ref.message == BISECTION_MSG
    q = p.copy()
    q.max_steps = ref.num_steps
    done = O.load("oracle").run_1d(q)
    raw = np.fromfile(out, dtype=np.uint8)
    total = p.W.shape[1]
    assert raw.size == 24 + 6 * total * 8
    assert int(raw[:8].view(np.int64)[0]) == ref.num_steps
    assert float(raw[8:16].view(np.float64)[0]) == ref.t
    assert float(raw[16:24].view(np.float64)[0]) == ref.dt
    state = raw[24:].view(np.float64).reshape(6, total)
    assert same_bits(state[:3], done.W) and same_bits(state[3:], done.U)


def _bisection_warnings(text):
    import re
    return [int(m) for m in re.findall(r"Bisection method did not converge after (\d+) iterations", text)]


@pytest.mark.parametrize("verbose", [0, 1])
def test_verbose_run_prints_the_bisection_warnings(gpu_available, oracle_mod, capfd, verbose):
    """Settings.verbose > 0: the failing face of the pressure-scaled Sod tube
    passes 500, 1000, ... 5000 bisection iterations before the error, and
    the run prints the reference's ten warnings; with verbose = 0 none.  The
    reference's own run is the comparison where it was built."""
    O = oracle_mod
    p = sod(O, 100, 200)
    p.W[2] *= 1e12
    p.U = conserved_1d(O, p)
    capfd.readouterr()
    gpu = H.run_1d(p.nx, p.g, (p.x_min, p.x_max), p.gamma, p.W, p.U, bc=p.bc, integrator=p.integrator,
                   riemann_solver=p.riemann_solver, slope_limiter=p.slope_limiter, cfl=p.cfl, tf=p.tf,
                   max_steps=p.max_steps, verbose=verbose)
    got = _bisection_warnings(capfd.readouterr().err)
    assert gpu.code == FAILURE and gpu.num_steps == 1
    want = list(range(500, 5001, 500)) if verbose else []
    assert got == want
    if verbose and O.reference_available():
        ref = O.load("ref_serial")
        ref.lib.ref_set_verbose(1)
        try:
            r = ref.run_1d(p)
            assert r.rc == FAILURE and r.num_steps == 1
            assert _bisection_warnings(capfd.readouterr().err) == got
        finally:
            ref.lib.ref_set_verbose(0)


@pytest.mark.parametrize("case,cfl", [("point_blast", 3.0), ("shear_layer", 2.0)])
def test_fp32_form_reports_the_hllc_error_and_returns_its_last_state(gpu_available, oracle_mod, case, cfl):
    """The FP32 state form meets the same device error on an unstable CFL
    number, from either of its face paths (x faces batched in shared memory,
    y faces in registers): the reference's code and message come back, the
    run stops at the failing step, and the arrays hold the FP32 state after
    the completed steps, bit for bit what a clean FP32 run of that many steps
    returns."""
    O = oracle_mod
    p = (O.point_blast if case == "point_blast" else O.shear_layer)(32, steps=80)
    p.cfl = cfl
    opt = H.default_options(precision=H.PRECISION_FP32)
    gpu = H.run_2d(p.nx, p.ny, p.g, (p.x_min, p.x_max, p.y_min, p.y_max), p.gamma, p.W, p.U,
                   bc=p.bc, integrator=p.integrator, riemann_solver=p.riemann_solver,
                   slope_limiter=p.slope_limiter, cfl=p.cfl, tf=p.tf, max_steps=p.max_steps, options=opt)
    assert gpu.code == VALUE_ERROR, (gpu.code, gpu.message)
    assert HLLC_MSG in gpu.message
    assert 0 < gpu.num_steps < p.max_steps
    clean = H.run_2d(p.nx, p.ny, p.g, (p.x_min, p.x_max, p.y_min, p.y_max), p.gamma, p.W, p.U,
                     bc=p.bc, integrator=p.integrator, riemann_solver=p.riemann_solver,
                     slope_limiter=p.slope_limiter, cfl=p.cfl, tf=p.tf, max_steps=gpu.num_steps,
                     options=opt)
    assert clean.code == 0 and clean.num_steps == gpu.num_steps
    assert clean.t == gpu.t
    assert same_bits(gpu.U, clean.U) and same_bits(gpu.W, clean.W)
