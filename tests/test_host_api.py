"""Host-side behaviour of the C-ABI library (CPU only, no compute on a GPU).

* every function declared in include/*.h is exported by libhydro_gb300.so;
* struct layouts match the reference headers (when the reference tree is
  present, a tiny C program prints sizeof/offsetof under both header sets);
* set-up semantics follow the reference: geometry, parameter finalisation,
  error codes and messages, host ghost fill, conversions;
* with no usable GPU, launch_simulation fails loudly (no CPU fallback).
"""
import ctypes as C
import os
import re
import subprocess
import sys

import numpy as np
import pytest

import hydrofv_gb300 as H

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402

REF_SRC = O.REF_SRC   # the reference's headers, staged by `make -C oracle stage`


def declared_functions():
    names = set()
    for f in os.listdir(INCLUDE):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(INCLUDE, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"typedef[^;]*;", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b([a-z_][a-z0-9_]*)\s*\(", text, flags=re.M):
            if m.group(1) not in ("if", "while", "return", "sizeof"):
                names.add(m.group(1))
    return names


def test_every_declared_function_is_exported(hydro_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", H.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = sorted(declared_functions() - exported)
    assert not missing, missing
    # the reference's public surface (src/hydro.h and the headers it includes) is all there
    for name in ["launch_simulation", "system_init", "free_system_memory",
                 "convert_conserved_to_primitive", "convert_primitive_to_conserved",
                 "finalize_boundary_condition_param", "set_boundary_condition",
                 "finalize_integrator_param", "integrator_launch_simulation", "muscl_hancock_2d",
                 "godunov_first_order_1d", "store_snapshot", "solve_flux_hllc_2d", "guess_p",
                 "solve_exact_1d", "limit_slope", "get_time_step_2d", "print_and_free_traceback"]:
        assert name in exported, name


STRUCT_PROBE = r"""
#include <stddef.h>
#include <stdio.h>
#include "hydro.h"
#define P(T, f) printf(#T "." #f " %zu\n", offsetof(T, f))
int main(void) {
    printf("System %zu\nBoundaryConditionParam %zu\nIntegratorParam %zu\nStoringParam %zu\n"
           "Settings %zu\nSimulationParam %zu\nSimulationStatus %zu\nErrorStatus %zu\n",
           sizeof(System), sizeof(BoundaryConditionParam), sizeof(IntegratorParam),
           sizeof(StoringParam), sizeof(Settings), sizeof(SimulationParam),
           sizeof(SimulationStatus), sizeof(ErrorStatus));
    P(System, num_ghost_cells_side); P(System, dx_); P(System, density_); P(System, volume_);
    P(BoundaryConditionParam, set_boundary_condition_cartesian_2d_y_max);
    P(BoundaryConditionParam, boundary_condition_flag_z_max_);
    P(IntegratorParam, tol); P(IntegratorParam, slope_limiter_flag_);
    P(StoringParam, storing_interval); P(StoringParam, store_count_);
    P(SimulationStatus, dt);
    return 0;
}
"""


def _probe(include_dir, tmp_path, tag):
    src = tmp_path / f"probe_{tag}.c"
    exe = tmp_path / f"probe_{tag}"
    src.write_text(STRUCT_PROBE)
    subprocess.run(["gcc", "-std=gnu99", f"-I{include_dir}", str(src), "-o", str(exe)], check=True)
    return subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout


def test_struct_layouts_match_ctypes(tmp_path):
    out = _probe(INCLUDE, tmp_path, "ours")
    sizes = dict(line.split() for line in out.splitlines())
    for name in ["System", "BoundaryConditionParam", "IntegratorParam", "StoringParam",
                 "Settings", "SimulationParam", "SimulationStatus", "ErrorStatus"]:
        assert int(sizes[name]) == C.sizeof(getattr(H, name)), name


@pytest.mark.skipif(not os.path.isdir(REF_SRC), reason="reference tree not present")
def test_struct_layouts_match_reference(tmp_path):
    assert _probe(INCLUDE, tmp_path, "ours") == _probe(REF_SRC, tmp_path, "ref")


def make_system(lib, nx=8, ny=6, g=2, coord="cartesian_2d"):
    keep = coord.encode()
    s = lib.get_new_system_struct()
    s.coord_sys = keep
    s.gamma = 1.4
    s.x_min, s.x_max, s.y_min, s.y_max = 0.0, 1.0, -1.0, 2.0
    s.num_cells_x, s.num_cells_y, s.num_ghost_cells_side = nx, ny, g
    return s, keep


def test_system_init_geometry(hydro_lib):
    lib = hydro_lib
    s, keep = make_system(lib)
    code, msg = H._consume(lib, lib.system_init(C.byref(s)))
    assert code == 0, msg
    assert s.coord_sys_flag_ == 2
    assert s.dx_ == 1.0 / 12 and s.dy_ == 3.0 / 10        # ghosts inside [x_min, x_max]
    mx = np.ctypeslib.as_array(s.mid_points_x_, shape=(12,))
    assert np.array_equal(mx, 0.0 + (np.arange(12) + 0.5) * (1.0 / 12))
    assert np.ctypeslib.as_array(s.surface_area_x_, shape=(12,))[0] == s.dy_
    assert np.ctypeslib.as_array(s.surface_area_y_, shape=(10,))[0] == s.dx_
    assert np.all(np.ctypeslib.as_array(s.volume_, shape=(120,)) == s.dx_ * s.dy_)
    lib.free_system_memory(C.byref(s))


@pytest.mark.parametrize("field,value,code,text", [
    ("gamma", 0.5, 2, "Gamma must be greater than 1"),
    ("num_ghost_cells_side", 0, 2, "Number of ghost cells per side must be at least 1"),
    ("num_cells_y", 0, 2, "Number of cells in y-direction must be positive"),
    ("x_max", -5.0, 2, "x_min must be less than x_max"),
])
def test_system_init_errors(hydro_lib, field, value, code, text):
    lib = hydro_lib
    s, keep = make_system(lib)
    setattr(s, field, value)
    rc, msg = H._consume(lib, lib.system_init(C.byref(s)))
    assert rc == code and text in msg


def test_unknown_coordinate_system(hydro_lib):
    lib = hydro_lib
    s, keep = make_system(lib, coord="polar_2d")
    rc, msg = H._consume(lib, lib.system_init(C.byref(s)))
    assert rc == 2 and "Coordinate system not recognized." in msg


def test_parameter_finalisation_errors(hydro_lib):
    lib = hydro_lib
    s, keep = make_system(lib)
    H._consume(lib, lib.system_init(C.byref(s)))
    bcp = lib.get_new_boundary_condition_param()
    names = [b"periodic", b"reflective", b"none", b"none"]
    bcp.boundary_condition_x_min, bcp.boundary_condition_x_max = names[0], names[1]
    bcp.boundary_condition_y_min, bcp.boundary_condition_y_max = names[2], names[3]
    rc, msg = H._consume(lib, lib.finalize_boundary_condition_param(C.byref(s), C.byref(bcp)))
    assert rc == 2 and "Periodic boundary condition mismatch for x_min and x_max." in msg
    bcp.boundary_condition_x_min = b"custom"
    rc, msg = H._consume(lib, lib.finalize_boundary_condition_param(C.byref(s), C.byref(bcp)))
    assert rc == 3 and "Custom boundary condition pointer for x_min is NULL." in msg
    bcp.boundary_condition_x_min = b"sticky"
    rc, msg = H._consume(lib, lib.finalize_boundary_condition_param(C.byref(s), C.byref(bcp)))
    assert rc == 2 and "x_min is not recognized" in msg

    ip = lib.get_new_integrator_param()
    assert (ip.cfl, ip.cfl_initial_shrink_factor, ip.cfl_initial_shrink_num_steps, ip.tol) == (0.5, 0.2, 10, 1e-6)
    rc, msg = H._consume(lib, lib.finalize_integrator_param(C.byref(ip)))
    assert rc == 3 and "Integrator is not set." in msg
    ip.integrator, ip.riemann_solver, ip.slope_limiter = b"muscl_hancock_2d", b"riemann_solver_hllc", b"superbee"
    rc, msg = H._consume(lib, lib.finalize_integrator_param(C.byref(ip)))
    assert rc == 2 and "Slope limiter not recognized." in msg
    ip.slope_limiter = b"minmod"
    ip.cfl = 0.0
    rc, msg = H._consume(lib, lib.finalize_integrator_param(C.byref(ip)))
    assert rc == 2 and "CFL number must be positive." in msg
    lib.free_system_memory(C.byref(s))


def test_host_ghost_fill_and_conversion_match_oracle(hydro_lib, oracle_mod):
    """set_boundary_condition and convert_primitive_to_conserved (set-up helpers)."""
    lib = hydro_lib
    O = oracle_mod
    for bc in [("reflective", "transmissive", "periodic", "periodic"),
               ("periodic", "periodic", "reflective", "none")]:
        p = O.random_problem_2d(9, 7, 3, bc, "minmod", 1)
        W = p.W.copy()
        W[:, :p.g, :] = 0.0     # wipe ghosts, let the library fill them
        W[:, -p.g:, :] = 0.0
        W[:, :, :p.g] = 0.0
        W[:, :, -p.g:] = 0.0
        h = H._SystemHandle(lib, "cartesian_2d", p.nx, p.ny, p.g, (0.0, 1.0, 0.0, 1.0), p.gamma)
        for dst, src in zip(h.fields(H.W2), W):
            dst[:] = src.reshape(-1)
        keep = []
        bcp, _ = H._params(lib, bc, "muscl_hancock_2d", "riemann_solver_hllc", "minmod", 0.5, keep)
        assert H._consume(lib, lib.finalize_boundary_condition_param(C.byref(h.s), C.byref(bcp)))[0] == 0
        assert H._consume(lib, lib.set_boundary_condition(C.byref(bcp), C.byref(h.s)))[0] == 0
        assert H._consume(lib, lib.convert_primitive_to_conserved(C.byref(h.s)))[0] == 0
        got = np.stack([f.copy() for f in h.fields(H.W2)]).reshape(W.shape)
        expect = W.copy()
        O.apply_bc_2d(expect, p.g, p.nx, p.ny, bc)
        assert np.array_equal(got, expect)
        U = np.stack([f.copy() for f in h.fields(H.U2)]).reshape(W.shape)
        dx, dy = 1.0 / (p.nx + 2 * p.g), 1.0 / (p.ny + 2 * p.g)
        assert np.array_equal(U, O.primitive_to_conserved_2d(expect, p.gamma, dx * dy))
        h.close()


def test_launch_checks_ghost_cells(hydro_lib, oracle_mod):
    p = oracle_mod.shear_layer(16, g=1, steps=1)
    r = H.run_2d(p.nx, p.ny, p.g, (0, 1, 0, 1), p.gamma, p.W, p.U, max_steps=1)
    assert r.code == 2 and "Number of ghost cells must be at least 2." in r.message


def test_launch_rejects_exact_solver_in_2d(hydro_lib, oracle_mod):
    p = oracle_mod.shear_layer(16, steps=1)
    r = H.run_2d(p.nx, p.ny, p.g, (0, 1, 0, 1), p.gamma, p.W, p.U, riemann_solver="riemann_solver_exact",
                 max_steps=1)
    assert r.code != 0


@pytest.mark.skipif(H.device_count() > 0 if os.path.exists(H.LIB_PATH) else False,
                    reason="a GPU is visible")
def test_no_cpu_fallback_without_gpu(hydro_lib, oracle_mod):
    p = oracle_mod.shear_layer(16, steps=2)
    r = H.run_2d(p.nx, p.ny, p.g, (0, 1, 0, 1), p.gamma, p.W, p.U, max_steps=2)
    assert r.code == 1 and "CUDA error" in r.message
    assert r.num_steps == 0
    # host arrays untouched
    assert np.array_equal(r.W, p.W) and np.array_equal(r.U, p.U)


def test_adjoint_rejects_boundary_none():
    """The adjoint session validates its inputs before touching a device."""
    from hydrofv_gb300.problems import random_problem_2d
    p = random_problem_2d(16, 16, seed=1, bc=("none",) * 4, limiter="minmod", steps=4, smooth=True)
    with pytest.raises(H.HydroError):
        H.Adjoint2D(p, steps=4, checkpoint_every=2)



def test_guess_p_divide_free_ratio_test_matches_reference(oracle_mod):
    """The PVRS test p_max/p_min <= 2 is decided by p_max <= 2 p_min for
    p_min > 0 in the library; the oracle keeps the reference's divide.  Edge
    values around the boundary (quotients within an ulp of 2, subnormal and
    huge pressures) must select the same guess."""
    import math
    rng = np.random.default_rng(5)
    orc = oracle_mod.load("oracle")
    lib = H.library()
    cases = []
    for _ in range(4000):
        p_min = 10.0 ** rng.uniform(-310, 300)
        k = int(rng.integers(-3, 4))
        p_max = 2.0 * p_min
        for _ in range(abs(k)):
            p_max = math.nextafter(p_max, math.inf if k > 0 else 0.0)
        cases.append((p_min, p_max))
    cases += [(5e-324, 1e-323), (5e-324, 1.5e-323), (1e308, 1.7e308), (1e308, 1.79e308)]
    for pl, pr in cases:
        for a in ((pl, pr), (pr, pl)):
            args = (1.4, 1.0, 0.0, a[0], 1.0, 1.0, 1e-3, a[1], 1.0, 1e-300)
            ref = orc.guess_p(*args)
            got = lib.guess_p(*args)
            assert (ref == got) or (math.isnan(ref) and math.isnan(got)), (a, ref, got)


@pytest.mark.parametrize("nx,ny", [(2048, 2048), (1024, 1024), (8192, 8192), (4096, 1000), (130, 7),
                                   (3, 260), (1000, 4096), (256, 256)])
@pytest.mark.parametrize("slots", [152, 608, 1216])
def test_guided_chunk_plan_covers_every_row_once(hydro_lib, nx, ny, slots):
    """The FP64 step's work items (guided row chunks: tall items first, the
    last rows in short items) decoded as the kernel decodes them: every
    interior row of every strip exactly once, the tall items before the
    short ones."""
    import hydrofv_gb300 as H
    g = 2
    (h1, h2, tail), rows = H.chunk_plan(nx, ny, g, slots)
    strips = (nx + 125) // 126
    assert 0 <= tail < ny and h1 >= 1 and (tail == 0 or 1 <= h2 <= h1)
    seen = np.zeros((strips, ny), dtype=np.int32)
    for strip, r0, r1 in rows:
        assert 0 <= strip < strips and g <= r0 < r1 <= g + ny
        seen[strip, r0 - g:r1 - g] += 1
    assert np.all(seen == 1)
    heights = rows[:, 2] - rows[:, 1]
    big = rows[:, 1] < g + ny - tail
    assert np.all(heights[big] <= h1) and np.all(heights[~big] <= max(h2, 1))
    if tail:
        assert np.all(np.diff(big.astype(int)) <= 0)      # tall items first


def _bisection_warnings(text):
    """The iteration counts of the exact solver's warnings in stderr text."""
    return [int(m) for m in re.findall(r"Bisection method did not converge after (\d+) iterations", text)]


def test_exact_solver_verbose_warnings_like_the_reference(hydro_lib, oracle_mod, capfd):
    """solve_exact_1d with verbose > 0 warns every 500 bisection iterations
    (src/riemann_solver_exact.c:736-744): a collision at pressures near 1e12,
    where the bisection cannot reach its absolute tolerance, prints ten
    warnings (500 ... 5000) before failing; verbose = 0 prints none."""
    L = (0.11595095827026866, 1130033.0105304043, 550729744742.7017)
    R = (0.002907116592475837, 4172977.0479090274, 4571920669538.1)
    out = [C.c_double() for _ in range(3)]
    for verbose, want in ((1, list(range(500, 5001, 500))), (0, [])):
        capfd.readouterr()
        code, msg = H._consume(hydro_lib, hydro_lib.solve_exact_1d(
            *[C.pointer(o) for o in out], 1.4, *L, *R, 1e-6, 0.0, verbose))
        assert code == 1 and "Bisection method did not converge after 5001 iterations" in msg
        assert _bisection_warnings(capfd.readouterr().err) == want
    O = oracle_mod
    if O.reference_available():
        ref = O.load("ref_serial")
        ref.lib.ref_set_verbose(1)
        try:
            capfd.readouterr()
            assert ref.exact_status(1.4, L, R)[0] == 2
            assert _bisection_warnings(capfd.readouterr().err) == list(range(500, 5001, 500))
        finally:
            ref.lib.ref_set_verbose(0)


@pytest.mark.parametrize("side,where", [(40, "last"), (1100, "first"), (1100, "middle"), (1100, "last")])
def test_non_uniform_volumes_are_rejected_before_any_gpu_work(hydro_lib, side, where):
    """The 2D path needs the uniform face areas and cell volumes system_init
    sets; a System whose volume array was changed in any cell is refused with
    NOT_IMPLEMENTED_ERROR on the host (grids above 2^20 cells are scanned by
    several host threads), and an untouched one passes the check (it then
    fails only where no GPU is visible, with the CUDA error)."""
    from hydrofv_gb300.problems import shear_layer
    p = shear_layer(side, steps=1)
    with H.Simulation2D(p.nx, p.ny, p.g, (0, 1, 0, 1), p.gamma, p.W, p.U, bc=p.bc,
                        slope_limiter=p.slope_limiter, cfl=p.cfl, tf=p.tf, max_steps=1) as sim:
        n = (p.nx + 2 * p.g) * (p.ny + 2 * p.g)
        vol = np.ctypeslib.as_array(sim.h.s.volume_, shape=(n,))
        k = {"first": 1, "middle": n // 2 + 17, "last": n - 1}[where]
        keep = vol[k]
        vol[k] = keep * (1.0 + 1e-15)
        code, msg, _, _ = sim.launch()
        assert code == 6, msg   # NOT_IMPLEMENTED_ERROR
        assert "uniform face areas and cell volumes" in msg
        vol[k] = keep
        if H.device_count() == 0:
            code, msg, _, _ = sim.launch()
            assert code != 6 and "CUDA" in msg, msg
