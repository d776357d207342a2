"""hydrofv_gb300 -- GB300-native finite-volume step behind hydroFV's C API.

The product is the C-ABI shared library ``libhydro_gb300.so`` (built in-tree
by :mod:`hydrofv_gb300.build`).  This module is a thin ctypes front-end for
Python callers, tests and the benchmark: it mirrors the C structs of
``include/*.h`` and drives the library through its public entry points
(``system_init``, ``launch_simulation``, ``hydro_gpu_launch_simulation``,
``hydro_gpu_solver_*``).  Nothing here computes hydrodynamics; if the library
is missing the import of :func:`library` fails loudly.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libhydro_gb300.so")

_dp = C.POINTER(C.c_double)


class ErrorStatus(C.Structure):
    _fields_ = [("return_code", C.c_int), ("traceback", C.c_void_p), ("traceback_code_", C.c_int)]


class System(C.Structure):
    _fields_ = [
        ("coord_sys", C.c_char_p),
        ("gamma", C.c_double), ("gravity", C.c_double),
        ("x_min", C.c_double), ("x_max", C.c_double),
        ("y_min", C.c_double), ("y_max", C.c_double),
        ("z_min", C.c_double), ("z_max", C.c_double),
        ("num_cells_x", C.c_int), ("num_cells_y", C.c_int), ("num_cells_z", C.c_int),
        ("num_ghost_cells_side", C.c_int),
        ("coord_sys_flag_", C.c_int),
        ("dx_", C.c_double), ("dy_", C.c_double), ("dz_", C.c_double),
        ("density_", _dp), ("velocity_x_", _dp), ("velocity_y_", _dp), ("velocity_z_", _dp),
        ("pressure_", _dp), ("mass_", _dp), ("momentum_x_", _dp), ("momentum_y_", _dp),
        ("momentum_z_", _dp), ("energy_", _dp),
        ("mid_points_x_", _dp), ("mid_points_y_", _dp), ("mid_points_z_", _dp),
        ("surface_area_x_", _dp), ("surface_area_y_", _dp), ("surface_area_z_", _dp),
        ("volume_", _dp),
    ]


class BoundaryConditionParam(C.Structure):
    _fields_ = [
        ("boundary_condition_x_min", C.c_char_p), ("boundary_condition_x_max", C.c_char_p),
        ("boundary_condition_y_min", C.c_char_p), ("boundary_condition_y_max", C.c_char_p),
        ("boundary_condition_z_min", C.c_char_p), ("boundary_condition_z_max", C.c_char_p),
        ("set_boundary_condition_1d_x_min", C.c_void_p), ("set_boundary_condition_1d_x_max", C.c_void_p),
        ("set_boundary_condition_cartesian_2d_x_min", C.c_void_p),
        ("set_boundary_condition_cartesian_2d_x_max", C.c_void_p),
        ("set_boundary_condition_cartesian_2d_y_min", C.c_void_p),
        ("set_boundary_condition_cartesian_2d_y_max", C.c_void_p),
        ("boundary_condition_flag_x_min_", C.c_int), ("boundary_condition_flag_x_max_", C.c_int),
        ("boundary_condition_flag_y_min_", C.c_int), ("boundary_condition_flag_y_max_", C.c_int),
        ("boundary_condition_flag_z_min_", C.c_int), ("boundary_condition_flag_z_max_", C.c_int),
    ]


class IntegratorParam(C.Structure):
    _fields_ = [
        ("integrator", C.c_char_p), ("riemann_solver", C.c_char_p), ("slope_limiter", C.c_char_p),
        ("cfl", C.c_double), ("cfl_initial_shrink_factor", C.c_double),
        ("cfl_initial_shrink_num_steps", C.c_int), ("tol", C.c_double),
        ("integrator_flag_", C.c_int), ("riemann_solver_flag_", C.c_int),
        ("slope_limiter_flag_", C.c_int),
    ]


class StoringParam(C.Structure):
    _fields_ = [
        ("output_dir", C.c_char_p), ("is_storing", C.c_bool), ("store_initial", C.c_bool),
        ("storing_interval", C.c_double), ("storing_method_flag_", C.c_int),
        ("store_count_", C.c_int),
    ]


class Settings(C.Structure):
    _fields_ = [("verbose", C.c_int), ("no_progress_bar", C.c_bool)]


class SimulationParam(C.Structure):
    _fields_ = [("tf", C.c_double)]


class SimulationStatus(C.Structure):
    _fields_ = [("num_steps", C.c_int64), ("t", C.c_double), ("dt", C.c_double)]


class HydroGpuOptions(C.Structure):
    _fields_ = [
        ("device", C.c_int), ("max_steps", C.c_int64), ("precision", C.c_int),
        ("chunk_steps", C.c_int), ("use_graph", C.c_int), ("block_threads", C.c_int),
        ("chunk_rows", C.c_int), ("autotune", C.c_int), ("sync_snapshots", C.c_int),
    ]


class HydroGpuAdjointStats(C.Structure):
    _fields_ = [
        ("forward_ms", C.c_double), ("recompute_ms", C.c_double), ("vjp_ms", C.c_double),
        ("tangent_ms", C.c_double), ("replay_ms", C.c_double), ("steps", C.c_int64),
        ("checkpoint_every", C.c_int64), ("checkpoints", C.c_int64),
        ("recompute_mismatches", C.c_int64), ("kernel_launches", C.c_int64),
        ("device_bytes", C.c_int64), ("interior_cells", C.c_int64),
    ]


class HydroGpuStats(C.Structure):
    _fields_ = [
        ("total_ms", C.c_double), ("h2d_ms", C.c_double), ("step_ms", C.c_double),
        ("d2h_ms", C.c_double), ("steps", C.c_int64), ("step_launches", C.c_int64),
        ("kernel_launches", C.c_int64), ("h2d_bytes", C.c_int64), ("d2h_bytes", C.c_int64),
        ("interior_cells", C.c_int64),
    ]


PRECISION_FP64 = 0
PRECISION_FP32 = 1

_P = C.POINTER
_SIGNATURES = {
    "get_new_system_struct": (System, []),
    "system_init": (ErrorStatus, [_P(System)]),
    "free_system_memory": (None, [_P(System)]),
    "get_new_boundary_condition_param": (BoundaryConditionParam, []),
    "finalize_boundary_condition_param": (ErrorStatus, [_P(System), _P(BoundaryConditionParam)]),
    "set_boundary_condition": (ErrorStatus, [_P(BoundaryConditionParam), _P(System)]),
    "convert_primitive_to_conserved": (ErrorStatus, [_P(System)]),
    "convert_conserved_to_primitive": (ErrorStatus, [_P(System)]),
    "add_geometry_source_term": (ErrorStatus, [_P(BoundaryConditionParam), _P(System), C.c_double]),
    "add_gravity_source_term_2d": (ErrorStatus, [_P(BoundaryConditionParam), _P(System), C.c_double]),
    "get_new_integrator_param": (IntegratorParam, []),
    "finalize_integrator_param": (ErrorStatus, [_P(IntegratorParam)]),
    "get_new_storing_param": (StoringParam, []),
    "finalize_storing_param": (ErrorStatus, [_P(StoringParam)]),
    "launch_simulation": (ErrorStatus, [_P(BoundaryConditionParam), _P(System), _P(IntegratorParam),
                                        _P(StoringParam), _P(Settings), _P(SimulationParam),
                                        _P(SimulationStatus)]),
    "hydro_gpu_trim_device_memory": (C.c_int, [C.c_int]),
    "hydro_gpu_default_options": (HydroGpuOptions, []),
    "hydro_gpu_set_process_options": (None, [_P(HydroGpuOptions)]),
    "hydro_gpu_launch_simulation": (ErrorStatus, [_P(BoundaryConditionParam), _P(System),
                                                  _P(IntegratorParam), _P(StoringParam),
                                                  _P(Settings), _P(SimulationParam),
                                                  _P(SimulationStatus), _P(HydroGpuOptions),
                                                  _P(HydroGpuStats)]),
    "hydro_gpu_solver_create": (ErrorStatus, [_P(C.c_void_p), _P(BoundaryConditionParam), _P(System),
                                              _P(IntegratorParam), _P(HydroGpuOptions)]),
    "hydro_gpu_solver_restart": (ErrorStatus, [C.c_void_p]),
    "hydro_gpu_solver_advance": (ErrorStatus, [C.c_void_p, C.c_int64, C.c_double,
                                               _P(SimulationStatus), _P(C.c_double)]),
    "hydro_gpu_solver_download": (ErrorStatus, [C.c_void_p, _P(System)]),
    "hydro_gpu_solver_kernel_launches": (C.c_int64, [C.c_void_p]),
    "hydro_gpu_solver_conserved_totals": (ErrorStatus, [C.c_void_p, _dp]),
    "hydro_gpu_solver_destroy": (None, [C.c_void_p]),
    "hydro_gpu_batch_create": (ErrorStatus, [_P(C.c_void_p), C.c_int, C.c_void_p, C.c_void_p,
                                             _P(IntegratorParam), _P(HydroGpuOptions)]),
    "hydro_gpu_batch_restart": (ErrorStatus, [C.c_void_p]),
    "hydro_gpu_batch_advance": (ErrorStatus, [C.c_void_p, C.c_int64, C.c_double, C.c_void_p,
                                              _P(C.c_double)]),
    "hydro_gpu_batch_download": (ErrorStatus, [C.c_void_p, C.c_void_p]),
    "hydro_gpu_batch_kernel_launches": (C.c_int64, [C.c_void_p]),
    "hydro_gpu_batch_destroy": (None, [C.c_void_p]),
    "hydro_gpu_adjoint_create": (ErrorStatus, [_P(C.c_void_p), _P(BoundaryConditionParam), _P(System),
                                               _P(IntegratorParam), C.c_int64, C.c_int,
                                               _P(HydroGpuOptions)]),
    "hydro_gpu_adjoint_forward": (ErrorStatus, [C.c_void_p, C.c_void_p]),
    "hydro_gpu_adjoint_backward": (ErrorStatus, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "hydro_gpu_adjoint_tangent": (ErrorStatus, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                C.c_void_p]),
    "hydro_gpu_adjoint_replay": (ErrorStatus, [C.c_void_p, C.c_void_p, C.c_void_p,
                                               _P(C.c_uint64)]),
    "hydro_gpu_adjoint_replay_frozen": (ErrorStatus, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "hydro_gpu_adjoint_dt": (ErrorStatus, [C.c_void_p, _dp]),
    "hydro_gpu_adjoint_set_tape": (None, [C.c_void_p, C.c_int]),
    "hydro_gpu_adjoint_stats": (None, [C.c_void_p, _P(HydroGpuAdjointStats)]),
    "hydro_gpu_adjoint_destroy": (None, [C.c_void_p]),
    "hydro_ad_hllc_jvp": (C.c_int, [C.c_double, C.c_double] + [_dp] * 6),
    "hydro_ad_hllc_vjp": (C.c_int, [C.c_double, C.c_double] + [_dp] * 5 + [_P(C.c_int)]),
    "hydro_ad_recon_jvp": (None, [C.c_int, C.c_int, C.c_double, C.c_double] + [_dp] * 10),
    "hydro_ad_recon_vjp": (None, [C.c_int, C.c_int, C.c_double, C.c_double] + [_dp] * 8),
    "hydro_ad_hllc_forced": (None, [C.c_double, C.c_double, _dp, _dp, C.c_int, _dp]),
    "hydro_ad_recon_forced": (None, [C.c_int, C.c_int, C.c_double, C.c_double, _dp, _dp, _dp, C.c_int,
                                     _dp, _dp, _P(C.c_int)]),
    "hydro_fx_eval_host": (None, [C.c_int, C.c_longlong, _dp, _dp, _dp, C.c_void_p]),
    "hydro_gpu_fx_eval": (C.c_int, [C.c_int, C.c_int, C.c_longlong, _dp, _dp, _dp, _dp, C.c_void_p]),
    "hydro_fx_div_seeded_host": (None, [C.c_longlong, _dp, _dp, C.c_void_p, _dp, C.c_void_p]),
    "hydro_fx_ratio_below_host": (None, [C.c_longlong, _dp, _dp, _dp, C.c_void_p, C.c_void_p]),
    "hydro_fx_quot_le_host": (None, [C.c_longlong, _dp, _dp, _dp, C.c_void_p, C.c_void_p]),
    "hydro_gpu_pointwise_eval": (C.c_int, [C.c_int, C.c_int, C.c_longlong, _dp, C.c_double, _dp, _dp, _dp,
                                           _dp, _P(C.c_int)]),
    "hydro_gpu_device_count": (C.c_int, []),
    "hydro_gpu_calibrate": (C.c_int, [C.c_int, _dp, _dp]),
    "hydro_gpu_sm_count": (C.c_int, [C.c_int]),
    "hydro_gpu_chunk_plan": (C.c_int, [C.c_int] * 4 + [_P(C.c_int)] * 4 + [C.c_int]),
    "hydro_gpu_version": (C.c_char_p, []),
    "free_traceback": (None, [_P(ErrorStatus)]),
    "solve_flux_hllc_2d": (ErrorStatus, [_dp] * 4 + [C.c_double] * 10),
    "solve_flux_exact_1d": (ErrorStatus, [_dp] * 3 + [C.c_double] * 9 + [C.c_int]),
    "solve_flux_hllc_1d": (ErrorStatus, [_dp] * 3 + [C.c_double] * 8),
    "solve_exact_1d": (ErrorStatus, [_dp] * 3 + [C.c_double] * 9 + [C.c_int]),
    "guess_p": (C.c_double, [C.c_double] * 10),
    "limit_slope": (ErrorStatus, [_dp, _P(IntegratorParam), C.c_double, C.c_double]),
    "get_time_step_2d": (C.c_double, [_P(System), C.c_double]),
}

_lib: C.CDLL | None = None


def library(path: str | None = None) -> C.CDLL:
    """Load libhydro_gb300.so (raises FileNotFoundError if it was not built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise FileNotFoundError(
            f"{p} not found; build it with `python -m hydrofv_gb300.build` (needs nvcc)")
    lib = C.CDLL(p)
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class HydroError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code
        self.message = message


def _consume(lib: C.CDLL, e: ErrorStatus) -> tuple[int, str]:
    """Return (code, traceback text) and release the traceback."""
    msg = ""
    if e.traceback:
        msg = C.string_at(e.traceback).decode(errors="replace")
    lib.free_traceback(C.byref(e))
    return e.return_code, msg


def device_count() -> int:
    return int(library().hydro_gpu_device_count())


def sm_count(device: int = 0) -> int:
    """Streaming multiprocessors of the device (0 when it cannot be queried)."""
    return int(library().hydro_gpu_sm_count(device))


def calibrate(device: int = 0) -> tuple[float, float]:
    """Measured (FP64, FP32) FMA throughput in TFLOP/s."""
    f64, f32 = C.c_double(0), C.c_double(0)
    if library().hydro_gpu_calibrate(device, C.byref(f64), C.byref(f32)) != 0:
        raise HydroError(1, "calibration kernel failed")
    return f64.value, f32.value


def default_options(**kw) -> HydroGpuOptions:
    o = library().hydro_gpu_default_options()
    for k, v in kw.items():
        setattr(o, k, v)
    return o


@dataclass
class RunResult:
    code: int
    message: str
    W: np.ndarray
    U: np.ndarray
    num_steps: int
    t: float
    dt: float
    stats: dict = field(default_factory=dict)


def _stats_dict(st: HydroGpuStats) -> dict:
    return {name: getattr(st, name) for name, _ in HydroGpuStats._fields_}


class _SystemHandle:
    """A System allocated by system_init with W/U copied in from numpy."""

    def __init__(self, lib, coord_sys: str, nx: int, ny: int, g: int, bounds, gamma: float):
        self.lib = lib
        self._coord = coord_sys.encode()
        s = lib.get_new_system_struct()
        s.coord_sys = self._coord
        s.gamma = gamma
        s.x_min, s.x_max = bounds[0], bounds[1]
        if ny > 0:
            s.y_min, s.y_max = bounds[2], bounds[3]
            s.num_cells_y = ny
        s.num_cells_x = nx
        s.num_ghost_cells_side = g
        code, msg = _consume(lib, lib.system_init(C.byref(s)))
        if code != 0:
            raise HydroError(code, msg)
        self.s = s
        self.n = (nx + 2 * g) * ((ny + 2 * g) if ny > 0 else 1)
        self.shape = ((ny + 2 * g), (nx + 2 * g)) if ny > 0 else ((nx + 2 * g),)

    def fields(self, names):
        return [np.ctypeslib.as_array(getattr(self.s, n), shape=(self.n,)) for n in names]

    def close(self):
        if self.s is not None:
            self.lib.free_system_memory(C.byref(self.s))
            self.s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


W2 = ("density_", "velocity_x_", "velocity_y_", "pressure_")
U2 = ("mass_", "momentum_x_", "momentum_y_", "energy_")
W1 = ("density_", "velocity_x_", "pressure_")
U1 = ("mass_", "momentum_x_", "energy_")


def _params(lib, bc, integrator, riemann_solver, slope_limiter, cfl, keep):
    bcp = lib.get_new_boundary_condition_param()
    names = ["x_min", "x_max", "y_min", "y_max"]
    for k, b in enumerate(bc):
        enc = b.encode() if b is not None else None
        keep.append(enc)
        setattr(bcp, "boundary_condition_" + names[k], enc)
    ip = lib.get_new_integrator_param()
    for attr, val in (("integrator", integrator), ("riemann_solver", riemann_solver),
                      ("slope_limiter", slope_limiter)):
        enc = val.encode() if val is not None else None
        keep.append(enc)
        setattr(ip, attr, enc)
    ip.cfl = cfl
    return bcp, ip


def _set_custom(bcp, custom_bc, keep):
    """Install BcCallback objects for the custom sides (kept alive in keep)."""
    names = ("x_min", "x_max", "y_min", "y_max")
    for side, cb in zip(names, custom_bc or (None,) * 4):
        if cb is not None:
            keep.append(cb)
            setattr(bcp, "set_boundary_condition_cartesian_2d_" + side, C.cast(cb, C.c_void_p).value)


class Simulation2D:
    """A 2D problem held in the reference's structs -- a System allocated by
    system_init with the padded W and U in its host arrays, and the boundary,
    integrator, storing, settings and simulation parameters -- launched
    through the drop-in entry point, hydro_gpu_launch_simulation (the host
    arrays in and out, host<->device copies inside the call).  W and U are
    (4, ny+2g, nx+2g) float64 arrays (rho,u,v,p / mass,mom_x,mom_y,energy);
    gravity sets System.gravity; custom_bc gives a problems.BcCallback per
    side whose boundary name is "custom"."""

    def __init__(self, nx: int, ny: int, g: int, bounds, gamma: float, W: np.ndarray, U: np.ndarray,
                 bc=("periodic",) * 4, integrator="muscl_hancock_2d",
                 riemann_solver="riemann_solver_hllc", slope_limiter="monotonized_central",
                 cfl=0.8, tf=1.0, max_steps=-1, options: HydroGpuOptions | None = None,
                 storing: dict | None = None, gravity: float = 0.0, custom_bc=None):
        lib = self.lib = library()
        self.h = _SystemHandle(lib, "cartesian_2d", nx, ny, g, bounds, gamma)
        self.h.s.gravity = gravity
        self._W0, self._U0 = W, U
        self.load(W, U)
        keep: list = []
        self._keep = keep
        self.bcp, self.ip = _params(lib, bc, integrator, riemann_solver, slope_limiter, cfl, keep)
        _set_custom(self.bcp, custom_bc, keep)
        sp = lib.get_new_storing_param()
        if storing:
            sp.is_storing = True
            sp.store_initial = bool(storing.get("store_initial", False))
            sp.storing_interval = float(storing["interval"])
            d = storing["output_dir"].encode()
            keep.append(d)
            sp.output_dir = d
        self.sp = sp
        self.settings = Settings(0, True)
        self.simp = SimulationParam(tf)
        self.opt = options if options is not None else lib.hydro_gpu_default_options()
        if max_steps is not None and max_steps >= 0:
            self.opt.max_steps = max_steps

    def load(self, W: np.ndarray, U: np.ndarray) -> None:
        """Copy a padded state into the System's host arrays."""
        for dst, src in zip(self.h.fields(W2), W):
            dst[:] = np.ascontiguousarray(src, dtype=np.float64).reshape(-1)
        for dst, src in zip(self.h.fields(U2), U):
            dst[:] = np.ascontiguousarray(src, dtype=np.float64).reshape(-1)

    def launch(self) -> tuple[int, str, SimulationStatus, dict]:
        """One hydro_gpu_launch_simulation call on the System as it stands:
        (code, message, status, stats).  The System's arrays hold the final
        state afterwards."""
        st = SimulationStatus(0, 0.0, 0.0)
        stats = HydroGpuStats()
        code, msg = _consume(self.lib, self.lib.hydro_gpu_launch_simulation(
            C.byref(self.bcp), C.byref(self.h.s), C.byref(self.ip), C.byref(self.sp),
            C.byref(self.settings), C.byref(self.simp), C.byref(st), C.byref(self.opt), C.byref(stats)))
        return code, msg, st, _stats_dict(stats)

    def result(self, code, msg, st, stats) -> RunResult:
        Wout = np.stack([f.copy() for f in self.h.fields(W2)]).reshape((4,) + self.h.shape)
        Uout = np.stack([f.copy() for f in self.h.fields(U2)]).reshape((4,) + self.h.shape)
        return RunResult(code, msg, Wout, Uout, st.num_steps, st.t, st.dt, stats)

    def close(self) -> None:
        self.h.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def run_2d(nx: int, ny: int, g: int, bounds, gamma: float, W: np.ndarray, U: np.ndarray,
           bc=("periodic",) * 4, integrator="muscl_hancock_2d",
           riemann_solver="riemann_solver_hllc", slope_limiter="monotonized_central",
           cfl=0.8, tf=1.0, max_steps=-1, options: HydroGpuOptions | None = None,
           storing: dict | None = None, gravity: float = 0.0, custom_bc=None) -> RunResult:
    """Run a 2D problem through hydro_gpu_launch_simulation (see
    Simulation2D) and return the final state."""
    with Simulation2D(nx, ny, g, bounds, gamma, W, U, bc=bc, integrator=integrator,
                      riemann_solver=riemann_solver, slope_limiter=slope_limiter, cfl=cfl, tf=tf,
                      max_steps=max_steps, options=options, storing=storing, gravity=gravity,
                      custom_bc=custom_bc) as sim:
        return sim.result(*sim.launch())


def run_1d(nx: int, g: int, bounds, gamma: float, W: np.ndarray, U: np.ndarray,
           bc=("transmissive", "transmissive"), integrator="godunov_first_order_1d",
           riemann_solver="riemann_solver_exact", slope_limiter="minmod", cfl=0.9, tf=0.2,
           max_steps=-1, options: HydroGpuOptions | None = None,
           coord_sys: str = "cartesian_1d", storing: dict | None = None,
           verbose: int = 0) -> RunResult:
    """Run a 1D problem (W, U: (3, nx+2g)) on a cartesian_1d, cylindrical_1d
    or spherical_1d grid.  storing: {"interval", "output_dir",
    "store_initial"} turns snapshots on, as for the 2D runs; verbose is
    Settings.verbose (> 0: the exact solver's bisection warnings)."""
    lib = library()
    h = _SystemHandle(lib, coord_sys, nx, 0, g, bounds, gamma)
    try:
        for dst, src in zip(h.fields(W1), W):
            dst[:] = src
        for dst, src in zip(h.fields(U1), U):
            dst[:] = src
        keep: list = []
        bcp, ip = _params(lib, list(bc) + [None, None], integrator, riemann_solver,
                          slope_limiter, cfl, keep)
        sp = lib.get_new_storing_param()
        if storing:
            sp.is_storing = True
            sp.store_initial = bool(storing.get("store_initial", False))
            sp.storing_interval = float(storing["interval"])
            d = storing["output_dir"].encode()
            keep.append(d)
            sp.output_dir = d
        settings = Settings(verbose, True)
        simp = SimulationParam(tf)
        st = SimulationStatus(0, 0.0, 0.0)
        opt = options if options is not None else lib.hydro_gpu_default_options()
        if max_steps is not None and max_steps >= 0:
            opt.max_steps = max_steps
        stats = HydroGpuStats()
        code, msg = _consume(lib, lib.hydro_gpu_launch_simulation(
            C.byref(bcp), C.byref(h.s), C.byref(ip), C.byref(sp), C.byref(settings),
            C.byref(simp), C.byref(st), C.byref(opt), C.byref(stats)))
        Wout = np.stack([f.copy() for f in h.fields(W1)])
        Uout = np.stack([f.copy() for f in h.fields(U1)])
        return RunResult(code, msg, Wout, Uout, st.num_steps, st.t, st.dt, _stats_dict(stats))
    finally:
        h.close()


class Solver2D:
    """Device-resident session (hydro_gpu_solver_*): upload once, step many
    times with the state kept in HBM."""

    def __init__(self, nx, ny, g, bounds, gamma, W, U, bc=("periodic",) * 4,
                 slope_limiter="monotonized_central", cfl=0.8,
                 options: HydroGpuOptions | None = None, gravity: float = 0.0, custom_bc=None):
        self.lib = lib = library()
        self._h = _SystemHandle(lib, "cartesian_2d", nx, ny, g, bounds, gamma)
        self._h.s.gravity = gravity
        for dst, src in zip(self._h.fields(W2), W):
            dst[:] = np.ascontiguousarray(src).reshape(-1)
        for dst, src in zip(self._h.fields(U2), U):
            dst[:] = np.ascontiguousarray(src).reshape(-1)
        self._keep: list = []
        bcp, ip = _params(lib, bc, "muscl_hancock_2d", "riemann_solver_hllc", slope_limiter,
                          cfl, self._keep)
        _set_custom(bcp, custom_bc, self._keep)
        self._bcp, self._ip = bcp, ip
        opt = options if options is not None else lib.hydro_gpu_default_options()
        self.handle = C.c_void_p()
        code, msg = _consume(lib, lib.hydro_gpu_solver_create(
            C.byref(self.handle), C.byref(bcp), C.byref(self._h.s), C.byref(ip), C.byref(opt)))
        if code != 0:
            raise HydroError(code, msg)
        self.cells = nx * ny

    def restart(self):
        code, msg = _consume(self.lib, self.lib.hydro_gpu_solver_restart(self.handle))
        if code != 0:
            raise HydroError(code, msg)

    def advance(self, steps: int, tf: float = 1e300) -> tuple[SimulationStatus, float]:
        st = SimulationStatus(0, 0.0, 0.0)
        ms = C.c_double(0.0)
        code, msg = _consume(self.lib, self.lib.hydro_gpu_solver_advance(
            self.handle, steps, tf, C.byref(st), C.byref(ms)))
        if code != 0:
            raise HydroError(code, msg)
        return st, ms.value

    def download(self) -> tuple[np.ndarray, np.ndarray]:
        code, msg = _consume(self.lib, self.lib.hydro_gpu_solver_download(self.handle,
                                                                          C.byref(self._h.s)))
        if code != 0:
            raise HydroError(code, msg)
        W = np.stack([f.copy() for f in self._h.fields(W2)]).reshape((4,) + self._h.shape)
        U = np.stack([f.copy() for f in self._h.fields(U2)]).reshape((4,) + self._h.shape)
        return W, U

    def conserved_totals(self) -> np.ndarray:
        """(mass, mom_x, mom_y, energy) over the interior, FP64 compensated sums."""
        out = np.zeros(4)
        code, msg = _consume(self.lib, self.lib.hydro_gpu_solver_conserved_totals(
            self.handle, out.ctypes.data_as(_dp)))
        if code != 0:
            raise HydroError(code, msg)
        return out

    def kernel_launches(self) -> int:
        return int(self.lib.hydro_gpu_solver_kernel_launches(self.handle))

    def close(self):
        if self.handle:
            self.lib.hydro_gpu_solver_destroy(self.handle)
            self.handle = C.c_void_p()
        self._h.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Batch2D:
    """Ensemble of independent 2D problems (hydro_gpu_batch_*): one launch per
    step for all instances, each with its own dt.  `problems` are objects with
    the fields of hydrofv_gb300.problems.Problem2D; integrator, limiter and CFL
    are taken from the first one."""

    def __init__(self, problems, options: HydroGpuOptions | None = None):
        self.lib = lib = library()
        self.n = len(problems)
        self._handles = []
        self._keep: list = []
        systems = (System * self.n)()
        bcps = (BoundaryConditionParam * self.n)()
        p0 = problems[0]
        for i, p in enumerate(problems):
            h = _SystemHandle(lib, "cartesian_2d", p.nx, p.ny, p.g,
                              (p.x_min, p.x_max, p.y_min, p.y_max), p.gamma)
            for dst, src in zip(h.fields(W2), p.W):
                dst[:] = np.ascontiguousarray(src).reshape(-1)
            for dst, src in zip(h.fields(U2), p.U):
                dst[:] = np.ascontiguousarray(src).reshape(-1)
            self._handles.append(h)
            systems[i] = h.s
            bcp, _ = _params(lib, p.bc, p0.integrator, p0.riemann_solver, p0.slope_limiter,
                             p0.cfl, self._keep)
            bcps[i] = bcp
        self._systems, self._bcps = systems, bcps
        _, ip = _params(lib, p0.bc, p0.integrator, p0.riemann_solver, p0.slope_limiter, p0.cfl,
                        self._keep)
        self._ip = ip
        opt = options if options is not None else lib.hydro_gpu_default_options()
        self.handle = C.c_void_p()
        code, msg = _consume(lib, lib.hydro_gpu_batch_create(
            C.byref(self.handle), self.n, C.cast(bcps, C.c_void_p),
            C.cast(systems, C.c_void_p), C.byref(ip), C.byref(opt)))
        if code != 0:
            raise HydroError(code, msg)
        self.cells = sum(p.nx * p.ny for p in problems)
        self.shapes = [h.shape for h in self._handles]

    def restart(self):
        code, msg = _consume(self.lib, self.lib.hydro_gpu_batch_restart(self.handle))
        if code != 0:
            raise HydroError(code, msg)

    def advance(self, steps: int, tf: float = 1e300):
        st = (SimulationStatus * self.n)()
        ms = C.c_double(0.0)
        code, msg = _consume(self.lib, self.lib.hydro_gpu_batch_advance(
            self.handle, steps, tf, C.cast(st, C.c_void_p), C.byref(ms)))
        if code != 0:
            raise HydroError(code, msg)
        return [(s.num_steps, s.t, s.dt) for s in st], ms.value

    def download(self):
        code, msg = _consume(self.lib, self.lib.hydro_gpu_batch_download(
            self.handle, C.cast(self._systems, C.c_void_p)))
        if code != 0:
            raise HydroError(code, msg)
        out = []
        for i, h in enumerate(self._handles):
            h.s = self._systems[i]
            W = np.stack([f.copy() for f in h.fields(W2)]).reshape((4,) + h.shape)
            U = np.stack([f.copy() for f in h.fields(U2)]).reshape((4,) + h.shape)
            out.append((W, U))
        return out

    def kernel_launches(self) -> int:
        return int(self.lib.hydro_gpu_batch_kernel_launches(self.handle))

    def close(self):
        if self.handle:
            self.lib.hydro_gpu_batch_destroy(self.handle)
            self.handle = C.c_void_p()
        for i, h in enumerate(self._handles):
            h.s = self._systems[i]
            h.close()
        self._handles = []

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


# ---------------------------------------------------------------- adjoint

def _ptr4(arrs):
    """(double*)[4] array of pointers to four contiguous float64 arrays."""
    t = (_dp * 4)()
    for k, a in enumerate(arrs):
        t[k] = a.ctypes.data_as(_dp)
    return t


class Adjoint2D:
    """Discrete adjoint / tangent-linear session (hydro_gpu_adjoint_*) of the
    2D MUSCL-Hancock + HLLC step: forward pass with checkpoints every
    `checkpoint_every` steps, reverse pass, tangent-linear model and frozen-dt
    replay.  Field arrays are (4, ny + 2G, nx + 2G) float64 in the order
    (rho, vx, vy, p); interior entries are read, ghost entries of outputs
    are 0."""

    def __init__(self, problem, steps: int, checkpoint_every: int,
                 options: HydroGpuOptions | None = None):
        self.lib = lib = library()
        p = problem
        self.shape = (4, p.ny + 2 * p.g, p.nx + 2 * p.g)
        self.steps = int(steps)
        self._h = _SystemHandle(lib, "cartesian_2d", p.nx, p.ny, p.g,
                                (p.x_min, p.x_max, p.y_min, p.y_max), p.gamma)
        for dst, src in zip(self._h.fields(W2), p.W):
            dst[:] = np.ascontiguousarray(src).reshape(-1)
        for dst, src in zip(self._h.fields(U2), p.U):
            dst[:] = np.ascontiguousarray(src).reshape(-1)
        self._keep: list = []
        bcp, ip = _params(lib, p.bc, p.integrator, p.riemann_solver, p.slope_limiter, p.cfl,
                          self._keep)
        self._bcp, self._ip = bcp, ip
        opt = options if options is not None else lib.hydro_gpu_default_options()
        self.handle = C.c_void_p()
        code, msg = _consume(lib, lib.hydro_gpu_adjoint_create(
            C.byref(self.handle), C.byref(bcp), C.byref(self._h.s), C.byref(ip), self.steps,
            int(checkpoint_every), C.byref(opt)))
        if code != 0:
            raise HydroError(code, msg)

    def _check(self, e):
        code, msg = _consume(self.lib, e)
        if code != 0:
            raise HydroError(code, msg)

    def _empty(self):
        return np.zeros(self.shape)

    def _in(self, W):
        W = np.ascontiguousarray(W, dtype=np.float64)
        if W.shape != self.shape:
            raise ValueError(f"expected shape {self.shape}, got {W.shape}")
        return W

    def forward(self) -> np.ndarray:
        """Run the forward pass; returns W^N (interior)."""
        out = self._empty()
        self._check(self.lib.hydro_gpu_adjoint_forward(self.handle, _ptr4(out)))
        return out

    def backward(self, seed: np.ndarray) -> np.ndarray:
        """dJ/dW0 for seed = dJ/dW^N."""
        seed = self._in(seed)
        grad = self._empty()
        self._check(self.lib.hydro_gpu_adjoint_backward(self.handle, _ptr4(seed), _ptr4(grad)))
        return grad

    def tangent(self, dw0: np.ndarray, w0: np.ndarray | None = None):
        """(W^N, dW^N) of the tangent-linear model in direction dw0."""
        dw0 = self._in(dw0)
        wN, dwN = self._empty(), self._empty()
        w0p = _ptr4(self._in(w0)) if w0 is not None else None
        self._keep_w0 = w0
        self._check(self.lib.hydro_gpu_adjoint_tangent(self.handle, w0p, _ptr4(dw0), _ptr4(wN),
                                                       _ptr4(dwN)))
        return wN, dwN

    def replay(self, w0: np.ndarray, signatures: bool = True):
        """(W^N, per-step branch signatures) of the frozen-dt replay from w0."""
        w0 = self._in(w0)
        wN = self._empty()
        sig = np.zeros(self.steps, dtype=np.uint64) if signatures else None
        sp = sig.ctypes.data_as(C.POINTER(C.c_uint64)) if sig is not None else None
        self._check(self.lib.hydro_gpu_adjoint_replay(self.handle, _ptr4(w0), _ptr4(wN), sp))
        return wN, sig

    def replay_frozen(self, w0: np.ndarray) -> np.ndarray:
        """W^N of the replay from w0 with the forward pass's dt AND branch
        decisions forced (the map the adjoint differentiates)."""
        w0 = self._in(w0)
        wN = self._empty()
        self._check(self.lib.hydro_gpu_adjoint_replay_frozen(self.handle, _ptr4(w0), _ptr4(wN)))
        return wN

    def set_tape(self, enabled: bool):
        """Tape the segment recomputation (default) or recompute in the sweep."""
        self.lib.hydro_gpu_adjoint_set_tape(self.handle, 1 if enabled else 0)

    def dt(self) -> np.ndarray:
        out = np.zeros(self.steps)
        self._check(self.lib.hydro_gpu_adjoint_dt(self.handle, out.ctypes.data_as(_dp)))
        return out

    def stats(self) -> dict:
        st = HydroGpuAdjointStats()
        self.lib.hydro_gpu_adjoint_stats(self.handle, C.byref(st))
        return {name: getattr(st, name) for name, _ in HydroGpuAdjointStats._fields_}

    def close(self):
        if self.handle:
            self.lib.hydro_gpu_adjoint_destroy(self.handle)
            self.handle = C.c_void_p()
        self._h.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def _vec(x):
    return np.ascontiguousarray(x, dtype=np.float64).reshape(4)


def ad_hllc_jvp(gamma, tol, L, R, dL, dR):
    """(F, dF, code) of the HLLC 2D flux in tangent mode (host build)."""
    F, dF = np.zeros(4), np.zeros(4)
    args = [_vec(a) for a in (L, R, dL, dR)]
    rc = library().hydro_ad_hllc_jvp(gamma, tol, *[a.ctypes.data_as(_dp) for a in args],
                                     F.ctypes.data_as(_dp), dF.ctypes.data_as(_dp))
    return F, dF, rc


def ad_hllc_vjp(gamma, tol, L, R, Fb):
    """(Lb, Rb, rc, branch code) of the HLLC 2D flux in reverse mode (host build)."""
    Lb, Rb = np.zeros(4), np.zeros(4)
    code = C.c_int(0)
    args = [_vec(a) for a in (L, R, Fb)]
    rc = library().hydro_ad_hllc_vjp(gamma, tol, *[a.ctypes.data_as(_dp) for a in args],
                                     Lb.ctypes.data_as(_dp), Rb.ctypes.data_as(_dp), C.byref(code))
    return Lb, Rb, rc, code.value


def ad_recon_jvp(limiter, direction, gamma, dtA, wm, w0, wp, dwm, dw0, dwp):
    """(lo, hi, dlo, dhi) of one cell's reconstruction in tangent mode."""
    outs = [np.zeros(4) for _ in range(4)]
    args = [_vec(a) for a in (wm, w0, wp, dwm, dw0, dwp)]
    library().hydro_ad_recon_jvp(limiter, direction, gamma, dtA,
                                 *[a.ctypes.data_as(_dp) for a in args],
                                 *[o.ctypes.data_as(_dp) for o in outs])
    return tuple(outs)


def ad_recon_vjp(limiter, direction, gamma, dtA, wm, w0, wp, lob, hib):
    """(wmb, w0b, wpb) of one cell's reconstruction in reverse mode."""
    outs = [np.zeros(4) for _ in range(3)]
    args = [_vec(a) for a in (wm, w0, wp, lob, hib)]
    library().hydro_ad_recon_vjp(limiter, direction, gamma, dtA,
                                 *[a.ctypes.data_as(_dp) for a in args],
                                 *[o.ctypes.data_as(_dp) for o in outs])
    return tuple(outs)


def ad_hllc_forced(gamma, tol, L, R, code):
    """HLLC 2D flux with the branch code given (host build)."""
    F = np.zeros(4)
    L, R = _vec(L), _vec(R)
    library().hydro_ad_hllc_forced(gamma, tol, L.ctypes.data_as(_dp), R.ctypes.data_as(_dp), int(code),
                                   F.ctypes.data_as(_dp))
    return F


def ad_recon_forced(limiter, direction, gamma, dtA, wm, w0, wp, code):
    """(lo, hi, natural code) of one cell's reconstruction with the limiter cases given."""
    lo, hi = np.zeros(4), np.zeros(4)
    nat = C.c_int(0)
    args = [_vec(a) for a in (wm, w0, wp)]
    library().hydro_ad_recon_forced(limiter, direction, gamma, dtA, *[a.ctypes.data_as(_dp) for a in args],
                                    int(code), lo.ctypes.data_as(_dp), hi.ctypes.data_as(_dp), C.byref(nat))
    return lo, hi, nat.value


def _fx_args(op, a, b):
    """Operands of the fx evaluations (op 1, sqrt, takes a alone)."""
    a = np.ascontiguousarray(a, dtype=np.float64).ravel()
    b = a if op == 1 else np.ascontiguousarray(b, dtype=np.float64).ravel()
    if b.shape != a.shape:
        raise ValueError("a and b must have the same size")
    return a, b


def fx_eval_host(op, a, b=None):
    """Integer-pipe FP64 division (op 0: a / b), square root (op 1:
    sqrt(a)) or power (op 2: pow(a, b)), host build: (results, fast-path
    flags)."""
    a, b = _fx_args(op, a, b)
    out = np.empty_like(a)
    ok = np.zeros(a.shape, dtype=np.uint8)
    library().hydro_fx_eval_host(int(op), a.size, a.ctypes.data_as(_dp), b.ctypes.data_as(_dp),
                                 out.ctypes.data_as(_dp), ok.ctypes.data)
    return out, ok.astype(bool)


def gpu_fx_eval(op, a, b=None, device=0):
    """The same on the GPU: (what the FP64 kernels compute, the hardware
    operation, fast-path flags)."""
    a, b = _fx_args(op, a, b)
    fast, hw = np.empty_like(a), np.empty_like(a)
    ok = np.zeros(a.shape, dtype=np.uint8)
    rc = library().hydro_gpu_fx_eval(int(device), int(op), a.size, a.ctypes.data_as(_dp),
                                     b.ctypes.data_as(_dp), fast.ctypes.data_as(_dp),
                                     hw.ctypes.data_as(_dp), ok.ctypes.data)
    if rc != 0:
        raise HydroError(rc, "hydro_gpu_fx_eval failed (CUDA error)")
    return fast, hw, ok.astype(bool)


def chunk_plan(nx, ny, g=2, slots=608):
    """The FP64 step's work-item plan: ((h1, h2, tail), rows) with rows an
    (n_items, 3) array of (strip, r0, r1) as the kernel decodes the items."""
    lib = library()
    h1, h2, tail = C.c_int(), C.c_int(), C.c_int()
    n = lib.hydro_gpu_chunk_plan(nx, ny, g, slots, C.byref(h1), C.byref(h2), C.byref(tail), None, 0)
    rows = np.zeros((n, 3), dtype=np.int32)
    lib.hydro_gpu_chunk_plan(nx, ny, g, slots, C.byref(h1), C.byref(h2), C.byref(tail),
                             rows.ctypes.data_as(_P(C.c_int)), n)
    return (h1.value, h2.value, tail.value), rows


def fx_ratio_below_host(x, y, tol):
    """The exact solver's convergence test RN(x / y) < tol decided without the
    divide (host build): (answers, decided flags)."""
    x = np.ascontiguousarray(x, dtype=np.float64).ravel()
    y = np.ascontiguousarray(np.broadcast_to(y, x.shape), dtype=np.float64).ravel()
    t = np.ascontiguousarray(np.broadcast_to(tol, x.shape), dtype=np.float64).ravel()
    out = np.zeros(x.size, dtype=np.uint8)
    dec = np.zeros(x.size, dtype=np.uint8)
    library().hydro_fx_ratio_below_host(x.size, x.ctypes.data_as(_dp), y.ctypes.data_as(_dp),
                                        t.ctypes.data_as(_dp), out.ctypes.data, dec.ctypes.data)
    return out.astype(bool), dec.astype(bool)


def fx_quot_le_host(x, y, z):
    """The solvers' vacuum-generation test RN(x / y) <= z decided without the
    divide (host build): (answers, decided flags)."""
    x = np.ascontiguousarray(x, dtype=np.float64).ravel()
    y = np.ascontiguousarray(np.broadcast_to(y, x.shape), dtype=np.float64).ravel()
    z = np.ascontiguousarray(np.broadcast_to(z, x.shape), dtype=np.float64).ravel()
    out = np.zeros(x.size, dtype=np.uint8)
    dec = np.zeros(x.size, dtype=np.uint8)
    library().hydro_fx_quot_le_host(x.size, x.ctypes.data_as(_dp), y.ctypes.data_as(_dp),
                                    z.ctypes.data_as(_dp), out.ctypes.data, dec.ctypes.data)
    return out.astype(bool), dec.astype(bool)


POINTWISE_OPS = {"hllc_2d": (0, 4), "guess_p": (1, 1), "exact_flux_1d": (2, 3), "hllc_1d": (3, 3),
                 "exact_1d": (4, 3), "exact_flux_1d_quad": (5, 3), "exact_1d_quad": (6, 3)}


def gpu_pointwise_eval(name, gamma, L, R, aux=None, tol=1e-6, device=0):
    """Device build of an exported pointwise function over n state pairs
    (L, R: (n, 4) arrays of rho, u, v, p; gamma: (n,)): (outputs, return
    codes).  name: "hllc_2d", "hllc_1d", "guess_p" (aux = (n, 2) sound
    speeds a_L, a_R), "exact_flux_1d" or "exact_1d" (aux = (n,) sample
    speeds), or "exact_flux_1d_quad" / "exact_1d_quad" (the same, as the 1D
    kernel computes them with four lanes per state pair).  Return codes: 0, 1 (HLLC wave speed), 3 or 4 (exact solver)."""
    op, width = POINTWISE_OPS[name]
    g = np.ascontiguousarray(gamma, dtype=np.float64).ravel()
    n = g.size
    L = np.ascontiguousarray(L, dtype=np.float64).reshape(n, 4)
    R = np.ascontiguousarray(R, dtype=np.float64).reshape(n, 4)
    need = {1: 2, 2: 1, 4: 1, 5: 1, 6: 1}.get(op, 0)
    a = np.ascontiguousarray(np.zeros(n * max(need, 1)) if aux is None else aux, dtype=np.float64).ravel()
    if a.size < n * need:
        raise ValueError(f"{name} needs {need} auxiliary values per state pair")
    out = np.empty(n * width)
    rc = np.empty(n, dtype=np.int32)
    code = library().hydro_gpu_pointwise_eval(int(device), op, n, g.ctypes.data_as(_dp), float(tol),
                                              L.ctypes.data_as(_dp), R.ctypes.data_as(_dp),
                                              a.ctypes.data_as(_dp), out.ctypes.data_as(_dp),
                                              rc.ctypes.data_as(_P(C.c_int)))
    if code != 0:
        raise HydroError(code, "hydro_gpu_pointwise_eval failed (CUDA error)")
    return (out if width == 1 else out.reshape(n, width)), rc


def fx_div_seeded_host(a, b, seed_scale):
    """Host build of the integer division with its FP32 reciprocal seed
    scaled by seed_scale: (results, fast-path flags)."""
    a, b = _fx_args(0, a, b)
    sc = np.ascontiguousarray(seed_scale, dtype=np.float32).ravel()
    if sc.shape != a.shape:
        raise ValueError("seed_scale must have the size of a")
    out = np.empty_like(a)
    ok = np.zeros(a.shape, dtype=np.uint8)
    library().hydro_fx_div_seeded_host(a.size, a.ctypes.data_as(_dp), b.ctypes.data_as(_dp), sc.ctypes.data,
                                       out.ctypes.data_as(_dp), ok.ctypes.data)
    return out, ok.astype(bool)
