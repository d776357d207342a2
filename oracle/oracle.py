"""ctypes front-end for the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
import this module.  It loads

* ``oracle/_build/liboracle.so`` -- this project's C restatement of the
  hydroFV algorithm (``oracle/hydro_oracle.c``), and
* ``oracle/_ref/libhydro_ref_{omp,serial}.so`` -- the unmodified reference
  sources built by ``make -C oracle ref`` (present only where the reference
  tree was available at build time),

and offers one ``run_2d`` / ``run_1d`` call shape for both, plus the seeded
initial-condition generators used by the parity tests and the benchmark.
"""
from __future__ import annotations

import ctypes as C
import os
import sys
import subprocess
import time
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if os.path.dirname(HERE) not in sys.path:
    sys.path.insert(0, os.path.dirname(HERE))
BUILD = os.path.join(HERE, "_build")
REFDIR = os.path.join(HERE, "_ref")

_dp = C.POINTER(C.c_double)
_i64p = C.POINTER(C.c_longlong)


# The reference's sources as `make stage` copies them (git-ignored; present
# wherever the reference tree was, or wherever the working tree was carried).
REF_SRC = os.path.join(REFDIR, "src")
REF_EXAMPLES = os.path.join(REFDIR, "examples")


def build(with_reference: bool | None = None) -> None:
    """Compile the restatement, stage the reference's sources where its tree
    exists, and compile the reference from the staged copy when there is one.
    HYDRO_REF_ROOT names another reference tree to stage from."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    stage = ["make", "-s", "-C", HERE, "stage"]
    if os.environ.get("HYDRO_REF_ROOT"):
        stage.append("REF_ROOT=" + os.environ["HYDRO_REF_ROOT"])
    subprocess.run(stage, check=True)
    if with_reference is None:
        with_reference = os.path.isdir(REF_SRC)
    if with_reference:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


_libs: dict[str, C.CDLL] = {}


def _bind(lib: C.CDLL, prefix: str) -> C.CDLL:
    f = getattr(lib, prefix + "run_2d")
    f.restype = C.c_int
    f.argtypes = ([C.c_int] * 3 + [C.c_double] * 5 + [C.c_char_p] * 7
                  + [C.c_double, C.c_double, C.c_longlong] + [_dp] * 8
                  + [_i64p, _dp, _dp, C.c_char_p, C.c_int])
    f = getattr(lib, prefix + "run_2d_ex")
    f.restype = C.c_int
    f.argtypes = ([C.c_int] * 3 + [C.c_double] * 5 + [C.c_char_p] * 7
                  + [C.c_double, C.c_double, C.c_longlong] + [_dp] * 8
                  + [_i64p, _dp, _dp, C.c_char_p, C.c_int] + [C.c_double] + [C.c_void_p] * 4)
    f = getattr(lib, prefix + "run_1d")
    f.restype = C.c_int
    f.argtypes = ([C.c_int] * 2 + [C.c_double] * 3 + [C.c_char_p] * 5
                  + [C.c_double, C.c_double, C.c_longlong] + [_dp] * 6
                  + [_i64p, _dp, _dp, C.c_char_p, C.c_int])
    f = getattr(lib, prefix + "run_1d_ex")
    f.restype = C.c_int
    f.argtypes = ([C.c_int] * 2 + [C.c_double] * 3 + [C.c_char_p] * 5
                  + [C.c_double, C.c_double, C.c_longlong] + [_dp] * 6
                  + [_i64p, _dp, _dp, C.c_char_p, C.c_int, C.c_char_p])
    f = getattr(lib, prefix + "hllc_2d")
    f.restype = C.c_int
    f.argtypes = [C.c_double] * 10 + [_dp]
    f = getattr(lib, prefix + "exact_flux_1d")
    f.restype = C.c_int
    f.argtypes = [C.c_double] * 9 + [_dp]
    f = getattr(lib, prefix + "hllc_1d")
    f.restype = C.c_int
    f.argtypes = [C.c_double] * 8 + [_dp]
    f = getattr(lib, prefix + "exact_1d")
    f.restype = C.c_int
    f.argtypes = [C.c_double] * 9 + [_dp]
    f = getattr(lib, prefix + "guess_p")
    f.restype = C.c_double
    f.argtypes = [C.c_double] * 10
    f = getattr(lib, prefix + "limit_slope")
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_double, C.c_double, _dp]
    f = getattr(lib, prefix + "geometry_source_1d")
    f.restype = C.c_int
    f.argtypes = [C.c_int] * 3 + [C.c_double] * 4 + [C.c_char_p] * 2 + [_dp] * 6
    f = getattr(lib, prefix + "gravity_source_2d")
    f.restype = C.c_int
    f.argtypes = [C.c_int] * 3 + [C.c_double] * 7 + [C.c_char_p] * 4 + [_dp] * 8
    if prefix == "ref_":
        lib.ref_set_verbose.restype = None
        lib.ref_set_verbose.argtypes = [C.c_int]
    f = getattr(lib, prefix + "exact_status")
    f.restype = C.c_int
    f.argtypes = [C.c_double] * 8 + [C.c_char_p, C.c_int]
    return lib


def load(kind: str = "oracle") -> "Backend":
    """kind: 'oracle' (restatement), 'ref' (reference, OpenMP) or 'ref_serial'."""
    if kind not in _libs:
        path = {
            "oracle": os.path.join(BUILD, "liboracle.so"),
            "ref": os.path.join(REFDIR, "libhydro_ref_omp.so"),
            "ref_serial": os.path.join(REFDIR, "libhydro_ref_serial.so"),
        }[kind]
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        lib = C.CDLL(path)
        _libs[kind] = _bind(lib, "oracle_" if kind == "oracle" else "ref_")
    return Backend(_libs[kind], "oracle_" if kind == "oracle" else "ref_")


def reference_available() -> bool:
    return os.path.exists(os.path.join(REFDIR, "libhydro_ref_omp.so"))


@dataclass
class Result:
    rc: int
    W: np.ndarray
    U: np.ndarray
    num_steps: int
    t: float
    dt: float
    message: str = ""
    seconds: float = 0.0


def _ptr(a: np.ndarray) -> C.POINTER(C.c_double):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


class Backend:
    def __init__(self, lib: C.CDLL, prefix: str):
        self.lib = lib
        self.prefix = prefix

    def run_2d(self, prob: Problem2D) -> Result:
        W = np.ascontiguousarray(prob.W.copy())
        U = np.ascontiguousarray(prob.U.copy())
        n = C.c_longlong(0)
        t = C.c_double(0)
        dt = C.c_double(0)
        err = C.create_string_buffer(4096)
        f = getattr(self.lib, self.prefix + "run_2d_ex")
        enc = lambda s: s.encode() if s is not None else None
        cbs = [C.cast(cb, C.c_void_p) if cb is not None else None
               for cb in getattr(prob, "custom_bc", (None,) * 4)]
        t0 = time.perf_counter()
        rc = f(prob.nx, prob.ny, prob.g, prob.x_min, prob.x_max, prob.y_min, prob.y_max,
               prob.gamma, enc(prob.integrator), enc(prob.riemann_solver),
               enc(prob.slope_limiter), *[enc(b) for b in prob.bc],
               prob.cfl, prob.tf, prob.max_steps,
               _ptr(W[0]), _ptr(W[1]), _ptr(W[2]), _ptr(W[3]),
               _ptr(U[0]), _ptr(U[1]), _ptr(U[2]), _ptr(U[3]),
               C.byref(n), C.byref(t), C.byref(dt), err, len(err),
               float(getattr(prob, "gravity", 0.0)), *cbs)
        secs = time.perf_counter() - t0
        return Result(rc, W, U, n.value, t.value, dt.value,
                      err.value.decode(errors="replace"), secs)

    def run_1d(self, prob: Problem1D) -> Result:
        W = np.ascontiguousarray(prob.W.copy())
        U = np.ascontiguousarray(prob.U.copy())
        n = C.c_longlong(0)
        t = C.c_double(0)
        dt = C.c_double(0)
        err = C.create_string_buffer(4096)
        f = getattr(self.lib, self.prefix + "run_1d_ex")
        enc = lambda s: s.encode() if s is not None else None
        t0 = time.perf_counter()
        rc = f(prob.nx, prob.g, prob.x_min, prob.x_max, prob.gamma,
               enc(prob.integrator), enc(prob.riemann_solver), enc(prob.slope_limiter),
               enc(prob.bc[0]), enc(prob.bc[1]), prob.cfl, prob.tf, prob.max_steps,
               _ptr(W[0]), _ptr(W[1]), _ptr(W[2]), _ptr(U[0]), _ptr(U[1]), _ptr(U[2]),
               C.byref(n), C.byref(t), C.byref(dt), err, len(err),
               enc(getattr(prob, "coord_sys", "cartesian_1d")))
        secs = time.perf_counter() - t0
        return Result(rc, W, U, n.value, t.value, dt.value, err.value.decode(errors="replace"), secs)

    def hllc_2d(self, gamma, L, R, tol=1e-6):
        out = np.zeros(4)
        rc = getattr(self.lib, self.prefix + "hllc_2d")(gamma, *L, *R, tol, _ptr(out))
        return rc, out

    def exact_flux_1d(self, gamma, L, R, tol=1e-6, speed=0.0):
        out = np.zeros(3)
        rc = getattr(self.lib, self.prefix + "exact_flux_1d")(gamma, *L, *R, tol, speed, _ptr(out))
        return rc, out

    def hllc_1d(self, gamma, L, R, tol=1e-6):
        out = np.zeros(3)
        rc = getattr(self.lib, self.prefix + "hllc_1d")(gamma, *L, *R, tol, _ptr(out))
        return rc, out

    def exact_1d(self, gamma, L, R, tol=1e-6, speed=0.0):
        """solve_exact_1d: the exact solution sampled at x/t = speed, (rho, u, p)."""
        out = np.zeros(3)
        rc = getattr(self.lib, self.prefix + "exact_1d")(gamma, *L, *R, tol, speed, _ptr(out))
        return rc, out

    def exact_status(self, gamma, L, R, tol=1e-6):
        """How solve_exact_1d ends: (0 solved | 1 bracket failure | 2 bisection
        not converged, message)."""
        err = C.create_string_buffer(4096)
        kind = getattr(self.lib, self.prefix + "exact_status")(gamma, *L, *R, tol, err, len(err))
        return kind, err.value.decode(errors="replace")

    def geometry_source_1d(self, prob: Problem1D, W: np.ndarray, U: np.ndarray, dt: float):
        """add_geometry_source_term on copies of (W, U): (rc, W, U)."""
        W = np.ascontiguousarray(W, dtype=np.float64).copy()
        U = np.ascontiguousarray(U, dtype=np.float64).copy()
        coord = {"cylindrical_1d": 2, "spherical_1d": 3}[prob.coord_sys]
        rc = getattr(self.lib, self.prefix + "geometry_source_1d")(
            coord, prob.nx, prob.g, prob.x_min, prob.x_max, prob.gamma, dt,
            prob.bc[0].encode(), prob.bc[1].encode(), *[_ptr(a) for a in W], *[_ptr(a) for a in U])
        return rc, W, U

    def gravity_source_2d(self, prob: Problem2D, W: np.ndarray, U: np.ndarray, dt: float):
        """add_gravity_source_term_2d on copies of (W, U): (rc, W, U)."""
        W = np.ascontiguousarray(W, dtype=np.float64).copy()
        U = np.ascontiguousarray(U, dtype=np.float64).copy()
        rc = getattr(self.lib, self.prefix + "gravity_source_2d")(
            prob.nx, prob.ny, prob.g, prob.x_min, prob.x_max, prob.y_min, prob.y_max, prob.gamma,
            float(prob.gravity), dt, *[b.encode() for b in prob.bc],
            *[_ptr(a) for a in W], *[_ptr(a) for a in U])
        return rc, W, U

    def guess_p(self, gamma, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, tol=1e-6):
        return getattr(self.lib, self.prefix + "guess_p")(
            gamma, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, tol)

    def limit_slope(self, flag, a, b):
        out = C.c_double(0)
        rc = getattr(self.lib, self.prefix + "limit_slope")(flag, a, b, C.byref(out))
        return rc, out.value


# Seeded workloads live with the package (hydrofv_gb300/problems.py); they are
# re-exported here so tests can use one namespace.
from hydrofv_gb300.problems import (  # noqa: E402,F401
    Problem1D, Problem2D, apply_bc_2d, four_quadrant, geometry_1d, lid_driven_cavity, lid_top_bc,
    mid_points, point_blast, primitive_to_conserved_1d, primitive_to_conserved_2d, random_problem_2d,
    rayleigh_taylor, sedov_1d, shear_layer, sod_1d,
)


def rel_l1(a: np.ndarray, b: np.ndarray, g: int) -> np.ndarray:
    """Per-field sum|a-b| / sum|b| over interior cells (arrays (F, ny', nx'))."""
    if a.ndim == 3:
        ia = a[:, g:-g, g:-g]
        ib = b[:, g:-g, g:-g]
        axes = (1, 2)
    else:
        ia = a[:, g:-g]
        ib = b[:, g:-g]
        axes = (1,)
    num = np.abs(ia - ib).sum(axis=axes)
    den = np.abs(ib).sum(axis=axes)
    return np.where(den > 0, num / np.where(den > 0, den, 1.0), num)
