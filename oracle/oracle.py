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
import math
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REFDIR = os.path.join(HERE, "_ref")

_dp = C.POINTER(C.c_double)
_i64p = C.POINTER(C.c_longlong)


def build(with_reference: bool | None = None) -> None:
    """Compile the restatement (and the reference, when its tree exists)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    ref_src = os.environ.get("HYDRO_REF_SRC", "/root/reference/src")
    if with_reference is None:
        with_reference = os.path.isdir(ref_src)
    if with_reference:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref_src}"], check=True)


_libs: dict[str, C.CDLL] = {}


def _bind(lib: C.CDLL, prefix: str) -> C.CDLL:
    f = getattr(lib, prefix + "run_2d")
    f.restype = C.c_int
    f.argtypes = ([C.c_int] * 3 + [C.c_double] * 5 + [C.c_char_p] * 7
                  + [C.c_double, C.c_double, C.c_longlong] + [_dp] * 8
                  + [_i64p, _dp, _dp, C.c_char_p, C.c_int])
    f = getattr(lib, prefix + "run_1d")
    f.restype = C.c_int
    f.argtypes = ([C.c_int] * 2 + [C.c_double] * 3 + [C.c_char_p] * 5
                  + [C.c_double, C.c_double, C.c_longlong] + [_dp] * 6
                  + [_i64p, _dp, _dp, C.c_char_p, C.c_int])
    f = getattr(lib, prefix + "hllc_2d")
    f.restype = C.c_int
    f.argtypes = [C.c_double] * 10 + [_dp]
    f = getattr(lib, prefix + "exact_flux_1d")
    f.restype = C.c_int
    f.argtypes = [C.c_double] * 9 + [_dp]
    f = getattr(lib, prefix + "guess_p")
    f.restype = C.c_double
    f.argtypes = [C.c_double] * 10
    f = getattr(lib, prefix + "limit_slope")
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_double, C.c_double, _dp]
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
class Problem2D:
    """A 2D Cartesian problem in the reference's padded layout."""
    nx: int
    ny: int
    g: int
    x_min: float
    x_max: float
    y_min: float
    y_max: float
    gamma: float
    W: np.ndarray              # (4, ny+2g, nx+2g): rho, u, v, p
    U: np.ndarray              # (4, ny+2g, nx+2g): mass, mom_x, mom_y, energy
    bc: tuple = ("periodic",) * 4
    integrator: str = "muscl_hancock_2d"
    riemann_solver: str = "riemann_solver_hllc"
    slope_limiter: str = "monotonized_central"
    cfl: float = 0.8
    tf: float = 1.0
    max_steps: int = -1
    name: str = ""

    def copy(self) -> "Problem2D":
        import copy
        p = copy.copy(self)
        p.W = self.W.copy()
        p.U = self.U.copy()
        return p

    @property
    def dx(self) -> float:
        return (self.x_max - self.x_min) / (self.nx + 2 * self.g)

    @property
    def dy(self) -> float:
        return (self.y_max - self.y_min) / (self.ny + 2 * self.g)


@dataclass
class Problem1D:
    nx: int
    g: int
    x_min: float
    x_max: float
    gamma: float
    W: np.ndarray              # (3, nx+2g): rho, u, p
    U: np.ndarray              # (3, nx+2g): mass, mom, energy
    bc: tuple = ("transmissive", "transmissive")
    integrator: str = "godunov_first_order_1d"
    riemann_solver: str = "riemann_solver_exact"
    slope_limiter: str = "minmod"
    cfl: float = 0.9
    tf: float = 0.2
    max_steps: int = -1
    name: str = ""

    def copy(self) -> "Problem1D":
        import copy
        p = copy.copy(self)
        p.W = self.W.copy()
        p.U = self.U.copy()
        return p


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
        import time
        W = np.ascontiguousarray(prob.W.copy())
        U = np.ascontiguousarray(prob.U.copy())
        n = C.c_longlong(0)
        t = C.c_double(0)
        dt = C.c_double(0)
        err = C.create_string_buffer(4096)
        f = getattr(self.lib, self.prefix + "run_2d")
        enc = lambda s: s.encode() if s is not None else None
        t0 = time.perf_counter()
        rc = f(prob.nx, prob.ny, prob.g, prob.x_min, prob.x_max, prob.y_min, prob.y_max,
               prob.gamma, enc(prob.integrator), enc(prob.riemann_solver),
               enc(prob.slope_limiter), *[enc(b) for b in prob.bc],
               prob.cfl, prob.tf, prob.max_steps,
               _ptr(W[0]), _ptr(W[1]), _ptr(W[2]), _ptr(W[3]),
               _ptr(U[0]), _ptr(U[1]), _ptr(U[2]), _ptr(U[3]),
               C.byref(n), C.byref(t), C.byref(dt), err, len(err))
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
        f = getattr(self.lib, self.prefix + "run_1d")
        enc = lambda s: s.encode() if s is not None else None
        rc = f(prob.nx, prob.g, prob.x_min, prob.x_max, prob.gamma,
               enc(prob.integrator), enc(prob.riemann_solver), enc(prob.slope_limiter),
               enc(prob.bc[0]), enc(prob.bc[1]), prob.cfl, prob.tf, prob.max_steps,
               _ptr(W[0]), _ptr(W[1]), _ptr(W[2]), _ptr(U[0]), _ptr(U[1]), _ptr(U[2]),
               C.byref(n), C.byref(t), C.byref(dt), err, len(err))
        return Result(rc, W, U, n.value, t.value, dt.value, err.value.decode(errors="replace"))

    def hllc_2d(self, gamma, L, R, tol=1e-6):
        out = np.zeros(4)
        rc = getattr(self.lib, self.prefix + "hllc_2d")(gamma, *L, *R, tol, _ptr(out))
        return rc, out

    def exact_flux_1d(self, gamma, L, R, tol=1e-6, speed=0.0):
        out = np.zeros(3)
        rc = getattr(self.lib, self.prefix + "exact_flux_1d")(gamma, *L, *R, tol, speed, _ptr(out))
        return rc, out

    def guess_p(self, gamma, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, tol=1e-6):
        return getattr(self.lib, self.prefix + "guess_p")(
            gamma, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, tol)

    def limit_slope(self, flag, a, b):
        out = C.c_double(0)
        rc = getattr(self.lib, self.prefix + "limit_slope")(flag, a, b, C.byref(out))
        return rc, out.value


# --------------------------------------------------------------------------
# Seeded initial conditions (one documented PRNG: numpy PCG64 via
# np.random.default_rng(seed)).  Geometry follows the reference: dx includes
# the ghost cells (src/system.c:291-309), mid points are x_min + (i+1/2) dx
# over the padded range (:318-356).
# --------------------------------------------------------------------------

def primitive_to_conserved_2d(W: np.ndarray, gamma: float, vol: float) -> np.ndarray:
    """src/system.c:885-905, element-wise in numpy (same IEEE operation order)."""
    rho, u, v, p = W
    m = rho * vol
    U = np.empty_like(W)
    U[0] = m
    U[1] = m * u
    U[2] = m * v
    U[3] = vol * (0.5 * rho * (u * u + v * v) + p / (gamma - 1.0))
    return U


def primitive_to_conserved_1d(W: np.ndarray, gamma: float, vol: float) -> np.ndarray:
    """src/system.c:868-882."""
    rho, u, p = W
    U = np.empty_like(W)
    U[0] = rho * vol
    U[1] = U[0] * u
    U[2] = vol * (0.5 * rho * u * u + p / (gamma - 1.0))
    return U


def apply_bc_2d(W: np.ndarray, g: int, nx: int, ny: int, bc) -> None:
    """Built-in ghost fill on W in place (src/boundary.c:513-777)."""
    flags = list(bc)
    for side in (0, 1):
        f = flags[side]
        if f == "none" or (f == "periodic" and side == 0):
            continue
        for k in range(g):
            rows = slice(g, g + ny)
            if f == "periodic":
                W[:, rows, g + nx + k] = W[:, rows, g + k]
                W[:, rows, g - 1 - k] = W[:, rows, g + nx - 1 - k]
                continue
            dst, src = (g - 1 - k, g + k) if side == 0 else (g + nx + k, g + nx - 1 - k)
            W[:, rows, dst] = W[:, rows, src]
            if f == "reflective":
                W[1, rows, dst] = -W[1, rows, src]
    for side in (0, 1):
        f = flags[2 + side]
        if f == "none" or (f == "periodic" and side == 0):
            continue
        cols = slice(g, g + nx)
        for k in range(g):
            if f == "periodic":
                W[:, g + ny + k, cols] = W[:, g + k, cols]
                W[:, g - 1 - k, cols] = W[:, g + ny - 1 - k, cols]
                continue
            dst, src = (g - 1 - k, g + k) if side == 0 else (g + ny + k, g + ny - 1 - k)
            W[:, dst, cols] = W[:, src, cols]
            if f == "reflective":
                W[2, dst, cols] = -W[2, src, cols]


def mid_points(lo: float, hi: float, n: int, g: int) -> np.ndarray:
    d = (hi - lo) / (n + 2 * g)
    return lo + (np.arange(n + 2 * g) + 0.5) * d


def shear_layer(n: int, g: int = 2, seed: int = 2024, steps: int = 200,
                limiter: str = "monotonized_central") -> Problem2D:
    """Shear layer on [0,1]^2, periodic, gamma=5/3: rho=2, vx=+0.5 for
    |y-0.5|<0.25 else rho=1, vx=-0.5; p=2.5; vy=0.01 sin(4 pi x); seeded
    uniform noise U[-1e-3, 1e-3] on vx then vy (row-major over the interior).
    MUSCL-Hancock + HLLC + MC, CFL 0.8, fixed step count."""
    gamma = 5.0 / 3.0
    N = n + 2 * g
    x = mid_points(0.0, 1.0, n, g)
    y = mid_points(0.0, 1.0, n, g)
    X, Y = np.meshgrid(x, y)
    W = np.zeros((4, N, N))
    inner = np.abs(Y - 0.5) < 0.25
    rho = np.where(inner, 2.0, 1.0)
    vx = np.where(inner, 0.5, -0.5)
    vy = 0.01 * np.sin(4.0 * math.pi * X)
    rng = np.random.default_rng(seed)
    noise_x = rng.uniform(-1e-3, 1e-3, size=(n, n))
    noise_y = rng.uniform(-1e-3, 1e-3, size=(n, n))
    I = (slice(g, g + n), slice(g, g + n))
    W[0][I] = rho[I]
    W[1][I] = vx[I] + noise_x
    W[2][I] = vy[I] + noise_y
    W[3][I] = 2.5
    bc = ("periodic",) * 4
    apply_bc_2d(W, g, n, n, bc)
    dx = 1.0 / N
    U = primitive_to_conserved_2d(W, gamma, dx * dx)
    return Problem2D(n, n, g, 0.0, 1.0, 0.0, 1.0, gamma, W, U, bc,
                     "muscl_hancock_2d", "riemann_solver_hllc", limiter,
                     cfl=0.8, tf=1e300, max_steps=steps, name=f"shear_layer_{n}")


def point_blast(n: int, g: int = 2, steps: int = 1000) -> Problem2D:
    """Point blast on [-1,1]^2, reflective, gamma=1.4, rho=1, u=v=0, background
    p=1e-5; total energy 1.0 shared equally by the cells with r < 2 dx and
    added as pressure p = (gamma-1) E_c / V.  Van Leer, CFL 0.4."""
    gamma = 1.4
    N = n + 2 * g
    x = mid_points(-1.0, 1.0, n, g)
    X, Y = np.meshgrid(x, x)
    dx = 2.0 / N
    vol = dx * dx
    W = np.zeros((4, N, N))
    I = (slice(g, g + n), slice(g, g + n))
    W[0][I] = 1.0
    W[3][I] = 1e-5
    r = np.sqrt(X * X + Y * Y)
    hot = np.zeros((N, N), dtype=bool)
    hot[I] = (r < 2.0 * dx)[I]
    count = int(hot.sum())
    E_c = 1.0 / count
    W[3][hot] += (gamma - 1.0) * E_c / vol
    bc = ("reflective",) * 4
    apply_bc_2d(W, g, n, n, bc)
    U = primitive_to_conserved_2d(W, gamma, vol)
    return Problem2D(n, n, g, -1.0, 1.0, -1.0, 1.0, gamma, W, U, bc,
                     "muscl_hancock_2d", "riemann_solver_hllc", "van_leer",
                     cfl=0.4, tf=1e300, max_steps=steps, name=f"point_blast_{n}")


def four_quadrant(n: int, rng: np.random.Generator, g: int = 2, steps: int = 500,
                  limiter: str = "minmod") -> Problem2D:
    """Four-quadrant Riemann problem on [0,1]^2, transmissive, gamma=1.4:
    quadrant states rho,p ~ U[0.1,2], u,v ~ U[-1,1], split at x=y=0.5."""
    gamma = 1.4
    N = n + 2 * g
    x = mid_points(0.0, 1.0, n, g)
    X, Y = np.meshgrid(x, x)
    q = rng.uniform(size=(4, 4))
    states = np.stack([0.1 + 1.9 * q[:, 0], -1.0 + 2.0 * q[:, 1],
                       -1.0 + 2.0 * q[:, 2], 0.1 + 1.9 * q[:, 3]], axis=1)
    quad = (X >= 0.5).astype(int) + 2 * (Y >= 0.5).astype(int)
    W = np.zeros((4, N, N))
    I = (slice(g, g + n), slice(g, g + n))
    for k in range(4):
        W[k][I] = states[quad, k][I]
    bc = ("transmissive",) * 4
    apply_bc_2d(W, g, n, n, bc)
    dx = 1.0 / N
    U = primitive_to_conserved_2d(W, gamma, dx * dx)
    return Problem2D(n, n, g, 0.0, 1.0, 0.0, 1.0, gamma, W, U, bc,
                     "muscl_hancock_2d", "riemann_solver_hllc", limiter,
                     cfl=0.8, tf=1e300, max_steps=steps, name=f"four_quadrant_{n}")


def random_problem_2d(nx: int, ny: int, seed: int, bc, limiter: str, steps: int,
                      g: int = 2, integrator: str = "muscl_hancock_2d",
                      smooth: bool = False) -> Problem2D:
    """Random smooth-ish or blocky states for edge-case parity tests."""
    rng = np.random.default_rng(seed)
    gamma = float(rng.choice([1.4, 5.0 / 3.0, 1.2]))
    N = (ny + 2 * g, nx + 2 * g)
    W = np.zeros((4,) + N)
    if smooth:
        x = mid_points(0.0, 1.0, nx, g)
        y = mid_points(0.0, 1.0, ny, g)
        X, Y = np.meshgrid(x, y)
        W[0] = 1.0 + 0.3 * np.sin(2 * math.pi * X) * np.cos(2 * math.pi * Y)
        W[1] = 0.3 * np.cos(2 * math.pi * Y)
        W[2] = 0.2 * np.sin(2 * math.pi * X)
        W[3] = 1.0 + 0.2 * np.cos(2 * math.pi * (X + Y))
        W += rng.uniform(-1e-3, 1e-3, size=W.shape)
    else:
        W[0] = rng.uniform(0.2, 2.0, size=N)
        W[1] = rng.uniform(-1.0, 1.0, size=N)
        W[2] = rng.uniform(-1.0, 1.0, size=N)
        W[3] = rng.uniform(0.2, 2.0, size=N)
    apply_bc_2d(W, g, nx, ny, bc)
    dx = 1.0 / (nx + 2 * g)
    dy = 1.0 / (ny + 2 * g)
    U = primitive_to_conserved_2d(W, gamma, dx * dy)
    return Problem2D(nx, ny, g, 0.0, 1.0, 0.0, 1.0, gamma, W, U, tuple(bc),
                     integrator, "riemann_solver_hllc", limiter, cfl=0.5,
                     tf=1e300, max_steps=steps, name=f"random_{nx}x{ny}_{seed}")


def sod_1d(n: int = 1000, g: int = 2) -> Problem1D:
    """Sod shock tube as in examples/sod_shock_1d/sod_shock_1d.c:47-62: left
    (1, 0, 1) for x < 0.5, right (0.125, 0, 0.1), set over the padded range;
    transmissive; Godunov first order + exact solver; CFL 0.9, tf = 0.2."""
    gamma = 1.4
    x = mid_points(0.0, 1.0, n, g)
    left = x < 0.5
    W = np.zeros((3, n + 2 * g))
    W[0] = np.where(left, 1.0, 0.125)
    W[1] = 0.0
    W[2] = np.where(left, 1.0, 0.1)
    vol = 1.0 / (n + 2 * g)
    U = primitive_to_conserved_1d(W, gamma, vol)
    return Problem1D(n, g, 0.0, 1.0, gamma, W, U, ("transmissive", "transmissive"),
                     "godunov_first_order_1d", "riemann_solver_exact", "minmod",
                     cfl=0.9, tf=0.2, max_steps=-1, name=f"sod_{n}")


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
