"""Seeded workload definitions (initial conditions and run parameters).

These are the problems the tests and the benchmark run, in the reference's
padded layout: (F, ny+2G, nx+2G) row-major arrays, W = (rho, u, v, p) and
U = volume totals (mass, mom_x, mom_y, energy).  Geometry follows the
reference: dx includes the ghost cells (src/system.c:291-309) and mid points
run over the padded range (src/system.c:318-356).  The conversion to U uses
the reference's operation order (src/system.c:849-917) in numpy float64.

One documented PRNG is used everywhere: numpy's PCG64 via
np.random.default_rng(seed).
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

_dp = C.POINTER(C.c_double)

# Custom boundary callback of a 2D side, as BoundaryConditionParam stores it
# (src/boundary.h:40-48): (density, velocity_x, velocity_y, pressure,
# num_ghost_cells_side, num_cells_x, num_cells_y), padded arrays in place.
BcCallback = C.CFUNCTYPE(None, _dp, _dp, _dp, _dp, C.c_int, C.c_int, C.c_int)


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
    gravity: float = 0.0
    custom_bc: tuple = (None, None, None, None)   # BcCallback per side for "custom" sides

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
    coord_sys: str = "cartesian_1d"   # or "cylindrical_1d", "spherical_1d"

    def copy(self) -> "Problem1D":
        import copy
        p = copy.copy(self)
        p.W = self.W.copy()
        p.U = self.U.copy()
        return p


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


def apply_bc_2d(W: np.ndarray, g: int, nx: int, ny: int, bc, custom=(None, None, None, None)) -> None:
    """Ghost fill on W in place, sides in the reference's order
    (src/boundary.c:513-777); custom sides call their BcCallback."""
    flags = list(bc)

    def call(side):
        assert W.flags.c_contiguous and W.dtype == np.float64
        ptrs = [W[q].ctypes.data_as(_dp) for q in range(4)]
        custom[side](*ptrs, g, nx, ny)

    for side in (0, 1):
        f = flags[side]
        if f == "custom":
            call(side)
            continue
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
        if f == "custom":
            call(2 + side)
            continue
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
                limiter: str = "monotonized_central", rho_p_noise: float = 0.0) -> Problem2D:
    """Shear layer on [0,1]^2, periodic, gamma=5/3: rho=2, vx=+0.5 for
    |y-0.5|<0.25 else rho=1, vx=-0.5; p=2.5; vy=0.01 sin(4 pi x); seeded
    uniform noise U[-1e-3, 1e-3] on vx then vy (row-major over the interior).
    MUSCL-Hancock + HLLC + MC, CFL 0.8, fixed step count.

    rho_p_noise > 0 also multiplies rho and p by 1 + U[-a, a] (a second
    seeded stream, so the velocity noise is unchanged): with piecewise
    constant rho and uniform p every limiter of those fields sits at its
    a = b = 0 kink, where the step has no derivative; the noise moves them
    off it."""
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
    if rho_p_noise > 0.0:
        rng2 = np.random.default_rng(seed + 1)
        W[0][I] *= 1.0 + rng2.uniform(-rho_p_noise, rho_p_noise, size=(n, n))
        W[3][I] *= 1.0 + rng2.uniform(-rho_p_noise, rho_p_noise, size=(n, n))
    bc = ("periodic",) * 4
    apply_bc_2d(W, g, n, n, bc)
    dx = 1.0 / N
    U = primitive_to_conserved_2d(W, gamma, dx * dx)
    name = f"shear_layer_{n}" + (f"_noise{rho_p_noise:g}" if rho_p_noise > 0.0 else "")
    return Problem2D(n, n, g, 0.0, 1.0, 0.0, 1.0, gamma, W, U, bc,
                     "muscl_hancock_2d", "riemann_solver_hllc", limiter,
                     cfl=0.8, tf=1e300, max_steps=steps, name=name)


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


def geometry_1d(x_min: float, x_max: float, n: int, g: int, coord_sys: str):
    """(surface_area_x, volume, mid_points_x) of a 1D grid as system_init sets
    them (src/system.c:318-356, :365-529): areas at the faces r = x_min + i dx
    (2 pi r cylindrical, entry 0 unset there and 0 here; 4 pi r^2 spherical;
    1 Cartesian), shell volumes, cell-centre mid points."""
    tot = n + 2 * g
    dx = (x_max - x_min) / tot
    i = np.arange(tot + 1, dtype=np.float64)
    r = x_min + i * dx
    if coord_sys == "cartesian_1d":
        area = np.ones(tot + 1)
        vol = np.full(tot, dx)
    elif coord_sys == "cylindrical_1d":
        area = 2.0 * math.pi * r
        area[0] = 0.0
        vol = math.pi * (r[1:] * r[1:] - r[:-1] * r[:-1])
    elif coord_sys == "spherical_1d":
        area = 4.0 * math.pi * r * r
        vol = (4.0 / 3.0) * math.pi * (r[1:] * r[1:] * r[1:] - r[:-1] * r[:-1] * r[:-1])
    else:
        raise ValueError(coord_sys)
    mid = x_min + (np.arange(tot) + 0.5) * dx
    return area, vol, mid


def conserved_to_primitive_1d(U: np.ndarray, gamma: float, vol) -> np.ndarray:
    """src/system.c:735-761."""
    m, mom, E = U
    W = np.empty_like(U)
    W[0] = m / vol
    W[1] = mom / m
    W[2] = (gamma - 1.0) * (E - 0.5 * m * W[1] * W[1]) / vol
    return W


def sod_1d(n: int = 1000, g: int = 2, coord_sys: str = "cartesian_1d") -> Problem1D:
    """Sod shock tube as in examples/sod_shock_1d/sod_shock_1d.c:47-62: left
    (1, 0, 1) for x < 0.5, right (0.125, 0, 0.1), set over the padded range;
    transmissive; Godunov first order + exact solver; CFL 0.9, tf = 0.2.  On
    cylindrical / spherical grids x is the radius."""
    gamma = 1.4
    x = mid_points(0.0, 1.0, n, g)
    left = x < 0.5
    W = np.zeros((3, n + 2 * g))
    W[0] = np.where(left, 1.0, 0.125)
    W[1] = 0.0
    W[2] = np.where(left, 1.0, 0.1)
    vol = geometry_1d(0.0, 1.0, n, g, coord_sys)[1] if coord_sys != "cartesian_1d" else 1.0 / (n + 2 * g)
    U = primitive_to_conserved_1d(W, gamma, vol)
    return Problem1D(n, g, 0.0, 1.0, gamma, W, U, ("transmissive", "transmissive"),
                     "godunov_first_order_1d", "riemann_solver_exact", "minmod",
                     cfl=0.9, tf=0.2, max_steps=-1, name=f"sod_{n}_{coord_sys}", coord_sys=coord_sys)


def sedov_1d(n_total: int = 64, g: int = 2, coord_sys: str = "cylindrical_1d",
             steps: int = -1) -> Problem1D:
    """Sedov blast as in examples/sedov_blast_1d/sedov_blast_1d.c:20-105: [0, 1.2],
    rho = 1, u = 0, p = 1e-5, reflective at r = 0 and transmissive outside; the
    first 3 interior cells get the energy E_0 / 3 (E_0 = 0.0673185, 0.311357,
    0.851072 for Cartesian, cylindrical, spherical) after W -> U, then U -> W
    and the ghost fill.  MUSCL-Hancock + HLLC + MC, CFL 0.4, tf = 1."""
    gamma = 1.4
    n = n_total - 2 * g
    area, vol, mid = geometry_1d(0.0, 1.2, n, g, coord_sys)
    W = np.zeros((3, n_total))
    W[0, g:g + n] = 1.0
    W[1, g:g + n] = 0.0
    W[2, g:g + n] = 1e-5
    bc = ("reflective", "transmissive")

    def fill(W):
        W[0, g - 1 - np.arange(g)] = W[0, g + np.arange(g)]
        W[1, g - 1 - np.arange(g)] = -W[1, g + np.arange(g)]
        W[2, g - 1 - np.arange(g)] = W[2, g + np.arange(g)]
        W[:, g + n + np.arange(g)] = W[:, g + n - 1 - np.arange(g)]

    fill(W)
    U = primitive_to_conserved_1d(W, gamma, vol)
    E0 = {"cartesian_1d": 0.0673185, "cylindrical_1d": 0.311357, "spherical_1d": 0.851072}[coord_sys] / 3
    U[2, g:g + 3] = E0
    W = conserved_to_primitive_1d(U, gamma, vol)
    fill(W)
    return Problem1D(n, g, 0.0, 1.2, gamma, W, U, bc, "muscl_hancock_1d", "riemann_solver_hllc",
                     "monotonized_central", cfl=0.4, tf=1.0, max_steps=steps,
                     name=f"sedov_{n}_{coord_sys}", coord_sys=coord_sys)




def random_problem_1d(nx: int, seed: int, bc, integrator: str = "godunov_first_order_1d",
                      riemann_solver: str = "riemann_solver_exact", limiter: str = "minmod",
                      steps: int = 20, g: int = 2) -> Problem1D:
    """Smooth random 1D states (plus a jump) for edge-case parity tests."""
    rng = np.random.default_rng(seed)
    gamma = float(rng.choice([1.4, 5.0 / 3.0]))
    x = mid_points(0.0, 1.0, nx, g)
    W = np.zeros((3, nx + 2 * g))
    W[0] = 1.0 + 0.3 * np.sin(2 * math.pi * x) + np.where(x < 0.5, 0.5, 0.0)
    W[1] = 0.2 * np.cos(2 * math.pi * x)
    W[2] = 1.0 + 0.2 * np.cos(4 * math.pi * x) + np.where(x < 0.3, 0.4, 0.0)
    W += rng.uniform(-1e-3, 1e-3, size=W.shape)
    vol = 1.0 / (nx + 2 * g)
    U = primitive_to_conserved_1d(W, gamma, vol)
    return Problem1D(nx, g, 0.0, 1.0, gamma, W, U, tuple(bc), integrator, riemann_solver,
                     limiter, cfl=0.8, tf=1e300, max_steps=steps, name=f"random1d_{nx}_{seed}")


def four_quadrant_ensemble(count: int = 256, seed: int = 4, steps: int = 500,
                           side_range=(128, 1024), limiter: str = "minmod"):
    """Batched ensemble of independent four-quadrant Riemann problems: grid side
    drawn log-uniform in side_range per instance, quadrant states
    rho, p ~ U[0.1, 2], u, v ~ U[-1, 1], gamma = 1.4, transmissive,
    MUSCL-Hancock + HLLC + minmod, CFL 0.8, per-instance dt."""
    rng = np.random.default_rng(seed)
    lo, hi = math.log(side_range[0]), math.log(side_range[1])
    sides = np.rint(np.exp(rng.uniform(lo, hi, size=count))).astype(int)
    return [four_quadrant(int(s), rng, steps=steps, limiter=limiter) for s in sides]


def right_half_density_squared(p: Problem2D, W: np.ndarray) -> tuple[float, np.ndarray]:
    """Objective of the adjoint workload: J = sum over the interior cells whose
    centre has x > (x_min + x_max)/2 of rho^2 * V (V the cell volume the
    problem's conserved state uses), and dJ/dW (zero elsewhere)."""
    x = mid_points(p.x_min, p.x_max, p.nx, p.g)
    mask = np.zeros(W.shape[1:], dtype=bool)
    mask[p.g:p.g + p.ny, p.g:p.g + p.nx] = True
    mask &= (x[None, :] > 0.5 * (p.x_min + p.x_max))
    vol = ((p.x_max - p.x_min) / (p.nx + 2 * p.g)) * ((p.y_max - p.y_min) / (p.ny + 2 * p.g))
    rho = W[0]
    J = math.fsum((rho[mask] ** 2).ravel()) * vol
    seed = np.zeros_like(W)
    seed[0][mask] = 2.0 * rho[mask] * vol
    return J, seed


def lid_top_bc(lid_u: float = 10.0, lid_v: float = -0.5) -> BcCallback:
    """Top-side callback of the modified lid-driven cavity example
    (examples/modified_lid_driven_cavity_2d/lid_driven_cavity_2d.c:39-58):
    every column of the top ghost rows mirrors density and pressure and
    takes the lid velocity."""
    def fn(rho, vx, vy, p, g, nx, ny):
        tx, ty = nx + 2 * g, ny + 2 * g
        R, X, Y, P = (np.ctypeslib.as_array(a, shape=(ty, tx)) for a in (rho, vx, vy, p))
        for j in range(g):
            R[g + ny + j, :] = R[g + ny - 1 - j, :]
            X[g + ny + j, :] = lid_u
            Y[g + ny + j, :] = lid_v
            P[g + ny + j, :] = P[g + ny - 1 - j, :]
    return BcCallback(fn)


def rayleigh_taylor(nx: int = 122, ny: int = 122, g: int = 3, steps: int = 200) -> Problem2D:
    """Rayleigh-Taylor example (examples/rayleign_taylor_2d/rayleigh_taylor_2d.c:
    20-110): [0,0.5] x [0,2], gamma 5/3, gravity 0.1, periodic x, reflective y;
    rho = 1 below y = 1, 2 above, hydrostatic p = 2.5 - 0.1 rho (y - 0.75),
    vy = 0.0025 (1 - cos 4 pi x)(1 - cos(4/3 pi (y - 0.5))); MUSCL-Hancock,
    MC, CFL 0.5."""
    gamma = 5.0 / 3.0
    grav = 0.1
    x = mid_points(0.0, 0.5, nx, g)
    y = mid_points(0.0, 2.0, ny, g)
    X, Y = np.meshgrid(x, y)
    W = np.zeros((4, ny + 2 * g, nx + 2 * g))
    I = (slice(g, g + ny), slice(g, g + nx))
    lower = Y < 1.0
    W[0][I] = np.where(lower, 1.0, 2.0)[I]
    W[1][I] = 0.0
    W[3][I] = np.where(lower, 2.5 - grav * 1.0 * (Y - 0.75), 2.5 - grav * 2.0 * (Y - 0.75))[I]
    W[2][I] = (0.0025 * (1.0 - np.cos(4 * math.pi * X)) * (1.0 - np.cos(4.0 / 3.0 * math.pi * (Y - 0.5))))[I]
    bc = ("periodic", "periodic", "reflective", "reflective")
    apply_bc_2d(W, g, nx, ny, bc)
    vol = (0.5 / (nx + 2 * g)) * (2.0 / (ny + 2 * g))
    U = primitive_to_conserved_2d(W, gamma, vol)
    return Problem2D(nx, ny, g, 0.0, 0.5, 0.0, 2.0, gamma, W, U, bc, "muscl_hancock_2d",
                     "riemann_solver_hllc", "monotonized_central", cfl=0.5, tf=1e300,
                     max_steps=steps, name=f"rayleigh_taylor_{nx}x{ny}", gravity=grav)


def lid_driven_cavity(n: int = 250, g: int = 3, steps: int = 200) -> Problem2D:
    """Modified lid-driven cavity example
    (examples/modified_lid_driven_cavity_2d/lid_driven_cavity_2d.c:20-110):
    [0,1]^2, gamma 5/3, rho = 1, u = v = 0, p = 1; reflective except a custom
    top side (lid_top_bc); MUSCL-Hancock, MC, CFL 0.5."""
    gamma = 5.0 / 3.0
    W = np.zeros((4, n + 2 * g, n + 2 * g))
    I = (slice(g, g + n), slice(g, g + n))
    W[0][I] = 1.0
    W[3][I] = 1.0
    bc = ("reflective", "reflective", "reflective", "custom")
    custom = (None, None, None, lid_top_bc())
    apply_bc_2d(W, g, n, n, bc, custom)
    vol = (1.0 / (n + 2 * g)) ** 2
    U = primitive_to_conserved_2d(W, gamma, vol)
    return Problem2D(n, n, g, 0.0, 1.0, 0.0, 1.0, gamma, W, U, bc, "muscl_hancock_2d",
                     "riemann_solver_hllc", "monotonized_central", cfl=0.5, tf=1e300,
                     max_steps=steps, name=f"lid_driven_cavity_{n}", custom_bc=custom)
