"""Generate the golden fixtures in tests/golden/ from the unmodified reference.

    make -C oracle ref          # compiles the reference's src/*.c into oracle/_ref
    python tests/golden/make_golden.py [name ...]   # all fixtures, or the named ones

Each fixture stores the reference's outputs (final W and U, status) for a
seeded problem from hydrofv_gb300.problems, plus a checksum of the inputs so a
change of the generators is detected instead of silently compared.  The
pointwise fixtures store reference outputs of the exported numerics on seeded
random states, including vacuum, two-rarefaction and two-shock cases.

This script runs only where the reference tree was compiled (oracle/_ref);
the tests read the committed .npz files and never need the reference.
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from hydrofv_gb300 import problems as P  # noqa: E402


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def cases_2d():
    rng = np.random.default_rng(7)
    out = {
        "shear_layer_48_mc_30": P.shear_layer(48, steps=30),
        "point_blast_40_vl_40": P.point_blast(40, steps=40),
        "four_quadrant_32_mm_40": P.four_quadrant(32, rng, steps=40),
    }
    for lim in ("minmod", "van_leer", "monotonized_central"):
        out[f"random_19x13_mixedbc_{lim}_15"] = P.random_problem_2d(
            19, 13, 5, ("reflective", "transmissive", "none", "reflective"), lim, 15, smooth=True)
    out["random_17x11_periodic_godunov_10"] = P.random_problem_2d(
        17, 11, 9, ("periodic",) * 4, "minmod", 10, smooth=True,
        integrator="godunov_first_order_2d")
    p = P.four_quadrant(24, np.random.default_rng(11), steps=-1)
    p.max_steps = -1
    p.tf = 0.04
    out["four_quadrant_24_mm_tf0.04"] = p
    # gravity source (the Rayleigh-Taylor example) and a custom side (the lid-driven cavity)
    out["rayleigh_taylor_24x40_g3_30"] = P.rayleigh_taylor(24, 40, g=3, steps=30)
    out["lid_cavity_32_g3_30"] = P.lid_driven_cavity(32, g=3, steps=30)
    return out


def cases_1d():
    sod = P.sod_1d(1000)
    mh = P.sod_1d(200)
    mh.integrator = "muscl_hancock_1d"
    mh.riemann_solver = "riemann_solver_hllc"
    mh.slope_limiter = "van_leer"
    mhx = P.sod_1d(100)
    mhx.integrator = "muscl_hancock_1d"
    mhx.riemann_solver = "riemann_solver_exact"
    mhx.slope_limiter = "monotonized_central"
    out = {"sod_1000_godunov_exact": sod, "sod_200_muscl_hllc_vl": mh,
           "sod_100_muscl_exact_mc": mhx}
    # cylindrical / spherical grids (geometry source) and the random-choice integrator
    for coord in ("cylindrical_1d", "spherical_1d"):
        p = P.sod_1d(100, coord_sys=coord)
        out[f"sod_100_{coord}_godunov_exact"] = p
        p = P.sod_1d(100, coord_sys=coord)
        p.integrator, p.riemann_solver, p.slope_limiter = "muscl_hancock_1d", "riemann_solver_hllc", "van_leer"
        out[f"sod_100_{coord}_muscl_hllc_vl"] = p
        out[f"sedov_60_{coord}_muscl_hllc_mc"] = P.sedov_1d(64, coord_sys=coord)
    for coord in ("cartesian_1d", "spherical_1d"):
        p = P.sod_1d(100, coord_sys=coord)
        p.integrator = "random_choice_1d"
        out[f"sod_100_{coord}_random_choice"] = p
    return out


def pointwise(ref):
    rng = np.random.default_rng(2024)
    n = 3000
    gam = rng.choice([1.4, 5.0 / 3.0, 1.2], size=n)
    rho = rng.uniform(0.05, 3.0, size=(n, 2))
    u = rng.uniform(-2.0, 2.0, size=(n, 2))
    v = rng.uniform(-1.0, 1.0, size=(n, 2))
    p = 10.0 ** rng.uniform(-3, 1, size=(n, 2))
    # strong expansions (vacuum generation) and near-vacuum states
    u[:200, 0] = -5.0
    u[:200, 1] = 5.0
    rho[200:230, 0] = 0.0
    rho[230:260, 1] = 0.0
    L = np.stack([rho[:, 0], u[:, 0], v[:, 0], p[:, 0]], axis=1)
    R = np.stack([rho[:, 1], u[:, 1], v[:, 1], p[:, 1]], axis=1)
    hllc = np.zeros((n, 4))
    hllc_rc = np.zeros(n, dtype=np.int32)
    for k in range(n):
        hllc_rc[k], hllc[k] = ref.hllc_2d(gam[k], L[k], R[k])
    m = 600
    ex = np.zeros((m, 3))
    ex_rc = np.zeros(m, dtype=np.int32)
    speeds = rng.uniform(-1.0, 1.0, size=m)
    speeds[: m // 2] = 0.0
    for k in range(m):
        ex_rc[k], ex[k] = ref.exact_flux_1d(gam[k], L[k, [0, 1, 3]], R[k, [0, 1, 3]], speed=speeds[k])
    # the 1D HLLC flux and the sampled exact solution on the same states
    hllc1 = np.zeros((m, 3))
    hllc1_rc = np.zeros(m, dtype=np.int32)
    ex_state = np.zeros((m, 3))
    ex_state_rc = np.zeros(m, dtype=np.int32)
    for k in range(m):
        hllc1_rc[k], hllc1[k] = ref.hllc_1d(gam[k], L[k, [0, 1, 3]], R[k, [0, 1, 3]])
        ex_state_rc[k], ex_state[k] = ref.exact_1d(gam[k], L[k, [0, 1, 3]], R[k, [0, 1, 3]], speed=speeds[k])
    gp = np.array([ref.guess_p(gam[k], L[k, 0], L[k, 1], L[k, 3], np.sqrt(gam[k] * L[k, 3] / max(L[k, 0], 1e-30)),
                               R[k, 0], R[k, 1], R[k, 3], np.sqrt(gam[k] * R[k, 3] / max(R[k, 0], 1e-30)))
                   for k in range(n)])
    a = rng.normal(size=1000)
    b = rng.normal(size=1000)
    b[:100] = a[:100]
    b[100:150] = 0.0
    lim = np.zeros((3, 1000))
    for f in (1, 2, 3):
        for k in range(1000):
            lim[f - 1, k] = ref.limit_slope(f, a[k], b[k])[1]
    return dict(gamma=gam, L=L, R=R, hllc=hllc, hllc_rc=hllc_rc, speeds=speeds, exact=ex,
                exact_rc=ex_rc, guess_p=gp, lim_a=a, lim_b=b, limited=lim, hllc_1d=hllc1,
                hllc_1d_rc=hllc1_rc, exact_state=ex_state, exact_state_rc=ex_state_rc)


def main():
    if not O.reference_available():
        sys.exit("oracle/_ref not built: run `make -C oracle ref` where the reference tree exists")
    ref = O.load("ref")
    ref_serial = O.load("ref_serial")
    only = set(sys.argv[1:])

    def wanted(name):
        return not only or name in only

    for name, p in cases_2d().items():
        if not wanted(name):
            continue
        r = ref.run_2d(p)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), W=r.W, U=r.U, rc=r.rc,
                            num_steps=r.num_steps, t=r.t, dt=r.dt, input_sha=digest(p.W, p.U))
        print(name, r.rc, r.num_steps, r.t)
    for name, p in cases_1d().items():
        if not wanted(name):
            continue
        r = ref_serial.run_1d(p)  # the reference's OpenMP 1D loops race; serial build
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), W=r.W, U=r.U, rc=r.rc,
                            num_steps=r.num_steps, t=r.t, dt=r.dt, input_sha=digest(p.W, p.U))
        print(name, r.rc, r.num_steps, r.t)
    if wanted("pointwise"):
        np.savez_compressed(os.path.join(HERE, "pointwise.npz"), **pointwise(ref))
        print("pointwise done")


if __name__ == "__main__":
    main()
