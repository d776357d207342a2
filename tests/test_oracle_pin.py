"""Pin the CPU oracle before trusting it (CPU only).

* The C restatement (oracle/hydro_oracle.c) must reproduce the committed
  golden fixtures -- outputs of the unmodified reference, generated by
  tests/golden/make_golden.py -- bit for bit.
* Where the reference was compiled here (oracle/_ref), restatement and
  reference are also compared live on further seeded cases.
* The library's exported pointwise numerics (host builds of the kernels'
  templates) are checked against the same golden pointwise vectors.
* Sod at t = 0.2 is checked for accuracy against the exact solution the
  reference ships (examples/sod_shock_1d/sol_cartesian_1d_0.2.npz) where
  the reference tree was staged (oracle/_ref/examples).
"""
import ctypes as C
import hashlib
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def bits_equal(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint64),
                          np.ascontiguousarray(b).view(np.uint64))


def golden_cases():
    import sys
    sys.path.insert(0, GOLDEN)
    import make_golden as MG
    return MG.cases_2d(), MG.cases_1d()


def test_golden_files_present():
    names = [f for f in os.listdir(GOLDEN) if f.endswith(".npz")]
    assert "pointwise.npz" in names
    assert len(names) >= 12


def test_restatement_matches_golden_2d(oracle_mod):
    O = oracle_mod
    orc = O.load("oracle")
    cases2, _ = golden_cases()
    for name, p in cases2.items():
        g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
        assert str(g["input_sha"]) == digest(p.W, p.U), f"{name}: generator drifted"
        r = orc.run_2d(p)
        assert r.rc == int(g["rc"]) == 0
        assert r.num_steps == int(g["num_steps"])
        assert r.t == float(g["t"]) and r.dt == float(g["dt"])
        assert bits_equal(r.U, g["U"]), name
        assert bits_equal(r.W, g["W"]), name


def test_restatement_matches_golden_1d(oracle_mod):
    O = oracle_mod
    orc = O.load("oracle")
    _, cases1 = golden_cases()
    for name, p in cases1.items():
        g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
        assert str(g["input_sha"]) == digest(p.W, p.U), f"{name}: generator drifted"
        r = orc.run_1d(p)
        assert r.rc == 0
        assert r.num_steps == int(g["num_steps"]) and r.t == float(g["t"])
        assert bits_equal(r.U, g["U"]), name
        assert bits_equal(r.W, g["W"]), name


def test_restatement_pointwise_matches_golden(oracle_mod):
    orc = oracle_mod.load("oracle")
    g = np.load(os.path.join(GOLDEN, "pointwise.npz"))
    for k in range(len(g["gamma"])):
        rc, f = orc.hllc_2d(g["gamma"][k], g["L"][k], g["R"][k])
        assert rc == g["hllc_rc"][k]
        if rc == 0:
            assert bits_equal(f, g["hllc"][k]), k
    for k in range(len(g["speeds"])):
        rc, f = orc.exact_flux_1d(g["gamma"][k], g["L"][k, [0, 1, 3]], g["R"][k, [0, 1, 3]],
                                  speed=g["speeds"][k])
        assert rc == g["exact_rc"][k]
        if rc == 0:
            assert bits_equal(f, g["exact"][k]), k
    for k in range(len(g["speeds"])):
        L3, R3 = g["L"][k, [0, 1, 3]], g["R"][k, [0, 1, 3]]
        rc, f = orc.hllc_1d(g["gamma"][k], L3, R3)
        assert rc == g["hllc_1d_rc"][k]
        assert bits_equal(f, g["hllc_1d"][k]), k
        rc, s = orc.exact_1d(g["gamma"][k], L3, R3, speed=g["speeds"][k])
        assert rc == g["exact_state_rc"][k]
        assert bits_equal(s, g["exact_state"][k]), k
    for f in (1, 2, 3):
        got = np.array([orc.limit_slope(f, a, b)[1] for a, b in zip(g["lim_a"], g["lim_b"])])
        assert bits_equal(got, g["limited"][f - 1])


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(HERE), "oracle", "_ref",
                                                    "libhydro_ref_omp.so")),
                    reason="reference not compiled in this tree")
def test_restatement_matches_reference_live(oracle_mod):
    O = oracle_mod
    ref, orc = O.load("ref"), O.load("oracle")
    from hydrofv_gb300.problems import random_problem_2d
    for seed, bc, lim in [(21, ("none", "periodic", "transmissive", "none"), "minmod"),
                          (22, ("periodic", "periodic", "reflective", "reflective"), "van_leer"),
                          (23, ("reflective", "none", "periodic", "periodic"), "monotonized_central")]:
        bc = list(bc)
        if "periodic" in bc[:2]:
            bc[0] = bc[1] = "periodic"
        p = random_problem_2d(23, 17, seed, tuple(bc), lim, 12, smooth=(seed % 2 == 0))
        a, b = ref.run_2d(p), orc.run_2d(p)
        assert a.rc == b.rc == 0
        assert bits_equal(a.U, b.U) and bits_equal(a.W, b.W)


def test_library_pointwise_exports_match_golden(hydro_lib):
    """Host builds of the kernels' numerics (exported as the reference's API)."""
    import hydrofv_gb300 as H
    lib = hydro_lib
    g = np.load(os.path.join(GOLDEN, "pointwise.npz"))
    out = [C.c_double() for _ in range(4)]
    worst = 0.0
    for k in range(len(g["gamma"])):
        L, R = g["L"][k], g["R"][k]
        e = lib.solve_flux_hllc_2d(*[C.byref(o) for o in out],
                                   g["gamma"][k], L[0], L[1], L[2], L[3], R[0], R[1], R[2], R[3], 1e-6)
        code, _ = H._consume(lib, e)
        assert (code == 0) == (g["hllc_rc"][k] == 0)
        if code == 0:
            got = np.array([o.value for o in out])
            ref = g["hllc"][k]
            both_nan = np.isnan(got) & np.isnan(ref)
            err = np.abs(got - ref)[~both_nan] / np.maximum(np.abs(ref)[~both_nan], 1e-300)
            if err.size:
                worst = max(worst, float(err.max()))
    # identical algorithm; only libm pow may differ from glibc's by an ulp
    assert worst <= 1e-14
    for k in range(len(g["speeds"])):
        L, R = g["L"][k], g["R"][k]
        e = lib.solve_flux_hllc_1d(*[C.byref(o) for o in out[:3]], g["gamma"][k], L[0], L[1], L[3],
                                   R[0], R[1], R[3], 1e-6)
        code, _ = H._consume(lib, e)
        assert code == g["hllc_1d_rc"][k]
        assert bits_equal(np.array([o.value for o in out[:3]]), g["hllc_1d"][k]), k
        e = lib.solve_exact_1d(*[C.byref(o) for o in out[:3]], g["gamma"][k], L[0], L[1], L[3],
                               R[0], R[1], R[3], 1e-6, g["speeds"][k], 0)
        code, _ = H._consume(lib, e)
        assert code == g["exact_state_rc"][k]
        assert bits_equal(np.array([o.value for o in out[:3]]), g["exact_state"][k]), k
    ip = H.IntegratorParam()
    res = C.c_double()
    for f in (1, 2, 3):
        ip.slope_limiter_flag_ = f
        got = []
        for a, b in zip(g["lim_a"], g["lim_b"]):
            H._consume(lib, lib.limit_slope(C.byref(res), C.byref(ip), a, b))
            got.append(res.value)
        assert bits_equal(np.array(got), g["limited"][f - 1])


import oracle as _O  # noqa: E402

# the exact Sod solution the reference ships, in the staged copy of its tree
SOD_EXACT = os.path.join(_O.REF_EXAMPLES, "sod_shock_1d", "sol_cartesian_1d_0.2.npz")


@pytest.mark.skipif(not os.path.exists(SOD_EXACT), reason="reference tree not present")
def test_sod_accuracy_against_reference_exact_solution(oracle_mod):
    """Accuracy (not parity): first-order Godunov at N=1000 vs the exact Sod solution."""
    O = oracle_mod
    g = np.load(os.path.join(GOLDEN, "sod_1000_godunov_exact.npz"))
    ex = np.load(SOD_EXACT)
    x = O.mid_points(0.0, 1.0, 1000, 2)[2:-2]
    rho = np.interp(x, ex["mid_points"], ex["density"])
    err = np.abs(g["W"][0, 2:-2] - rho).mean()
    assert err < 5e-3, err


@pytest.mark.parametrize("bc,ok", [(("reflective", "periodic"), False), (("periodic", "transmissive"), False),
                                   (("periodic", "periodic"), True)])
def test_periodic_mismatch_rejected_like_the_reference_1d(oracle_mod, bc, ok):
    """A periodic side needs a periodic opposite side (src/boundary.c:258-305):
    the restatement returns the reference's error code and message, and
    agrees with the compiled reference where it exists."""
    O = oracle_mod
    from hydrofv_gb300.problems import random_problem_1d
    p = random_problem_1d(16, 3, bc, "godunov_first_order_1d", "riemann_solver_exact", "minmod", steps=2)
    for b in [O.load("oracle")] + ([O.load("ref_serial")] if O.reference_available() else []):
        r = b.run_1d(p)
        if ok:
            assert r.rc == 0, r.message
        else:
            assert r.rc == 2 and "Periodic boundary condition mismatch for x_min and x_max" in r.message


@pytest.mark.parametrize("bc,which", [(("transmissive", "periodic", "periodic", "periodic"), "x_min and x_max"),
                                      (("periodic", "periodic", "reflective", "periodic"), "y_min and y_max"),
                                      (("reflective", "periodic", "none", "periodic"), "y_min and y_max"),
                                      (("periodic",) * 4, None)])
def test_periodic_mismatch_rejected_like_the_reference_2d(oracle_mod, bc, which):
    O = oracle_mod
    from hydrofv_gb300.problems import random_problem_2d
    p = random_problem_2d(12, 10, 3, bc, "minmod", 2)
    for b in [O.load("oracle")] + ([O.load("ref")] if O.reference_available() else []):
        r = b.run_2d(p)
        if which is None:
            assert r.rc == 0, r.message
        else:
            assert r.rc == 2 and f"Periodic boundary condition mismatch for {which}" in r.message, r.message
    if which is not None:
        # the library rejects it on the host, before any GPU work
        import hydrofv_gb300 as H
        r = H.run_2d(p.nx, p.ny, p.g, (p.x_min, p.x_max, p.y_min, p.y_max), p.gamma, p.W, p.U, bc=p.bc,
                     slope_limiter=p.slope_limiter, max_steps=2)
        assert r.code == 2 and f"Periodic boundary condition mismatch for {which}" in r.message
