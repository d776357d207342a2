"""GPU parity of the 2D MUSCL-Hancock + HLLC step against the CPU oracle.

The FP64 drop-in must agree with the reference algorithm to <= 1e-12
relative L1 per conserved field (interior cells) after the stated number of
steps; the tests also report the maximum absolute difference and check the
ghost layers, the status (num_steps, t, dt) and the full padded W.
"""
import numpy as np
import pytest

import hydrofv_gb300 as H

pytestmark = pytest.mark.gpu

REL_L1_TOL = 1e-12


def run_gpu(p, **kw):
    return H.run_2d(p.nx, p.ny, p.g, (p.x_min, p.x_max, p.y_min, p.y_max), p.gamma, p.W, p.U,
                    bc=p.bc, integrator=p.integrator, riemann_solver=p.riemann_solver,
                    slope_limiter=p.slope_limiter, cfl=p.cfl, tf=p.tf, max_steps=p.max_steps,
                    gravity=p.gravity, custom_bc=p.custom_bc, **kw)


def assert_parity(p, gpu, ref, tol=REL_L1_TOL):
    import oracle as O
    assert gpu.code == 0, gpu.message
    assert ref.rc == 0, ref.message
    assert gpu.num_steps == ref.num_steps
    assert abs(gpu.t - ref.t) <= 1e-13 * max(1.0, abs(ref.t))
    assert abs(gpu.dt - ref.dt) <= 1e-12 * abs(ref.dt)
    l1 = O.rel_l1(gpu.U, ref.U, p.g)
    assert np.all(l1 <= tol), f"relative L1 per field {l1}"
    l1w = O.rel_l1(gpu.W, ref.W, p.g)
    assert np.all(l1w <= tol), f"relative L1 of W {l1w}"
    # every padded cell (ghost layers included, corners NaN-aware)
    both_nan = np.isnan(gpu.U) & np.isnan(ref.U)
    assert np.allclose(gpu.U[~both_nan], ref.U[~both_nan], rtol=1e-9, atol=1e-13)
    both_nan = np.isnan(gpu.W) & np.isnan(ref.W)
    assert np.allclose(gpu.W[~both_nan], ref.W[~both_nan], rtol=1e-9, atol=1e-13)
    return l1


@pytest.mark.parametrize("limiter", ["minmod", "van_leer", "monotonized_central"])
def test_shear_layer_small(gpu_available, oracle_mod, limiter):
    O = oracle_mod
    p = O.shear_layer(64, steps=40, limiter=limiter)
    ref = O.load("oracle").run_2d(p)
    gpu = run_gpu(p)
    assert_parity(p, gpu, ref)


@pytest.mark.parametrize("case", ["shear_layer", "point_blast"])
def test_bit_identical_to_the_oracle(gpu_available, oracle_mod, case):
    """The device divide, square root and pow are correctly rounded, like the
    host's (glibc's pow in all but rare cases), so these runs -- the shear
    layer's two-rarefaction faces take three pow each -- reproduce the
    oracle's interior state bit for bit."""
    O = oracle_mod
    p = O.shear_layer(256, steps=100) if case == "shear_layer" else O.point_blast(256, steps=200)
    ref = O.load("oracle").run_2d(p)
    gpu = run_gpu(p)
    assert gpu.code == 0 and ref.rc == 0, gpu.message
    g = p.g
    assert np.array_equal(gpu.U[:, g:-g, g:-g].view(np.uint64), ref.U[:, g:-g, g:-g].view(np.uint64))
    assert np.array_equal(gpu.W[:, g:-g, g:-g].view(np.uint64), ref.W[:, g:-g, g:-g].view(np.uint64))


@pytest.mark.parametrize("case", ["shear_layer", "point_blast"])
def test_headline_workload_bit_identical(gpu_available, oracle_mod, case):
    """The benchmark workload itself -- the 2048 x 2048 shear layer, MC,
    periodic, 200 steps -- through the drop-in call: the interior state, the
    step count and the clock equal the oracle's bit for bit (the oracle takes
    ~15 s on 16 host cores).  Likewise the point blast of the precision study
    (Van Leer, reflective) at 2048 x 2048, 200 steps, the largest size the
    oracle finishes in seconds."""
    O = oracle_mod
    p = O.shear_layer(2048, steps=200) if case == "shear_layer" else O.point_blast(2048, steps=200)
    ref = O.load("oracle").run_2d(p)
    gpu = run_gpu(p)
    assert gpu.code == 0 and ref.rc == 0, gpu.message
    assert gpu.num_steps == ref.num_steps == 200
    assert gpu.t == ref.t and gpu.dt == ref.dt
    g = p.g
    assert np.array_equal(gpu.U[:, g:-g, g:-g].view(np.uint64), ref.U[:, g:-g, g:-g].view(np.uint64))
    assert np.array_equal(gpu.W[:, g:-g, g:-g].view(np.uint64), ref.W[:, g:-g, g:-g].view(np.uint64))


@pytest.mark.parametrize("bc", [("none",) * 4, ("reflective",) * 4, ("transmissive",) * 4,
                                ("reflective", "transmissive", "periodic", "periodic"),
                                ("transmissive", "none", "reflective", "transmissive")])
@pytest.mark.parametrize("shape", [(19, 13), (130, 7), (3, 260)])
def test_boundaries_and_ragged_shapes(gpu_available, oracle_mod, bc, shape):
    O = oracle_mod
    nx, ny = shape
    p = O.random_problem_2d(nx, ny, 11, bc, "monotonized_central", 12, smooth=True)
    ref = O.load("oracle").run_2d(p)
    gpu = run_gpu(p)
    assert_parity(p, gpu, ref)


def test_point_blast_van_leer(gpu_available, oracle_mod):
    O = oracle_mod
    p = O.point_blast(96, steps=60)
    ref = O.load("oracle").run_2d(p)
    gpu = run_gpu(p)
    assert_parity(p, gpu, ref)


def test_run_to_tf(gpu_available, oracle_mod):
    """No step limit: the loop stops on t >= tf with the last dt clipped."""
    O = oracle_mod
    p = O.four_quadrant(40, np.random.default_rng(3), steps=-1)
    p.max_steps = -1
    p.tf = 0.05
    ref = O.load("oracle").run_2d(p)
    gpu = run_gpu(p)
    assert ref.t == pytest.approx(0.05)
    assert_parity(p, gpu, ref)


# ----------------------------------------------------------- gravity, custom sides

GOLDEN = __import__("os").path.join(__import__("os").path.dirname(__import__("os").path.abspath(__file__)),
                                     "golden")


@pytest.mark.parametrize("integrator", ["muscl_hancock_2d", "godunov_first_order_2d"])
def test_gravity_source_rayleigh_taylor(gpu_available, oracle_mod, integrator):
    """The gravity source (RK4 kick after the step, src/source_term.c:185-259)
    on the Rayleigh-Taylor example's set-up (G = 3, periodic x, reflective y)."""
    O = oracle_mod
    p = O.rayleigh_taylor(40, 64, g=3, steps=80)
    p.integrator = integrator
    gpu = run_gpu(p)
    ref = O.load("oracle").run_2d(p)
    l1 = assert_parity(p, gpu, ref)
    assert np.all(l1 == 0.0), l1


def test_custom_side_lid_cavity(gpu_available, oracle_mod):
    """A custom side: the lid-driven cavity's top callback runs on the host
    after every step and its ghost rows feed the next step."""
    O = oracle_mod
    p = O.lid_driven_cavity(48, g=3, steps=80)
    gpu = run_gpu(p)
    ref = O.load("oracle").run_2d(p)
    # <= 1e-12 relative L1; the lid drives two-rarefaction faces, whose pow
    # may differ from the CPU's by an ulp
    assert_parity(p, gpu, ref)
    # the lid rows hold the callback's velocity
    assert np.all(gpu.W[1, p.g + p.ny:, :] == 10.0)


@pytest.mark.parametrize("name", ["rayleigh_taylor_24x40_g3_30", "lid_cavity_32_g3_30"])
def test_gravity_and_custom_against_reference_golden(gpu_available, name):
    """Against the unmodified reference's outputs (committed fixtures)."""
    import os
    import sys
    sys.path.insert(0, GOLDEN)
    import make_golden as MG
    p = MG.cases_2d()[name]
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    gpu = run_gpu(p)
    assert gpu.code == 0, gpu.message
    assert gpu.num_steps == int(g["num_steps"]) and gpu.t == float(g["t"])
    import oracle as O
    assert np.all(O.rel_l1(gpu.U, g["U"], p.g) <= REL_L1_TOL)
    assert np.all(O.rel_l1(gpu.W, g["W"], p.g) <= REL_L1_TOL)


def test_custom_side_session_in_chunks(gpu_available, oracle_mod):
    """The device-resident session with a custom side, advanced in two calls."""
    O = oracle_mod
    p = O.lid_driven_cavity(40, g=3, steps=50)
    with H.Solver2D(p.nx, p.ny, p.g, (p.x_min, p.x_max, p.y_min, p.y_max), p.gamma, p.W, p.U,
                    bc=p.bc, slope_limiter=p.slope_limiter, cfl=p.cfl, custom_bc=p.custom_bc) as s:
        s.advance(20)
        st, _ = s.advance(30)
        assert st.num_steps == 50
        W, U = s.download()
    ref = O.load("oracle").run_2d(p)
    assert np.all(O.rel_l1(U, ref.U, p.g) <= REL_L1_TOL)
    assert np.all(O.rel_l1(W, ref.W, p.g) <= REL_L1_TOL)


def test_fp32_gravity_and_custom_rejection(gpu_available, oracle_mod):
    O = oracle_mod
    p = O.rayleigh_taylor(32, 48, g=3, steps=40)
    r64 = run_gpu(p)
    r32 = run_gpu(p, options=H.default_options(precision=H.PRECISION_FP32))
    assert r32.code == 0, r32.message
    l1 = O.rel_l1(r32.U, r64.U, p.g)
    assert l1[0] < 1e-6 and l1[3] < 1e-6, l1     # mass and energy (the velocities start at 0)
    q = O.lid_driven_cavity(16, g=3, steps=4)
    r = run_gpu(q, options=H.default_options(precision=H.PRECISION_FP32))
    assert r.code != 0 and "FP64" in r.message


# ----------------------------------------------------------- the reference itself

@pytest.mark.parametrize("case", ["shear_layer", "point_blast", "four_quadrant", "godunov_periodic"])
def test_against_the_compiled_reference(gpu_available, oracle_mod, case):
    """The GPU run against the unmodified reference, compiled on this machine
    from its staged sources (oracle/_ref), not only against the
    restatement: interior state, step count and clock bit for bit."""
    O = oracle_mod
    if not O.reference_available():
        pytest.skip("reference not compiled here (make -C oracle stage ref)")
    if case == "shear_layer":
        p = O.shear_layer(256, steps=60)
    elif case == "point_blast":
        p = O.point_blast(192, steps=80)
    elif case == "four_quadrant":
        p = O.four_quadrant(128, np.random.default_rng(4), steps=60)
    else:
        p = O.random_problem_2d(70, 50, 9, ("periodic",) * 4, "minmod", 30, smooth=True,
                                integrator="godunov_first_order_2d")
    ref = O.load("ref").run_2d(p)
    gpu = run_gpu(p)
    assert gpu.code == 0 and ref.rc == 0, (gpu.message, ref.message)
    assert gpu.num_steps == ref.num_steps and gpu.t == ref.t and gpu.dt == ref.dt
    g = p.g
    if case == "four_quadrant":
        # two-rarefaction faces take pow; glibc's misrounds ~0.1% of them
        assert np.all(O.rel_l1(gpu.U, ref.U, g) <= REL_L1_TOL)
    else:
        assert np.array_equal(gpu.U[:, g:-g, g:-g].view(np.uint64), ref.U[:, g:-g, g:-g].view(np.uint64))
        assert np.array_equal(gpu.W[:, g:-g, g:-g].view(np.uint64), ref.W[:, g:-g, g:-g].view(np.uint64))


def test_repeated_launches_reuse_device_memory(gpu_available, oracle_mod):
    """Consecutive launches take their state from the device memory the
    previous one handed back to the library's pool (no fresh mapping each
    call): results stay identical across calls, and after
    hydro_gpu_trim_device_memory hands the cache back, the next call
    allocates again and still agrees."""
    O = oracle_mod
    p = O.shear_layer(96, steps=25)
    ref = O.load("oracle").run_2d(p)
    outs = [run_gpu(p) for _ in range(3)]
    assert H.library().hydro_gpu_trim_device_memory(0) == 0
    outs.append(run_gpu(p))
    for gpu in outs:
        assert gpu.code == 0 and gpu.num_steps == ref.num_steps
        assert np.array_equal(gpu.U, outs[0].U, equal_nan=True)
        assert np.array_equal(gpu.W, outs[0].W, equal_nan=True)   # corners: NaN
    assert_parity(p, outs[0], ref)


def test_concurrent_launches_from_two_host_threads(gpu_available, oracle_mod):
    """Two host threads calling the drop-in at once (ctypes releases the GIL
    for the call) on different Systems: each run takes its own stream,
    control blocks and pool memory, and both results equal the sequential
    ones bit for bit."""
    import threading
    O = oracle_mod
    probs = [O.shear_layer(160, steps=30), O.point_blast(144, steps=40)]
    seq = [run_gpu(p) for p in probs]
    out = [None, None]

    def work(k):
        out[k] = [run_gpu(probs[k]) for _ in range(3)]

    threads = [threading.Thread(target=work, args=(k,)) for k in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for k in range(2):
        for r in out[k]:
            assert r.code == 0, r.message
            assert r.num_steps == seq[k].num_steps and r.t == seq[k].t
            assert np.array_equal(r.U, seq[k].U, equal_nan=True)
            assert np.array_equal(r.W, seq[k].W, equal_nan=True)


@pytest.mark.parametrize("g", [3, 4])
@pytest.mark.parametrize("limiter", ["minmod", "van_leer", "monotonized_central"])
def test_wider_ghost_layers(gpu_available, oracle_mod, g, limiter):
    """More ghost layers than MUSCL-Hancock needs (the reference allows any
    G >= 2): the boundary remap of every built-in side and the one-sided
    update of the first ghost layer at G = 3 and 4."""
    O = oracle_mod
    p = O.random_problem_2d(37, 29, 5 + g, ("reflective", "transmissive", "periodic", "periodic"),
                            limiter, 15, g=g, smooth=True)
    ref = O.load("oracle").run_2d(p)
    gpu = run_gpu(p)
    assert_parity(p, gpu, ref)


@pytest.mark.parametrize("nx", [125, 126, 127, 252, 253])
def test_strip_edges(gpu_available, oracle_mod, nx):
    """Grid widths around the step kernel's strip width (126 interior
    columns per CTA): a last strip of one, two or no extra columns, with a
    short grid so the row chunks are ragged too."""
    O = oracle_mod
    p = O.random_problem_2d(nx, 21, nx, ("transmissive", "reflective", "none", "reflective"),
                            "monotonized_central", 12, smooth=True)
    ref = O.load("oracle").run_2d(p)
    gpu = run_gpu(p)
    assert_parity(p, gpu, ref)
