"""Integer-pipe FP64 division and square root (fp64_int.cuh).

The FP64 kernels compute a / b and sqrt(x) with integer multiplies and an
exact remainder check instead of the FP64 pipe's FMA sequences; the results
must be the IEEE round-to-nearest-even values bit for bit.  The host build of
the same code (host FP32 seeds) is checked here on the CPU against numpy's
IEEE operations; the device build is checked on the GPU against both the
hardware operations and numpy.
"""
import numpy as np
import pytest

import hydrofv_gb300 as h

SIGN = np.uint64(0x8000000000000000)


def _doubles(rng, n, emin, emax, signed=True):
    """Random normal doubles with exponents uniform in [emin, emax] (biased)."""
    frac = rng.integers(0, 1 << 52, size=n, dtype=np.uint64)
    exp = rng.integers(emin, emax + 1, size=n).astype(np.uint64)
    b = (exp << np.uint64(52)) | frac
    if signed:
        b |= rng.integers(0, 2, size=n, dtype=np.uint64) << np.uint64(63)
    return b.view(np.float64)


def _same_bits(x, y):
    xb, yb = x.view(np.uint64), y.view(np.uint64)
    return (xb == yb) | (np.isnan(x) & np.isnan(y))


def _edge_mantissas():
    """Mantissa patterns that stress the rounding: powers of two, all ones,
    near-halves, alternating bits, and their neighbours."""
    pats = [0, 1, 2, (1 << 52) - 1, (1 << 52) - 2, 1 << 51, (1 << 51) - 1, (1 << 51) + 1,
            0x5555555555555, 0xAAAAAAAAAAAAA, 0x0000000000001, 0xFFFFFFFFFFFFE, 0x8000000000001]
    return np.array(pats, dtype=np.uint64)


def _edge_operands():
    m = _edge_mantissas()
    vals = []
    for e in (1, 2, 500, 1022, 1023, 1024, 1500, 2045, 2046):
        vals.append(((np.uint64(e) << np.uint64(52)) | m).view(np.float64))
    v = np.concatenate(vals)
    return np.concatenate([v, -v])


def _expected_fast_div(a, b):
    """Where the fast path must apply: normal b, and a zero or normal with a
    quotient exponent (before rounding) inside the normal range."""
    ab, bb = a.view(np.uint64), b.view(np.uint64)
    ea = ((ab >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    eb = ((bb >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    ma = (ab & np.uint64((1 << 52) - 1))
    mb = (bb & np.uint64((1 << 52) - 1))
    e = ea - eb + 1023 - (ma < mb).astype(np.int64)
    a_zero = (ab << np.uint64(1)) == 0
    b_norm = (eb >= 1) & (eb <= 2046)
    return b_norm & (a_zero | ((ea >= 1) & (ea <= 2046) & (e >= 1) & (e <= 2046)))


def test_host_division_matches_ieee_on_random_operands():
    rng = np.random.default_rng(1)
    n = 1 << 20
    a = _doubles(rng, n, 900, 1150)
    b = _doubles(rng, n, 900, 1150)
    out, ok = h.fx_eval_host(0, a, b)
    assert ok.all()
    with np.errstate(all="ignore"):
        ref = a / b
    assert _same_bits(out, ref).all()


def test_host_division_full_exponent_range_and_fallback_set():
    rng = np.random.default_rng(2)
    n = 1 << 20
    a = _doubles(rng, n, 0, 2047)
    b = _doubles(rng, n, 0, 2047)
    out, ok = h.fx_eval_host(0, a, b)
    with np.errstate(all="ignore"):
        ref = a / b
    assert np.array_equal(ok, _expected_fast_div(a, b))
    assert _same_bits(out[ok], ref[ok]).all()


def test_host_division_edge_mantissas_and_exponents():
    v = _edge_operands()
    a = np.repeat(v, v.size)
    b = np.tile(v, v.size)
    out, ok = h.fx_eval_host(0, a, b)
    with np.errstate(all="ignore"):
        ref = a / b
    assert np.array_equal(ok, _expected_fast_div(a, b))
    assert _same_bits(out[ok], ref[ok]).all()
    # quotients that round up to the overflow threshold become infinities
    big = np.array([np.finfo(np.float64).max] * 3)
    den = np.array([1.0 - 2.0 ** -53 * 3, np.nextafter(1.0, 0.0), 0.5])
    out, ok = h.fx_eval_host(0, big, den)
    with np.errstate(all="ignore"):
        ref = big / den
    assert _same_bits(out[ok], ref[ok]).all()


def test_host_division_exact_quotients_and_zero_numerators():
    rng = np.random.default_rng(3)
    q = rng.integers(1, 1 << 26, size=4096).astype(np.float64)
    d = rng.integers(1, 1 << 26, size=4096).astype(np.float64)
    a = q * d                                   # exact: < 2^52
    out, ok = h.fx_eval_host(0, a, d)
    assert ok.all() and np.array_equal(out, q)
    z = np.array([0.0, -0.0, 0.0, -0.0])
    den = np.array([3.0, 3.0, -3.0, -3.0])
    out, ok = h.fx_eval_host(0, z, den)
    assert ok.all() and np.array_equal(out.view(np.uint64), (z / den).view(np.uint64))


def test_host_division_seed_check_catches_bad_seeds():
    """The divide trusts its FP32 reciprocal seed only when the seed's exact
    residual is small; a perturbed seed either still gives RN(a/b) or takes
    the fallback, never a wrong quotient.  Mantissas near 2 are included
    (their reciprocal seed sits at 0.5, where a low seed changes scale)."""
    rng = np.random.default_rng(31)
    n = 1 << 19
    a = _doubles(rng, n, 1000, 1050)
    b = _doubles(rng, n, 1000, 1050)
    b[: n // 8] = np.nextafter(2.0 ** rng.integers(-20, 20, n // 8), 0.0) * rng.choice([1.0, -1.0], n // 8)
    with np.errstate(all="ignore"):
        ref = a / b
    for spread in (2.0 ** -23, 2.0 ** -21.5, 2.0 ** -20, 2.0 ** -16, 0.5):
        scale = (1.0 + rng.uniform(-spread, spread, n)).astype(np.float32)
        out, ok = h.fx_div_seeded_host(a, b, scale)
        assert _same_bits(out[ok], ref[ok]).all(), spread
        if spread <= 2.0 ** -23:
            assert ok.all()
    for far in (0.75, 1.3):                                  # seeds off by 25-30%
        out, ok = h.fx_div_seeded_host(a, b, np.full(n, far, dtype=np.float32))
        assert not ok.any()


def test_host_division_special_operands_take_the_fallback():
    sp = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -2.2e-308, 1.0])
    a = np.repeat(sp, sp.size)
    b = np.tile(sp, sp.size)
    _, ok = h.fx_eval_host(0, a, b)
    assert np.array_equal(ok, _expected_fast_div(a, b))


def test_host_sqrt_matches_ieee():
    rng = np.random.default_rng(4)
    x = _doubles(rng, 1 << 20, 1, 2046, signed=False)
    out, ok = h.fx_eval_host(1, x)
    assert ok.all()
    assert _same_bits(out, np.sqrt(x)).all()
    v = _edge_operands()
    v = v[v > 0]
    sq = np.arange(1, 1 << 16, dtype=np.float64) ** 2   # perfect squares
    for x in (v, sq, sq * 4.0, sq * 2.0 ** -600, np.nextafter(sq, 0.0), np.nextafter(sq, np.inf)):
        out, ok = h.fx_eval_host(1, x)
        assert ok.all()
        assert _same_bits(out, np.sqrt(x)).all()


def test_host_sqrt_special_operands_take_the_fallback():
    sp = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, 2.3e-308, -1.0, 1.0, 4.0])
    _, ok = h.fx_eval_host(1, sp)
    assert np.array_equal(ok, [False, False, False, False, False, False, True, False, True, True])


@pytest.mark.gpu
def test_gpu_division_is_bitwise_ieee(gpu_available):
    rng = np.random.default_rng(5)
    n = 1 << 22
    sets = [(_doubles(rng, n, 900, 1150), _doubles(rng, n, 900, 1150)),
            (_doubles(rng, n, 0, 2047), _doubles(rng, n, 0, 2047))]
    v = _edge_operands()
    sets.append((np.repeat(v, v.size), np.tile(v, v.size)))
    sp = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -2.2e-308, 1.0, 3.0])
    sets.append((np.repeat(sp, sp.size), np.tile(sp, sp.size)))
    for a, b in sets:
        fast, hw, ok = h.gpu_fx_eval(0, a, b)
        with np.errstate(all="ignore"):
            ref = a / b
        assert _same_bits(fast, hw).all()
        assert _same_bits(hw, ref).all()
        assert np.array_equal(ok, _expected_fast_div(a, b))


@pytest.mark.gpu
def test_gpu_sqrt_is_bitwise_ieee(gpu_available):
    rng = np.random.default_rng(6)
    x = np.concatenate([_doubles(rng, 1 << 22, 1, 2046, signed=False), _edge_operands(),
                        np.arange(1, 1 << 16, dtype=np.float64) ** 2,
                        np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -1.0])])
    fast, hw, ok = h.gpu_fx_eval(1, x)
    assert _same_bits(fast, hw).all()
    assert _same_bits(hw, np.sqrt(np.where(x < 0, np.nan, x))).all()
    assert ok[:1 << 22].all()


# ---------------------------------------------------------------- pow

# exponents the solvers use: (g-1)/2g, 2g/(g-1), 2/(g-1), g, 1/g, (g-1)/2g,
# -(g+1)/2g for g = 1.4 and 5/3
SOLVER_EXPONENTS = [0.2 / 1.4, 1.4 / 0.2, 2 / 0.4, 1.4, 1 / 1.4, 0.4 / 2.8, -2.4 / 2.8,
                    (1 / 3) / (5 / 3), (5 / 3) / (1 / 3), 2 / (2 / 3), 5 / 3, 0.6, -(8 / 3) / (10 / 3)]


def _correctly_rounded_pow(x, y):
    mp = pytest.importorskip("mpmath")
    mp.mp.prec = 200
    return np.array([float(mp.power(mp.mpf(a), mp.mpf(b))) for a, b in zip(x, y)])


def test_host_pow_is_correctly_rounded_on_solver_exponents():
    rng = np.random.default_rng(11)
    x = np.exp(rng.uniform(-12, 12, 1500 * len(SOLVER_EXPONENTS)))
    y = np.repeat(SOLVER_EXPONENTS, 1500)
    out, ok = h.fx_eval_host(2, x, y)
    assert ok.all()
    assert np.array_equal(out.view(np.uint64), _correctly_rounded_pow(x, y).view(np.uint64))


def test_host_pow_is_correctly_rounded_on_wide_operands():
    rng = np.random.default_rng(12)
    x = np.concatenate([np.exp(rng.uniform(-700, 700, 6000)), rng.uniform(0.5, 2.0, 6000),
                        1.0 + rng.uniform(-1e-9, 1e-9, 2000)])
    y = np.concatenate([rng.uniform(-1, 1, 6000), rng.uniform(-40, 40, 6000), rng.uniform(-500, 500, 2000)])
    out, ok = h.fx_eval_host(2, x, y)
    assert ok.mean() > 0.99
    ref = _correctly_rounded_pow(x[ok], y[ok])
    assert np.array_equal(out[ok].view(np.uint64), ref.view(np.uint64))


def test_host_pow_table_boundaries_and_exact_results():
    x = np.array([1.0 + k / 128 for k in range(129)] + [np.nextafter(1.0 + k / 128, 0) for k in range(1, 129)]
                 + [1.0 + (2 * k + 1) / 256 for k in range(128)] + [np.nextafter(1.0, 2.0), np.nextafter(1.0, 0.0)])
    for yv in (0.2, 7.0, -3.5, 0.5, 100.0, -300.0, 511.0):
        y = np.full(x.size, yv)
        out, ok = h.fx_eval_host(2, x, y)
        with np.errstate(all="ignore"):
            normal = np.abs(np.log2(x) * yv) < 1020      # results that stay normal
        assert ok[normal].mean() > 0.95 and not ok[~normal].any()   # short mantissas: midpoints
        ref = _correctly_rounded_pow(x[ok], y[ok])
        assert np.array_equal(out[ok].view(np.uint64), ref.view(np.uint64))
    # exact powers come out exact
    out, ok = h.fx_eval_host(2, np.array([4.0, 2.0, 9.0, 0.25, 1024.0, 1.0]), np.array([0.5, 10.0, 0.5, -2.0, 0.1, 123.4]))
    assert ok.all() and np.array_equal(out, [2.0, 1024.0, 3.0, 16.0, 2.0, 1.0])


def test_host_pow_agrees_with_the_c_library_pow():
    """glibc's pow (what the reference calls) is correctly rounded in all but
    a small fraction of cases; where it differs, by one ulp."""
    import ctypes
    import ctypes.util
    libm = ctypes.CDLL(ctypes.util.find_library("m"))
    libm.pow.restype = ctypes.c_double
    libm.pow.argtypes = [ctypes.c_double, ctypes.c_double]
    rng = np.random.default_rng(13)
    x = np.exp(rng.uniform(-6, 6, 4000 * len(SOLVER_EXPONENTS)))
    y = np.repeat(SOLVER_EXPONENTS, 4000)
    out, ok = h.fx_eval_host(2, x, y)
    assert ok.all()
    ref = np.array([libm.pow(a, b) for a, b in zip(x, y)])
    d = np.abs(out.view(np.int64) - ref.view(np.int64))
    assert d.max() <= 1
    assert (d != 0).mean() < 5e-3


def test_host_pow_special_operands_take_the_fallback():
    x = np.array([0.0, -1.0, np.inf, np.nan, 5e-324, 2.0, 2.0, 2.0, 2.0, 1e300, 1e-300, 2.0, 2.0])
    y = np.array([2.0, 2.0, 2.0, 2.0, 2.0, 0.0, 512.0, 1023.9, -1022.5, 2.0, 2.0, np.nan, 1e-320])
    _, ok = h.fx_eval_host(2, x, y)
    assert not ok.any()


@pytest.mark.gpu
def test_gpu_pow_matches_the_host_build_bitwise(gpu_available):
    """The device build is the same integer algorithm (no seeds): bit-identical
    to the host build wherever its fast path applies; elsewhere it is the
    hardware pow."""
    rng = np.random.default_rng(14)
    x = np.concatenate([np.exp(rng.uniform(-12, 12, 1 << 21)), np.exp(rng.uniform(-700, 700, 1 << 20)),
                        np.array([0.0, -1.0, np.inf, np.nan, 5e-324, 2.0, 2.0, 1e300])])
    y = np.concatenate([rng.choice(SOLVER_EXPONENTS, 1 << 21), rng.uniform(-1, 1, 1 << 20),
                        np.array([2.0, 2.0, 2.0, 2.0, 2.0, 0.0, 512.0, 2.0])])
    fast, hw, ok = h.gpu_fx_eval(2, x, y)
    host, hok = h.fx_eval_host(2, x, y)
    assert np.array_equal(ok, hok)
    assert np.array_equal(fast[ok].view(np.uint64), host[ok].view(np.uint64))
    assert _same_bits(fast[~ok], hw[~ok]).all()
    # the hardware pow is within a few ulps of the correctly rounded result
    d = np.abs(fast[ok].view(np.int64) - hw[ok].view(np.int64))
    assert d.max() <= 4


# ---------------------------------------------------------------- limiters

def _slope_pairs(rng, n):
    """Slope pairs: same and opposite signs over a wide range, ties, zeros of
    both signs, infinities, NaN, subnormals and products near underflow."""
    a = rng.normal(size=n) * 10.0 ** rng.uniform(-30, 30, n)
    b = rng.normal(size=n) * 10.0 ** rng.uniform(-30, 30, n)
    b[: n // 8] = a[: n // 8] * rng.choice([1.0, 2.0, 0.5, -1.0], n // 8)        # ties and MC kinks
    sp = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -2e-310, 1e-160, -3e-170, 1e300, 2.0])
    a = np.concatenate([a, np.repeat(sp, sp.size)])
    b = np.concatenate([b, np.tile(sp, sp.size)])
    return a, b


def test_host_bit_sign_test_matches_the_product():
    rng = np.random.default_rng(21)
    a, b = _slope_pairs(rng, 200000)
    t, _ = h.fx_eval_host(6, a, b)
    with np.errstate(all="ignore"):
        ref = a * b <= 0.0
    decided = t >= 0
    assert np.array_equal(t[decided] == 1, ref[decided])
    assert decided[:200000].mean() > 0.99
    finite = np.isfinite(a) & np.isfinite(b)
    assert not decided[~finite & ((a != 0) | ~np.isfinite(b)) & ((b != 0) | ~np.isfinite(a))].any()


@pytest.mark.gpu
@pytest.mark.parametrize("op", [3, 4, 5], ids=["minmod", "van_leer", "mc"])
def test_gpu_limiters_match_the_fp64_expressions(gpu_available, op):
    """The device limiters decide the sign test and the minima on the bits;
    the results are the host build's FP64 expressions bit for bit."""
    rng = np.random.default_rng(22 + op)
    a, b = _slope_pairs(rng, 1 << 21)
    fast, _, ok = h.gpu_fx_eval(op, a, b)
    host, _ = h.fx_eval_host(op, a, b)
    assert _same_bits(fast, host).all()
    assert ok[: 1 << 21].mean() > 0.99


def test_pow_tables_match_their_generator():
    """pow_tables.h is generated by gen_pow_tables.py (300-bit mpmath); the
    committed header must be exactly its output."""
    pytest.importorskip("mpmath")
    import contextlib
    import importlib.util
    import io
    import os
    here = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "hydrofv_gb300", "csrc", "gpu")
    spec = importlib.util.spec_from_file_location("gen_pow_tables", os.path.join(here, "gen_pow_tables.py"))
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        gen.main()
    with open(os.path.join(here, "pow_tables.h")) as f:
        assert buf.getvalue() == f.read()


def test_convergence_test_without_divide():
    """The exact solver's convergence test RN(x / y) < tol, decided by two
    multiplies where a margin allows: wherever it decides, the answer is that
    of the IEEE divide, including quotients within a few ulps of tol."""
    rng = np.random.default_rng(12)
    n = 400_000
    tols = np.concatenate([np.full(n // 2, 1e-6), 10.0 ** rng.uniform(-12, -1, n // 2)])
    y = 10.0 ** rng.uniform(-6, 6, n)
    # quotients spread around tol, many within a few ulps of it
    k = rng.integers(-40, 41, n)
    q = tols * (1.0 + k * 2.0 ** -52) * np.where(rng.random(n) < 0.5, 1.0, 10.0 ** rng.uniform(-3, 3, n))
    x = q * y
    x[:1000] = 0.0
    out, dec = h.fx_ratio_below_host(x, y, tols)
    ref = (x / y) < tols
    assert np.array_equal(out[dec], ref[dec])
    assert dec.mean() > 0.8
    # outside the guarded range nothing is decided
    _, d2 = h.fx_ratio_below_host(np.array([1.0, np.nan, 1e301]), np.array([1e-300, 1.0, 1.0]),
                                  np.array([1e-6, 1e-6, 1e-6]))
    assert not d2.any()


def test_vacuum_test_without_divide():
    """The solvers' vacuum-generation test RN(2 (a_L + a_R) / (gamma + 1)) <=
    u_R - u_L, decided from the exponents without the divide: wherever it
    decides, the answer is that of the IEEE divide, including quotients within
    a few ulps of z (which it must leave undecided)."""
    rng = np.random.default_rng(13)
    n = 400_000
    y = rng.choice([2.4, 8.0 / 3.0, 2.2], n)
    x = 2.0 * (10.0 ** rng.uniform(-3, 2, n))
    k = rng.integers(-40, 41, n)
    z = (x / y) * (1.0 + k * 2.0 ** -52)
    z[: n // 4] = rng.uniform(-3, 3, n // 4)            # typical velocity jumps
    z[n // 4: n // 4 + 1000] = 0.0
    z[n // 4 + 1000: n // 4 + 2000] = -0.0
    x[:500] = 0.0
    out, dec = h.fx_quot_le_host(x, y, z)
    ref = (x / y) <= z
    assert np.array_equal(out[dec], ref[dec])
    assert dec[: n // 4].mean() > 0.9
    # NaN and infinite operands and a zero z are left to the divide; a tiny
    # normal z is decided by its exponent
    xs = np.array([np.nan, 1.0, np.inf, 1.0, 1.0, 1.0, 0.0])
    zs = np.array([1.0, np.nan, 1.0, 0.0, -0.0, 1e-300, 1.0])
    o2, d2 = h.fx_quot_le_host(xs, 2.4, zs)
    assert d2.tolist() == [False, False, False, False, False, True, False]
    assert not o2[5]
