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
def test_gpu_division_is_bitwise_ieee():
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
def test_gpu_sqrt_is_bitwise_ieee():
    rng = np.random.default_rng(6)
    x = np.concatenate([_doubles(rng, 1 << 22, 1, 2046, signed=False), _edge_operands(),
                        np.arange(1, 1 << 16, dtype=np.float64) ** 2,
                        np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -1.0])])
    fast, hw, ok = h.gpu_fx_eval(1, x)
    assert _same_bits(fast, hw).all()
    assert _same_bits(hw, np.sqrt(np.where(x < 0, np.nan, x))).all()
    assert ok[:1 << 22].all()
