/*
 * fp64_int.cuh -- correctly rounded FP64 division and square root on the
 * integer pipes.
 *
 * GB300 retires FP64 at 2 lanes/clk/SM against 128 for FP32 and INT32, and
 * the FP64 MUSCL-Hancock step is bound by its FP64 pipe, which in turn is
 * mostly busy with the FMA sequences behind '/' and sqrt.  The functions
 * here compute the same IEEE-754 round-to-nearest-even results with 32/64-bit
 * integer multiplies (IMAD) and one FP32 MUFU seed, leaving the FP64 pipe to
 * the additions and multiplications of the scheme.
 *
 * Division a / b of normal operands (mantissas ma, mb in [2^52, 2^53)):
 *   1. y0 ~ 1/mb from the FP32 reciprocal of mb's leading 24 bits
 *      (relative error ~2^-22), as a 32-bit fixed-point Y0 ~ 2^84/mb;
 *   2. one Newton step in integer arithmetic, Y1 = Y0 (1 + e0) with the
 *      exact residual e0 = 1 - mb Y0 2^-84; Y1 <= 2^116/mb and its relative
 *      error is ~e0^2 ~ 2^-44;
 *   3. the quotient Q = floor(ma 2^(52+s) / mb) (s = [ma < mb], so Q has 53
 *      bits) by a multiply-high with Y1, one correction by the remainder
 *      times Y1, and one single-step fix, which make Q exact whenever the
 *      seed's residual is small (|e0| < 3 2^61, checked; the bounds are in
 *      div_fast);
 *   4. round-to-nearest-even on the remainder (2R against mb).
 * This is the reciprocal-multiply-and-correct form of long division
 * (Knuth, TAOCP vol. 2, 4.3.1; Moller & Granlund, "Improved division by
 * invariant integers", IEEE TC 2011) applied to the 53-bit mantissas.
 *
 * Square root of a normal positive x (mantissa m, M = m or 2m so that the
 * exponent left over is even, M in [2^52, 2^54)):
 *   1. y0 ~ 1/sqrt(M 2^-52) from the FP32 reciprocal square root, Y0 = y0 2^32;
 *   2. one integer Newton step for the reciprocal square root,
 *      Y1 = Y0 (1 + e0/2), e0 = 1 - M 2^-52 y0^2, which stays below the exact
 *      value (1/sqrt(1-e) >= 1 + e/2);
 *   3. S1 = M Y1 2^-64 <= sqrt(M 2^52), one Heron correction with the exact
 *      integer residual M 2^52 - S1^2, at most two single-step fixes;
 *   4. an exact 128-bit check that 0 <= M 2^52 - S^2 <= 2S, then rounding
 *      up where the residual exceeds S (a square root is never a midpoint).
 *
 * Correctness does not rest on the seed's accuracy: the divide checks the
 * seed's exact residual, the square root verifies its result exactly, and
 * every operand or result outside the fast path
 * (zero, subnormal, infinite, NaN, negative for sqrt, quotients that
 * overflow the normal range before rounding or underflow) or a failed check
 * takes the hardware operation.  The results are therefore bit-identical to
 * '/' and sqrt.  Host builds keep the plain operators; the integer forms are
 * also compiled for the host (with host seeds) so that they can be checked
 * against the host's IEEE operations on the CPU.
 *
 * The same file holds the other FP64-pipe savings of the step kernel, each
 * exact: the slope limiter's sign test on the bits (product_nonpositive),
 * ordered comparisons (lt, le), and the reference's "+ 0.0" terms
 * (add_zero, zero_minus).  All of them read a double's bits through an
 * opaque move (bits): with a plain bitcast the compiler recognises zero,
 * sign and exponent tests as floating-point class tests and emits FP64
 * compares again.  The divide and square root run out of line on the device
 * (div_dev, sqrt_dev), one copy per kernel: inlined at the step kernel's ~40
 * call sites they overflow the instruction cache.
 */
#ifndef HYDRO_GPU_FP64_INT_CUH
#define HYDRO_GPU_FP64_INT_CUH

#include <math.h>
#include <string.h>

#ifdef __CUDACC__
#define FXHD __host__ __device__ __forceinline__
#else
#define FXHD static inline
#endif

namespace hydro {
namespace fx {

typedef unsigned long long u64;
typedef long long i64;

/* The bits of a double.  On the device through an opaque move: a plain
 * bitcast lets the compiler recognise the bit tests below (zero, exponent
 * range, sign) as floating-point class tests and emit them as FP64 compares
 * on the FP64 pipe, which is what these forms exist to avoid. */
FXHD u64 bits(double x)
{
#if defined(__CUDA_ARCH__)
    u64 u;
    asm("mov.b64 %0, %1;" : "=l"(u) : "d"(x));
    return u;
#else
    u64 b;
    memcpy(&b, &x, sizeof b);
    return b;
#endif
}

FXHD double from_bits(u64 b)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((i64) b);
#else
    double x;
    memcpy(&x, &b, sizeof x);
    return x;
#endif
}

FXHD unsigned fbits(float x)
{
#if defined(__CUDA_ARCH__)
    return (unsigned) __float_as_uint(x);
#else
    unsigned b;
    memcpy(&b, &x, sizeof b);
    return b;
#endif
}

FXHD float from_fbits(unsigned b)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float(b);
#else
    float x;
    memcpy(&x, &b, sizeof x);
    return x;
#endif
}

FXHD u64 mulhi(u64 a, u64 b)
{
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (u64) (((unsigned __int128) a * b) >> 64);
#endif
}

/* FP32 seeds: reciprocal and reciprocal square root of x in [1, 4). */
FXHD float rcp_seed(float x)
{
#if defined(__CUDA_ARCH__)
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
#else
    return 1.0f / x;
#endif
}

FXHD float rsqrt_seed(float x)
{
#if defined(__CUDA_ARCH__)
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
#else
    return 1.0f / sqrtf(x);
#endif
}

/* y in [0.5, 1] (an FP32 seed) as a 32-bit fixed-point value y 2^32,
 * saturated at 2^32 - 1.  Seeds outside [0.5, 1] give a poor estimate,
 * which the exact check turns into the fallback. */
FXHD unsigned seed_fixed(float y)
{
    const unsigned fy = fbits(y);
    return (fy >= 0x3f800000u) ? 0xffffffffu : (((fy & 0x7fffffu) | 0x800000u) << 8);
}

static const u64 FRAC = 0x000fffffffffffffull;
static const u64 HIDDEN = 0x0010000000000000ull;
static const u64 SIGN = 0x8000000000000000ull;

/* RN(a / b) when `ok` comes back true (see the header comment).
 * seed_scale multiplies the FP32 reciprocal seed: 1 in the kernels; the
 * tests perturb it to exercise the seed check. */
FXHD double div_fast(double a, double b, bool &ok, float seed_scale = 1.0f)
{
    const u64 ua = bits(a), ub = bits(b);
    const unsigned ea = (unsigned) (ua >> 52) & 0x7ffu, eb = (unsigned) (ub >> 52) & 0x7ffu;
    const u64 sign = (ua ^ ub) & SIGN;
    const u64 ma = (ua & FRAC) | HIDDEN, mb = (ub & FRAC) | HIDDEN;
    const int s = ma < mb ? 1 : 0;
    const int e = (int) ea - (int) eb + 1023 - s;          /* biased exponent of the quotient */

    const unsigned Y0 = seed_fixed(rcp_seed(from_fbits(0x3f800000u | (unsigned) ((mb >> 29) & 0x7fffffu))) * seed_scale);
    /* mb Y0 (85 bits) from two 32 x 32 products.  Its low 64 bits, negated,
     * are the residual e0 = 2^84 - mb Y0 exactly when the high bits are
     * 2^20 - 1 with e0 > 0, or 2^20 with e0 <= 0 (so |2^84 - mb Y0| < 2^63) */
    const u64 t = (u64) (unsigned) mb * Y0;
    const u64 hm = (u64) (unsigned) (mb >> 32) * Y0 + (t >> 32);
    const i64 e0 = (i64) (0ull - ((hm << 32) | (t & 0xffffffffull)));
    const unsigned top = (unsigned) (hm >> 32);
    /* the seed is good enough when |e0| < 3 2^61 (relative error < 2^-21.4):
     * then Y1 <= 2^116 / mb with relative error < 2^-42.8, the first
     * remainder R lies in [0, 2^64), the correction leaves it in [0, 2 mb)
     * and one step finishes the exact quotient (a seed outside the bound
     * takes the hardware divide) */
    const bool seed_ok = (top == (1u << 20) - 1u ? e0 > 0 : (top == (1u << 20) && e0 <= 0))
                      && e0 < 3 * (1ll << 61) && e0 > -3 * (1ll << 61);
    const i64 d = ((i64) (int) (e0 >> 32) * (i64) Y0) >> 20; /* Y0 e0 2^-52 */
    const u64 Y1 = ((u64) Y0 << 32) + (u64) d;               /* ~2^116 / mb, from below */

    const u64 A_lo = ma << (52 + s);
    u64 Q = mulhi(ma << s, Y1);                              /* <= floor(A / mb), A = ma 2^(52+s) */
    u64 R = A_lo - Q * mb;
    const u64 dq = ((R >> 32) * (Y1 >> 32)) >> 52;
    Q += dq;
    R -= dq * mb;
    if (R >= mb) { Q += 1; R -= mb; }
    const bool exact = seed_ok;
    const u64 r2 = R << 1;
    Q += (r2 > mb || (r2 == mb && (Q & 1ull))) ? 1ull : 0ull;
    const u64 res = sign | (((u64) (unsigned) (e - 1) << 52) + Q);

    const bool b_normal = eb - 1u < 2046u;
    const bool a_zero = (ua << 1) == 0ull;
    ok = b_normal && (a_zero || (ea - 1u < 2046u && (unsigned) (e - 1) < 2046u && exact));
    return from_bits(a_zero ? sign : res);
}

/* RN(sqrt(x)) when `ok` comes back true. */
FXHD double sqrt_fast(double x, bool &ok)
{
    const u64 ux = bits(x);
    const unsigned ex = (unsigned) (ux >> 52);                /* sign bit included */
    const int odd = (ex & 1u) ? 0 : 1;                        /* unbiased exponent - 52 is odd */
    const u64 M = ((ux & FRAC) | HIDDEN) << odd;              /* [2^52, 2^54) */

    const float fm = from_fbits(((127u + (unsigned) odd) << 23) | (unsigned) ((ux >> 29) & 0x7fffffu));
    const unsigned Y0 = seed_fixed(rsqrt_seed(fm));
    const u64 Y0sq = (u64) Y0 * Y0;                           /* y0^2 2^64 */
    const i64 e0 = (i64) ((1ull << 62) - mulhi(M << 10, Y0sq));   /* (1 - M 2^-52 y0^2) 2^62 */
    const i64 d = ((i64) (int) (e0 >> 11) * (i64) Y0) >> 20;      /* Y0 e0 2^-31 */
    const u64 Y1 = ((u64) Y0 << 32) + (u64) d - 2ull;             /* ~2^64 / sqrt(M 2^-52), from below */

    const u64 X_lo = M << 52, X_hi = M >> 12;                 /* X = M 2^52 */
    u64 S = mulhi(M, Y1);
    const u64 R1 = X_lo - S * S;
    S += ((R1 >> 32) * (Y1 >> 32)) >> 53;
    i64 R = (i64) (X_lo - S * S);
    if (R < 0) { S -= 1; R += (i64) (2 * S + 1); }
    if (R > (i64) (2 * S)) { R -= (i64) (2 * S + 1); S += 1; }
    if (R > (i64) (2 * S)) { R -= (i64) (2 * S + 1); S += 1; }

    const u64 P_lo = S * S, P_hi = mulhi(S, S);
    const bool exact = (X_hi - P_hi - (X_lo < P_lo ? 1ull : 0ull)) == 0ull
                    && R >= 0 && (u64) R <= 2 * S;
    S += ((u64) R > S) ? 1ull : 0ull;
    const int t = ((int) ex - 1075 - odd) >> 1;               /* exponent left over, halved */
    const u64 res = ((u64) (unsigned) (t + 1048) << 52) + S;

    ok = ex - 1u < 2046u && exact;
    return from_bits(res);
}

/*
 * The limiter's sign test a * b <= 0 decided on the bits where that is exact
 * without the multiply: 1 (true), 0 (false), or -1 when it is not decided
 * here (a NaN or infinite operand, a subnormal one, or a product of normal
 * operands small enough to underflow to zero: the caller evaluates the FP64
 * expression).  A zero times a finite operand is a signed zero (true);
 * otherwise the product's sign is the XOR of the signs, and for
 * ea + eb >= 973 the product is at least 2^-1074 in magnitude.
 */
FXHD int product_nonpositive(u64 ua, u64 ub)
{
    const u64 aa = ua & ~SIGN, ab = ub & ~SIGN;
    const unsigned ea = (unsigned) (aa >> 52), eb = (unsigned) (ab >> 52);
    if (ea == 0x7ffu || eb == 0x7ffu) return -1;
    if (aa == 0ull || ab == 0ull) return 1;
    if (ea == 0u || eb == 0u || ea + eb < 973u) return -1;
    return (int) ((ua ^ ub) >> 63);
}

/* Ordered key of a non-NaN double's bits: monotone in the value, with +0
 * and -0 equal. */
FXHD i64 okey(u64 b) { return (i64) b >= 0 ? (i64) b : -(i64) (b & ~SIGN); }
FXHD bool nan_bits(u64 b) { return (b & ~SIGN) > 0x7ff0000000000000ull; }

#if defined(__CUDACC__)
/* Hardware operations for the cases the fast paths leave out; kept out of
 * line so that the fast path's call sites stay small. */
static __device__ __noinline__ double div_hw(double a, double b) { return a / b; }
static __device__ __noinline__ double sqrt_hw(double x) { return sqrt(x); }

/* The device forms, out of line: one copy per kernel instead of one per
 * call site.  The step kernel has ~40 divide / square-root sites; inlined,
 * their integer sequences overflow the instruction cache (measured on the
 * 2048^2 shear layer: 744 M cell-updates/s inlined, 819 M out of line). */
static __device__ __noinline__ double div_dev(double a, double b)
{
    bool ok;
    const double q = div_fast(a, b, ok);
    return ok ? q : div_hw(a, b);
}

/* 1 / x: the divide with a known numerator, which the compiler folds into
 * the integer sequence (the quotient step becomes a shift of Y1). */
static __device__ __noinline__ double rcp_dev(double x)
{
    bool ok;
    const double q = div_fast(1.0, x, ok);
    return ok ? q : div_hw(1.0, x);
}

static __device__ __noinline__ double sqrt_dev(double x)
{
    bool ok;
    const double r = sqrt_fast(x, ok);
    return ok ? r : sqrt_hw(x);
}
#endif

}  // namespace fx

/* a / b and sqrt(x) as the kernels use them: the integer forms on the
 * device for double (the non-template overloads), the operators for every
 * other type and on the host. */
template <class R>
FXHD R dv(R a, R b) { return a / b; }

template <class R>
FXHD R sq(R x) { return sqrt(x); }

/* 1 / x as the kernels evaluate it (the value of dv(1, x)). */
template <class R>
FXHD R rv(R x) { return R(1) / x; }

FXHD double rv(double x)
{
#if defined(__CUDA_ARCH__)
    return fx::rcp_dev(x);
#else
    return 1.0 / x;
#endif
}

FXHD double dv(double a, double b)
{
#if defined(__CUDA_ARCH__)
    return fx::div_dev(a, b);
#else
    return a / b;
#endif
}

FXHD double sq(double x)
{
#if defined(__CUDA_ARCH__)
    return fx::sqrt_dev(x);
#else
    return sqrt(x);
#endif
}

/* x + 0.0 and 0.0 - x as the kernels evaluate them (the reference's literal
 * "+ 0.0" terms, which only turn -0.0 into +0.0).  On the device, for
 * double, a compare and select on the bits: x + 0.0 is x except that -0.0
 * becomes +0.0, and 0.0 - x is -x except that both zeros give +0.0.  A NaN
 * stays a NaN (its payload bits are not canonicalised as an FP64 add would). */
template <class R>
FXHD R add_zero(R x) { return x + R(0); }

template <class R>
FXHD R zero_minus(R x) { return R(0) - x; }

FXHD double add_zero(double x)
{
#if defined(__CUDA_ARCH__)
    const fx::u64 u = fx::bits(x);
    return fx::from_bits(u == fx::SIGN ? 0ull : u);
#else
    return x + 0.0;
#endif
}

FXHD double zero_minus(double x)
{
#if defined(__CUDA_ARCH__)
    const fx::u64 u = fx::bits(x);
    return fx::from_bits((u << 1) == 0ull ? 0ull : (u ^ fx::SIGN));
#else
    return 0.0 - x;
#endif
}

/* x == 0.0 (either zero; false for NaN), on the bits for double on the device. */
template <class R>
FXHD bool eq_zero(R x) { return x == R(0); }

FXHD bool eq_zero(double x)
{
#if defined(__CUDA_ARCH__)
    return (fx::bits(x) << 1) == 0ull;
#else
    return x == 0.0;
#endif
}

/* Ordered comparisons as the kernels evaluate them: IEEE semantics (false
 * when either operand is NaN, +0 == -0), on the integer pipes for double on
 * the device. */
template <class R>
FXHD bool lt(R a, R b) { return a < b; }

template <class R>
FXHD bool le(R a, R b) { return a <= b; }

FXHD bool lt(double a, double b)
{
#if defined(__CUDA_ARCH__)
    const fx::u64 ua = fx::bits(a), ub = fx::bits(b);
    return !fx::nan_bits(ua) && !fx::nan_bits(ub) && fx::okey(ua) < fx::okey(ub);
#else
    return a < b;
#endif
}

FXHD bool le(double a, double b)
{
#if defined(__CUDA_ARCH__)
    const fx::u64 ua = fx::bits(a), ub = fx::bits(b);
    return !fx::nan_bits(ua) && !fx::nan_bits(ub) && fx::okey(ua) <= fx::okey(ub);
#else
    return a <= b;
#endif
}

}  // namespace hydro

#endif
