/*
 * pow_int.cuh -- FP64 pow(x, y) on the integer pipes, for x > 0.
 *
 * The two-rarefaction star-pressure guess takes three pow per face (and the
 * vacuum samplers and the 1D exact solver more); on GB300 the FMA-based
 * library pow is a long chain on the 2-lane FP64 pipe.  This form computes
 * 2^(y log2 x) in 128-bit fixed point with integer multiplies only:
 *
 *   log2 x = e + log2 m,  m in [1, 2), by two table reductions
 *     m * INV1[i] * INV2[j] = 1 + r,  |r| < 2^-14.9  (the products are exact),
 *     log2 m = LG1[i] + LG2[j] + log2(1 + r),
 *     log2(1 + r) = r/ln2 - r^2 h(r),  h = sum_k (-r)^(k-2) / (k ln2), k = 2..6
 *   (Tang's table-driven logarithm, ACM TOMS 16(4), 1990, with a second
 *   reduction step so that a short series suffices);
 *   P = y log2 x, exact product, truncated to 80 fraction bits;
 *   2^P = 2^n 2^(k1/128) 2^(k2/16384) 2^g,  g < 2^-14,
 *     2^g - 1 = u + u^2/2 + u^3/6 + u^4/24,  u = g ln2
 *   (Tang's table-driven exponential, ACM TOMS 15(2), 1989, two levels).
 * The tables (pow_tables.h, from gen_pow_tables.py) hold the reductions'
 * logarithms and powers of two to 100 / 127 fraction bits.
 *
 * Accuracy: log2 x is carried to ~2^-98 absolute and P to 2^-79, 2^P to
 * ~2^-77 relative before the final round-to-nearest-even, so for the
 * exponents of the solvers (|y| <= 8) the result is the correctly rounded
 * x^y.  Results within 2^-25 ulp of a rounding midpoint (exact midpoints,
 * which need x with few significant bits and an integer y, and a fraction
 * ~2^-23 of all others) are not decided and take the library pow, as do
 * every x <= 0, zero or subnormal y, |y| >= 512, infinity, NaN, overflow and
 * underflow.  glibc's pow, which the reference solver calls, is correctly
 * rounded in all but ~0.1% of cases (it differed by one ulp on 474 of
 * 600,000 solver-like operands), far closer than the hardware library's pow.
 */
#ifndef HYDRO_GPU_POW_INT_CUH
#define HYDRO_GPU_POW_INT_CUH

#include <math.h>
#ifdef __cplusplus
#include <cmath>
using std::pow;
#endif

#include "fp64_int.cuh"
#include "pow_tables.h"

namespace hydro {
namespace fx {

typedef unsigned __int128 u128;
typedef __int128 i128;

struct Q128 {
    u64 hi, lo;
};

static const unsigned h_pow_inv1[128] = HYDRO_POW_INV1;
static const Q128 h_pow_lg1[128] = HYDRO_POW_LG1;
static const unsigned h_pow_inv2[129] = HYDRO_POW_INV2;
static const Q128 h_pow_lg2[129] = HYDRO_POW_LG2;
static const Q128 h_pow_ex1[128] = HYDRO_POW_EX1;
static const Q128 h_pow_ex2[128] = HYDRO_POW_EX2;
#if defined(__CUDACC__)
static __device__ const unsigned d_pow_inv1[128] = HYDRO_POW_INV1;
static __device__ const Q128 d_pow_lg1[128] = HYDRO_POW_LG1;
static __device__ const unsigned d_pow_inv2[129] = HYDRO_POW_INV2;
static __device__ const Q128 d_pow_lg2[129] = HYDRO_POW_LG2;
static __device__ const Q128 d_pow_ex1[128] = HYDRO_POW_EX1;
static __device__ const Q128 d_pow_ex2[128] = HYDRO_POW_EX2;
#endif

#if defined(__CUDA_ARCH__)
#define HYDRO_POW_T(name) d_pow_##name
#else
#define HYDRO_POW_T(name) h_pow_##name
#endif

FXHD u128 q128(const Q128 &q) { return ((u128) q.hi << 64) | q.lo; }

/* a b / 2^127 for a, b < 2^127 (truncated; error below 3 units). */
FXHD u128 mul_q127(u128 a, u128 b)
{
    const u64 ah = (u64) (a >> 64), al = (u64) a, bh = (u64) (b >> 64), bl = (u64) b;
    return (((u128) ah * bh) << 1) + (((u128) ah * bl) >> 63) + (((u128) al * bh) >> 63);
}

/* c r / 2^77 with c in Q62 and r in Q77: the product in Q62. */
FXHD i64 mul_q62_q77(i64 c, i64 r) { return (i64) (((i128) c * r) >> 77); }

/* RN(x^y) when `ok` comes back true (see the header comment). */
FXHD double pow_fast(double x, double y, bool &ok)
{
    const u64 ux = bits(x), uy = bits(y);
    const unsigned ex = (unsigned) (ux >> 52);                 /* sign included: x > 0 normal <=> 1..2046 */
    const unsigned ey = (unsigned) (uy >> 52) & 0x7ffu;
    const bool y_neg = (uy >> 63) != 0;
    const u64 m = (ux & FRAC) | HIDDEN;
    const u64 my = (uy & FRAC) | HIDDEN;

    /* ---- log2 m = LG1[i] + LG2[j] + log2(1 + r), Q100 ---- */
    const int i = (int) ((m >> 45) & 127u);
    const u128 A = (u128) m * HYDRO_POW_T(inv1)[i];               /* m INV1, < 2^74 */
    const i128 a1 = (i128) A - ((i128) 1 << 73);                  /* r1 2^73 */
    int j = (int) ((a1 + ((i128) 1 << 58)) >> 59);                /* round(r1 2^14) */
    j = j < -64 ? -64 : (j > 64 ? 64 : j);
    const u128 B = A * HYDRO_POW_T(inv2)[j + 64];                 /* < 2^105 */
    const i128 R103 = (i128) B - ((i128) 1 << 103);               /* r 2^103 */

    const bool r_neg = R103 < 0;
    const u128 Ra = r_neg ? (u128) (-R103) : (u128) R103;
    const u64 Rl = (u64) Ra, Rh = (u64) (Ra >> 64);                /* Rh < 2^25 */
    const u64 Kh = HYDRO_POW_INVLN2_HI, Kl = HYDRO_POW_INVLN2_LO;  /* 2^127 / ln2 */
    const u128 lead_a = ((((u128) Rl * Kh) >> 64) + (u128) Rh * Kh + (((u128) Rh * Kl) >> 64)) >> 2;
    const i128 lead = r_neg ? -(i128) lead_a : (i128) lead_a;    /* r / ln2, Q100 */

    const i64 r77 = (i64) (R103 >> 26);                           /* |r| 2^77 < 2^62.2 */
    i64 h = (i64) HYDRO_POW_D5 - mul_q62_q77((i64) HYDRO_POW_D6, r77);
    h = (i64) HYDRO_POW_D4 - mul_q62_q77(h, r77);
    h = (i64) HYDRO_POW_D3 - mul_q62_q77(h, r77);
    h = (i64) HYDRO_POW_D2 - mul_q62_q77(h, r77);                 /* h(r), Q62 */
    const i64 rh = (i64) (((i128) h * r77) >> 62);                /* r h, Q77 */
    const i128 tail = ((i128) r77 * rh) >> 54;                    /* r^2 h, Q100 */

    const i128 ell = (i128) q128(HYDRO_POW_T(lg1)[i]) + (i128) q128(HYDRO_POW_T(lg2)[j + 64]) + lead - tail;
    const i128 F = ((i128) ((int) (ex & 0x7ffu) - 1023) << 100) + ell;   /* log2 x, Q100 */

    /* ---- P = y log2 x, Q80 ---- */
    const bool f_neg = F < 0;
    const u128 Fa = f_neg ? (u128) (-F) : (u128) F;               /* < 2^111 */
    const u128 T = (((u128) (u64) Fa * my) >> 64) + (u128) (u64) (Fa >> 64) * my;   /* |F| my / 2^64 */
    const int sh = 1031 - (int) ey;                               /* |P| 2^80 = T >> sh */
    const u128 Pa = (sh > 127) ? (u128) 0 : (T >> (sh < 0 ? 0 : sh));
    const bool in_range = Pa < ((u128) 1022 << 80);
    const i128 Pq = (f_neg != y_neg) ? -(i128) Pa : (i128) Pa;
    const int n = (int) (i64) (Pq >> 80);                          /* floor(P) */
    const u128 f = (u128) Pq & (((u128) 1 << 80) - 1);

    /* ---- 2^f = (1 + V)(1 + q), Q127 ---- */
    const int k1 = (int) (f >> 73), k2 = (int) (f >> 66) & 127;
    const u64 g78 = (u64) ((f & (((u128) 1 << 66) - 1)) >> 2);     /* g 2^78 */
    const u128 u = ((u128) g78 * HYDRO_POW_LN2_Q64) >> 15;         /* g ln2, Q127 */
    const u64 u78 = (u64) (u >> 49);
    const u128 u2 = ((u128) u78 * u78) >> 29;                      /* u^2, Q127 */
    const u64 u3 = (u64) (((u128) (u64) (u2 >> 49) * u78) >> 78);  /* u^3, Q78 */
    const u64 u4 = (u64) (((u128) u3 * u78) >> 78);                /* u^4, Q78 */
    const u64 t34 = (u64) (((u128) u3 * HYDRO_POW_INV6_Q64) >> 64) + (u64) (((u128) u4 * HYDRO_POW_INV24_Q64) >> 64);
    const u128 q = u + (u2 >> 1) + ((u128) t34 << 49);              /* 2^g - 1 */
    const u128 a = q128(HYDRO_POW_T(ex1)[k1]), b = q128(HYDRO_POW_T(ex2)[k2]);
    const u128 V = a + b + mul_q127(a, b);
    u128 W = V + q + mul_q127(V, q);                               /* 2^f - 1 */
    if (W >> 127) W = ((u128) 1 << 127) - 1;

    /* ---- round to 53 bits and pack ---- */
    u64 mant = (u64) (W >> 75);
    const u128 rem = W & (((u128) 1 << 75) - 1), half = (u128) 1 << 74;
    mant += (rem > half) ? 1ull : 0ull;
    /* within the error bound (2^-25 ulp) of a midpoint the rounding is not
     * decided: exact midpoints (x with few significant bits, integer y) land
     * here; they take the library pow */
    const u128 dist = (rem > half) ? rem - half : half - rem;
    const bool decided = dist > ((u128) 1 << 51);
    const int E = n + 1023;
    ok = (ex - 1u < 2046u) && (ey - 1u < 2046u) && sh >= 0 && in_range && decided
      && (unsigned) (E - 1) < 2046u;
    return from_bits(((u64) (unsigned) (E - 1) << 52) + HIDDEN + mant);
}

#if defined(__CUDACC__)
static __device__ __noinline__ double pow_hw(double x, double y) { return pow(x, y); }

/* The device pow, out of line (one copy per kernel instead of one per call
 * site), like the divide and square root of fp64_int.cuh. */
static __device__ __noinline__ double pow_dev(double x, double y)
{
    bool ok;
    const double r = pow_fast(x, y, ok);
    return ok ? r : pow_hw(x, y);
}
#endif

}  // namespace fx

/* pow as the kernels use it: the integer form on the device for double
 * (the non-template overload), the hardware exp2/log2 form (__powf) on the
 * device for float -- the FP32 state form, whose other divides and square
 * roots are approximate too --, the library pow on the host. */
template <class R>
FXHD R pw(R x, R y) { return pow(x, y); }

#if defined(__CUDA_ARCH__)
FXHD float pw(float x, float y) { return __powf(x, y); }
#endif

FXHD double pw(double x, double y)
{
#if defined(__CUDA_ARCH__)
    return fx::pow_dev(x, y);
#else
    return pow(x, y);
#endif
}

}  // namespace hydro

#endif
