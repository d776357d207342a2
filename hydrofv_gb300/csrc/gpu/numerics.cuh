/*
 * numerics.cuh -- pointwise finite-volume numerics shared by every kernel.
 *
 * Device (and host-callable) restatements of hydroFV's pointwise routines.
 * Each expression keeps the reference's operand order and grouping so that
 * the FP64 kernels, compiled with --fmad=false, perform the same IEEE-754
 * operation sequence as the reference CPU code:
 *
 *   sound speed           src/utils.c:23-26
 *   slope limiters        src/slope_limiter.c:49-91
 *   star-pressure guess   src/riemann_solver.c:154-224
 *   vacuum sampling       src/riemann_solver.c:230-733
 *   HLLC 2D / 1D          src/riemann_solver_hllc.c:30-40, :42-200, :202-376
 *   exact solver 1D       src/riemann_solver_exact.c:332-1080
 *   Hancock predictor     src/integrator_muscl_hancock.c:682-755 (x),
 *                         :967-1041 (y), :185-246 (1D)
 *   U -> W conversion     src/system.c:735-802
 *
 * Constants the reference recomputes inline on every call (gamma+1,
 * (gamma-1)/(gamma+1), 0.5+0.5/gamma, ...) are computed once on the host with
 * the identical expression and passed in `GasConst`; the result is the same
 * double, so this changes nothing but the instruction count.
 */
#ifndef HYDRO_GPU_NUMERICS_CUH
#define HYDRO_GPU_NUMERICS_CUH

#include <math.h>
#include <string.h>

#include "fp64_int.cuh"
#include "pow_int.cuh"
#ifdef __cplusplus
#include <cmath>
#include <type_traits>
using std::fabs;
using std::fmin;
using std::pow;
using std::sqrt;
#endif

#ifdef __CUDACC__
#define HD __host__ __device__ __forceinline__
#else
#define HD static inline
#endif

namespace hydro {

enum : int {
    LIM_MINMOD = 1,
    LIM_VAN_LEER = 2,
    LIM_MC = 3,
};

enum : int {
    BC_NONE = 1,
    BC_REFLECTIVE = 2,
    BC_TRANSMISSIVE = 3,
    BC_PERIODIC = 4,
    BC_CUSTOM = 5,      /* host callback: ghost W is written by the host, read as stored */
};

/* Device error codes (mapped to ErrorStatus on the host). */
enum : int {
    DEV_OK = 0,
    DEV_ERR_HLLC_WAVE_SPEED = 1,   /* src/riemann_solver_hllc.c:372-375 */
    DEV_ERR_DT_ZERO = 2,           /* src/integrator_muscl_hancock.c:545-549 */
    DEV_ERR_EXACT_BRACKET = 3,     /* src/riemann_solver_exact.c:702-707 */
    DEV_ERR_EXACT_BISECTION = 4,   /* src/riemann_solver_exact.c:745-754 */
    DEV_ERR_SPIN_LIMIT = 5,        /* a bounded device-side wait gave up */
};

template <class R>
struct GasConst {
    R gamma;
    R gm1;          /* gamma - 1.0 */
    R gp1;          /* gamma + 1.0 */
    R half_gm1;     /* 0.5 * (gamma - 1.0) */
    R half_gm1_g;   /* (0.5 * (gamma - 1.0)) / gamma */
    R g_half_gm1;   /* gamma / (0.5 * (gamma - 1.0)) */
    R q_coef;       /* 0.5 + 0.5 / gamma */
    R gm1_gp1;      /* (gamma - 1.0) / (gamma + 1.0) */
    R two_gp1;      /* 2.0 / (gamma + 1.0) */
    R two_gm1;      /* 2.0 / (gamma - 1.0) */
    R g_gm1;        /* gamma / (gamma - 1.0) */
    R gm1_2g;       /* (gamma - 1.0) / (2.0 * gamma) */
    R gp1_2g;       /* (gamma + 1.0) / (2.0 * gamma) */
    R neg_gp1_2g;   /* -0.5 * (gamma + 1.0) / gamma */
    R inv_g;        /* 1.0 / gamma */
    R inv_gm1;      /* 1.0 / (gamma - 1.0) (the adjoint's reverse code) */
    R tol;          /* integrator tolerance (guess_p floor, exact solver) */
};

/* Build the constants with the reference's own expressions. */
template <class R>
HD GasConst<R> make_gas_const(double gamma, double tol)
{
    GasConst<R> c;
    c.gamma = (R) gamma;
    c.gm1 = (R) (gamma - 1.0);
    c.gp1 = (R) (gamma + 1.0);
    c.half_gm1 = (R) (0.5 * (gamma - 1.0));
    c.half_gm1_g = (R) ((0.5 * (gamma - 1.0)) / gamma);
    c.g_half_gm1 = (R) (gamma / (0.5 * (gamma - 1.0)));
    c.q_coef = (R) (0.5 + 0.5 / gamma);
    c.gm1_gp1 = (R) ((gamma - 1.0) / (gamma + 1.0));
    c.two_gp1 = (R) (2.0 / (gamma + 1.0));
    c.two_gm1 = (R) (2.0 / (gamma - 1.0));
    c.g_gm1 = (R) (gamma / (gamma - 1.0));
    c.gm1_2g = (R) ((gamma - 1.0) / (2.0 * gamma));
    c.gp1_2g = (R) ((gamma + 1.0) / (2.0 * gamma));
    c.neg_gp1_2g = (R) (-0.5 * (gamma + 1.0) / gamma);
    c.inv_g = (R) (1.0 / gamma);
    c.inv_gm1 = (R) (1.0 / (gamma - 1.0));
    c.tol = (R) tol;
    return c;
}

/* ------------------------------------------------------------------ basics */

template <class R>
HD R sound_speed(const GasConst<R> &c, R rho, R p)
{
    return sq(dv(c.gamma * p, rho));
}

/*
 * On the device, for double, the sign test and the minima are decided on the
 * bits (fx::product_nonpositive; the minimum of two positive doubles is the
 * minimum of their bit patterns), leaving the FP64 pipe a + b and the two
 * scalings.  The results are those of the expressions below bit for bit;
 * operands the bit test does not decide take the expressions themselves.
 */
template <int LIM, class R>
HD R limit_slope(R a, R b)
{
#if defined(__CUDA_ARCH__)
    if constexpr (std::is_same<R, double>::value) {
        const fx::u64 ua = fx::bits(a), ub = fx::bits(b);
        const int t = fx::product_nonpositive(ua, ub);
        if (t > 0) return R(0);
        if (t == 0) {
            const fx::u64 aa = ua & ~fx::SIGN, ab = ub & ~fx::SIGN;
            if (LIM == LIM_MINMOD) return (aa < ab) ? a : b;
            if (LIM == LIM_VAN_LEER) return dv(R(2) * a * b, a + b + R(1e-10));
            const double two_m = 2.0 * fx::from_bits(aa < ab ? aa : ab);     /* 2 fmin(|a|, |b|) */
            const double avg = ((ua >> 63) ? -0.5 : 0.5) * (a + b);           /* > 0 */
            const fx::u64 ua2 = fx::bits(avg), ut = fx::bits(two_m);
            return fx::from_bits((ua2 < ut ? ua2 : ut) | (ua & fx::SIGN));  /* +-fmin(avg, two_m) */
        }
    }
#endif
    if (a * b <= R(0)) return R(0);
    if (LIM == LIM_MINMOD) return (fabs(a) < fabs(b)) ? a : b;
    if (LIM == LIM_VAN_LEER) return dv(R(2) * a * b, a + b + R(1e-10));
    if (a > R(0)) return fmin(R(0.5) * (a + b), R(2) * fmin(fabs(a), fabs(b)));
    return -fmin(R(-0.5) * (a + b), R(2) * fmin(fabs(a), fabs(b)));
}

/* Runtime-dispatched limiter (1D paths and host exports). */
template <class R>
HD R limit_slope_rt(int lim, R a, R b)
{
    switch (lim) {
    case LIM_MINMOD: return limit_slope<LIM_MINMOD>(a, b);
    case LIM_VAN_LEER: return limit_slope<LIM_VAN_LEER>(a, b);
    default: return limit_slope<LIM_MC>(a, b);
    }
}

/*
 * p_max / p_min <= 2, decided without the divide where that is exact.  For
 * p_min > 0 (normal or subnormal) the rounded quotient is <= 2 exactly when
 * p_max <= 2 p_min: if p_max > 2 p_min, the next representable p_max above
 * 2 p_min puts the exact quotient more than half an ulp of 2 above 2, so it
 * cannot round down to 2; otherwise the quotient is <= 2 and rounding is
 * monotone.  (2 p_min overflowing is consistent too: both tests are true.)
 * Zero, negative and NaN pressures take the reference's divide.
 */
template <class R>
HD bool ratio_at_most_two(R p_max, R p_min)
{
    if (lt(R(0), p_min)) return le(p_max, R(2) * p_min);
    return p_max / p_min <= R(2);
}

/*
 * RN(x / y) < tol for x >= 0 and y > 0 (the exact solver's convergence test),
 * decided without the divide where a margin allows.  With T = RN(RN(tol y) c):
 *   c = 1 - 2^-50:  x < T implies x / y < tol (1 - 2^-51), so RN(x / y) is at
 *                   least one ulp below tol: true;
 *   c = 1 + 2^-50:  x > T implies x / y > tol (1 + 2^-51), so RN(x / y) >= tol:
 *                   false
 * (each rounding is within a factor 1 +- 2^-53, and one ulp of tol is at most
 * tol 2^-52).  The bounds need tol y to be a normal double: otherwise, and
 * between the two margins, `decided` comes back false and the caller divides.
 */
FXHD bool ratio_below_fast(double x, double y, double tol, bool &decided)
{
    const double ty = tol * y;
    decided = false;
    if (!(ty > 1e-290 && ty < 1e290 && x <= 1e300)) return false;
    if (x < ty * (1.0 - 0x1p-50)) { decided = true; return true; }
    if (x > ty * (1.0 + 0x1p-50)) { decided = true; return false; }
    return false;
}

template <class R>
HD bool ratio_below(R x, R y, R tol) { return dv(x, y) < tol; }

HD bool ratio_below(double x, double y, double tol)
{
#if defined(__CUDA_ARCH__)
    bool decided;
    const bool r = ratio_below_fast(x, y, tol, decided);
    if (decided) return r;
#endif
    return dv(x, y) < tol;
}

/*
 * RN(x / y) <= z for x > 0 and y > 0 normal (the vacuum-generation test of
 * the HLLC and exact solvers: x = 2 (a_L + a_R), y = gamma + 1, z = u_R - u_L),
 * decided from the exponents alone where they leave no doubt, with integer
 * operations only (the FP64 step kernels are bound by their FP64 pipe).  With
 * d = e_x - e_y (unbiased exponents), x / y lies in (2^(d-1), 2^(d+1)), so
 * RN(x / y) lies in [2^(d-1), 2^(d+1)]; z lies in [2^e_z, 2^(e_z+1)).  So:
 *   z < 0 (nonzero):   false (the quotient is positive);
 *   e_z >= d + 1:      RN(x / y) <= 2^(d+1) <= z: true;
 *   e_z <= d - 2:      z < 2^(d-1) <= RN(x / y): false.
 * Zero, subnormal, infinite and NaN operands and e_z in {d - 1, d} are not
 * decided (`decided` false): the caller divides.
 */
FXHD bool quot_le_fast(double x, double y, double z, bool &decided)
{
    const fx::u64 bx = fx::bits(x), by = fx::bits(y), bz = fx::bits(z);
    const int ex = (int) (bx >> 52), ey = (int) (by >> 52);           /* sign bit included */
    const int ez = (int) ((bz >> 52) & 0x7ffu);
    decided = false;
    if ((unsigned) (ex - 1) >= 2046u || (unsigned) (ey - 1) >= 2046u) return false;
    if (bz >> 63) {
        if ((bz << 1) != 0ull && ez != 0x7ff) decided = true;          /* finite z < 0 */
        return false;
    }
    if ((unsigned) (ez - 1) >= 2046u) return false;
    const int d = ex - ey;
    if (ez - 1023 >= d + 1) { decided = true; return true; }
    if (ez - 1023 <= d - 2) { decided = true; return false; }
    return false;
}

template <class R>
HD bool quot_le(R x, R y, R z) { return le(dv(x, y), z); }

HD bool quot_le(double x, double y, double z)
{
#if defined(__CUDA_ARCH__)
    bool decided;
    const bool r = quot_le_fast(x, y, z, decided);
    if (decided) return r;
#endif
    return le(dv(x, y), z);
}

/* Star-pressure guess (PVRS / two-rarefaction / two-shock). */
template <class R>
HD R guess_p(const GasConst<R> &c, R rho_L, R u_L, R p_L, R a_L,
             R rho_R, R u_R, R p_R, R a_R)
{
    const R p_min = (p_L > p_R) ? p_R : p_L;
    const R p_max = (p_L > p_R) ? p_L : p_R;
    const R ppv = R(0.5) * (p_L + p_R) - R(0.125) * (u_R - u_L) * (rho_L + rho_R) * (a_L + a_R);
    R pg;
    if (ratio_at_most_two(p_max, p_min) && (p_min <= ppv && ppv <= p_max)) {
        pg = ppv;
    } else if (ppv < p_min) {
        pg = dv(a_L + a_R - c.half_gm1 * (u_R - u_L),
                dv(a_L, pw(p_L, c.half_gm1_g)) + dv(a_R, pw(p_R, c.half_gm1_g)));
        pg = pw(pg, c.g_half_gm1);
    } else {
        const R gL = sq(dv(dv(R(2), c.gp1 * rho_L), ppv + p_L * c.gm1_gp1));
        const R gR = sq(dv(dv(R(2), c.gp1 * rho_R), ppv + p_R * c.gm1_gp1));
        pg = dv(gL * p_L + gR * p_R - (u_R - u_L), gL + gR);
    }
    if (pg < c.tol) pg = c.tol;
    return pg;
}

/* ---------------------------------------------------------------- vacuum */

template <class R>
HD void sample_right_vacuum(const GasConst<R> &c, R rho, R u, R v, R p, R a, R S, R o[4])
{
    if (S <= (u - a)) { o[0] = rho; o[1] = u; o[2] = v; o[3] = p; return; }
    const R front = u + dv(R(2) * a, c.gm1);
    if (S < front) {
        R tmp = c.two_gp1 + dv((u - S) * c.gm1, c.gp1 * a);
        tmp = pw(tmp, c.two_gm1);
        o[0] = rho * tmp;
        o[1] = dv((a + c.half_gm1 * u + S) * R(2), c.gp1);
        o[2] = v;
        o[3] = p * pw(tmp, c.gamma);
    } else {
        o[0] = R(0); o[1] = R(0); o[2] = R(0); o[3] = R(0);
    }
}

template <class R>
HD void sample_left_vacuum(const GasConst<R> &c, R rho, R u, R v, R p, R a, R S, R o[4])
{
    if (S >= (u + a)) { o[0] = rho; o[1] = u; o[2] = v; o[3] = p; return; }
    const R front = u - dv(R(2) * a, c.gm1);
    if (S > front) {
        R tmp = c.two_gp1 - dv((u - S) * c.gm1, c.gp1 * a);
        tmp = pw(tmp, c.two_gm1);
        o[0] = rho * tmp;
        o[1] = dv((-a + c.half_gm1 * u + S) * R(2), c.gp1);
        o[2] = v;
        o[3] = p * pw(tmp, c.gamma);
    } else {
        o[0] = R(0); o[1] = R(0); o[2] = R(0); o[3] = R(0);
    }
}

/* The reference routes rho_L <= 0 to the "right vacuum" sampler fed with the
 * left state, and uses 2a/(gamma-1) (no velocity term) as the
 * vacuum-generation front speeds; both are kept as written. */
template <class R>
HD void solve_vacuum(const GasConst<R> &c,
                     R rho_L, R u_L, R v_L, R p_L, R a_L,
                     R rho_R, R u_R, R v_R, R p_R, R a_R, R S, R o[4])
{
    if (rho_L <= R(0) && rho_R <= R(0)) { o[0] = o[1] = o[2] = o[3] = R(0); return; }
    if (rho_L <= R(0)) { sample_right_vacuum(c, rho_L, u_L, v_L, p_L, a_L, S, o); return; }
    if (rho_R <= R(0)) { sample_left_vacuum(c, rho_R, u_R, v_R, p_R, a_R, S, o); return; }
    const R SL = dv(R(2) * a_L, c.gm1);
    const R SR = dv(R(2) * a_R, c.gm1);
    if (S <= SL) { sample_right_vacuum(c, rho_L, u_L, v_L, p_L, a_L, S, o); return; }
    if (SR <= S) { sample_left_vacuum(c, rho_R, u_R, v_R, p_R, a_R, S, o); return; }
    o[0] = o[1] = o[2] = o[3] = R(0);
}

/* ------------------------------------------------------------------ HLLC */

template <class R>
HD R hllc_q(const GasConst<R> &c, R p_X, R p_star)
{
    if (le(p_star, p_X)) return R(1);
    return sq(R(1) + c.q_coef * (dv(p_star, p_X) - R(1)));
}

/*
 * HLLC flux, 2D form, in three phases so a caller can batch faces by regime:
 *
 *   hllc_classify   sound speeds, the vacuum / vacuum-generation test and the
 *                   star-pressure guess regime (PVRS, two-rarefaction or
 *                   two-shock), src/riemann_solver_hllc.c:218-287 and
 *                   src/riemann_solver.c:154-183;
 *   guess_p_trrs /
 *   guess_p_tsrs    the two expensive guesses (src/riemann_solver.c:184-215);
 *   hllc_finish     the guess floor, wave speeds, S*, and the flux of the
 *                   region that contains x/t = 0 (src/riemann_solver_hllc.c:289-375).
 *
 * The region flux is written once for the selected side K (L for 0 <= S_L
 * and the left star region, R otherwise): the supersonic fluxes
 * rho*u*u + p, rho*u*v, u*(E + p) are the same operations as the star
 * branch's F_K terms, so only the star correction is conditional.
 * hllc_flux_2d chains the phases and is operation-for-operation the
 * reference's solve_flux_hllc_2d.
 */
enum : int {
    PREG_VACUUM = 0,
    PREG_PVRS = 1,
    PREG_TRRS = 2,
    PREG_TSRS = 3,
};

template <class R>
HD int hllc_classify(const GasConst<R> &c, R rho_L, R u_L, R p_L, R rho_R, R u_R, R p_R,
                     R &a_L, R &a_R, R &ppv)
{
    a_L = lt(R(0), rho_L) ? sound_speed(c, rho_L, p_L) : R(0);
    a_R = lt(R(0), rho_R) ? sound_speed(c, rho_R, p_R) : R(0);
    ppv = R(0);
    if (le(rho_L, R(0)) || le(rho_R, R(0)) || quot_le((a_L + a_R) * R(2), c.gp1, u_R - u_L))
        return PREG_VACUUM;
    const bool l_above = lt(p_R, p_L);
    const R p_min = l_above ? p_R : p_L;
    const R p_max = l_above ? p_L : p_R;
    ppv = R(0.5) * (p_L + p_R) - R(0.125) * (u_R - u_L) * (rho_L + rho_R) * (a_L + a_R);
    if (ratio_at_most_two(p_max, p_min) && (le(p_min, ppv) && le(ppv, p_max))) return PREG_PVRS;
    if (lt(ppv, p_min)) return PREG_TRRS;
    return PREG_TSRS;
}

/* The *_z / *_g forms also hand back the guesses' intermediate factors
 * (p^((g-1)/2g) of each side for the two-rarefaction guess, g_K of each
 * side for the two-shock guess), which the adjoint's tape keeps; they
 * evaluate the same expressions as the plain forms below. */
template <class R>
HD R guess_p_trrs_z(const GasConst<R> &c, R u_L, R p_L, R a_L, R u_R, R p_R, R a_R, R &zL, R &zR)
{
    zL = pw(p_L, c.half_gm1_g);
    zR = pw(p_R, c.half_gm1_g);
    const R pg = dv(a_L + a_R - c.half_gm1 * (u_R - u_L), dv(a_L, zL) + dv(a_R, zR));
    return pw(pg, c.g_half_gm1);
}

template <class R>
HD R guess_p_trrs(const GasConst<R> &c, R u_L, R p_L, R a_L, R u_R, R p_R, R a_R)
{
    const R pg = dv(a_L + a_R - c.half_gm1 * (u_R - u_L),
                    dv(a_L, pw(p_L, c.half_gm1_g)) + dv(a_R, pw(p_R, c.half_gm1_g)));
    return pw(pg, c.g_half_gm1);
}

template <class R>
HD R guess_p_tsrs_g(const GasConst<R> &c, R rho_L, R u_L, R p_L, R rho_R, R u_R, R p_R, R ppv, R &gL, R &gR)
{
    gL = sq(dv(dv(R(2), c.gp1 * rho_L), ppv + p_L * c.gm1_gp1));
    gR = sq(dv(dv(R(2), c.gp1 * rho_R), ppv + p_R * c.gm1_gp1));
    return dv(gL * p_L + gR * p_R - (u_R - u_L), gL + gR);
}

template <class R>
HD R guess_p_tsrs(const GasConst<R> &c, R rho_L, R u_L, R p_L, R rho_R, R u_R, R p_R, R ppv)
{
    const R gL = sq(dv(dv(R(2), c.gp1 * rho_L), ppv + p_L * c.gm1_gp1));
    const R gR = sq(dv(dv(R(2), c.gp1 * rho_R), ppv + p_R * c.gm1_gp1));
    return dv(gL * p_L + gR * p_R - (u_R - u_L), gL + gR);
}

/* Flux of the vacuum / vacuum-generation case (src/riemann_solver_hllc.c:249-287). */
template <class R>
HD void hllc_vacuum_flux(const GasConst<R> &c, R rho_L, R u_L, R v_L, R p_L, R a_L,
                         R rho_R, R u_R, R v_R, R p_R, R a_R, R F[4])
{
    R s[4];
    solve_vacuum(c, rho_L, u_L, v_L, p_L, a_L, rho_R, u_R, v_R, p_R, a_R, R(0), s);
    const R E = s[0] * (R(0.5) * (s[1] * s[1] + s[2] * s[2]) + dv(s[3], s[0] * c.gm1));
    F[0] = s[0] * s[1];
    F[1] = s[0] * s[1] * s[1] + s[3];
    F[2] = s[0] * s[1] * s[2];
    F[3] = s[1] * (E + s[3]);
}

/* From the (unfloored) star-pressure guess to the flux.  Returns DEV_OK or
 * DEV_ERR_HLLC_WAVE_SPEED.  wave (may be null) receives q_L, q_R and S*, the
 * intermediates the adjoint's tape keeps. */
template <class R>
HD int hllc_finish(const GasConst<R> &c, R rho_L, R u_L, R v_L, R p_L, R a_L,
                   R rho_R, R u_R, R v_R, R p_R, R a_R, R pg, R F[4], R *wave = nullptr)
{
    const R ps = lt(pg, c.tol) ? c.tol : pg;
    const R q_L = hllc_q(c, p_L, ps);
    const R q_R = hllc_q(c, p_R, ps);
    const R S_L = u_L - a_L * q_L;
    const R S_R = u_R + a_R * q_R;
    const R S_s = dv(p_R - p_L + rho_L * u_L * (S_L - u_L) - rho_R * u_R * (S_R - u_R),
                     rho_L * (S_L - u_L) - rho_R * (S_R - u_R));
    if (wave) { wave[0] = q_L; wave[1] = q_R; wave[2] = S_s; }
    int region;
    if (le(R(0), S_L)) region = 0;
    else if (le(S_L, R(0)) && le(R(0), S_s)) region = 1;
    else if (le(S_s, R(0)) && le(R(0), S_R)) region = 2;
    else if (le(S_R, R(0))) region = 3;
    else return DEV_ERR_HLLC_WAVE_SPEED;
    const bool left = region <= 1;
    const R rho = left ? rho_L : rho_R;
    const R u = left ? u_L : u_R;
    const R v = left ? v_L : v_R;
    const R p = left ? p_L : p_R;
    const R E = rho * (R(0.5) * (u * u + v * v) + dv(p, rho * c.gm1));
    const R fm = rho * u;
    F[0] = fm;
    F[1] = fm * u + p;
    F[2] = fm * v;
    F[3] = u * (E + p);
    if (region == 1 || region == 2) {
        const R S = left ? S_L : S_R;
        const R rs = dv(rho * (S - u), S - S_s);
        const R es = rs * (dv(E, rho) + (S_s - u) * (S_s + dv(p, rho * (S - u))));
        F[0] = fm + S * (rs - rho);
        F[1] = F[1] + S * (rs * S_s - rho * u);
        F[2] = F[2] + S * (rs * v - rho * v);
        F[3] = F[3] + S * (es - E);
    }
    return DEV_OK;
}

/*
 * HLLC flux, 2D form.  (u = normal velocity, v = tangential.)  F receives
 * (mass, normal momentum, tangential momentum, energy).  Returns DEV_OK or
 * DEV_ERR_HLLC_WAVE_SPEED (no branch matched, i.e. a NaN wave speed).
 */
template <class R>
HD int hllc_flux_2d(const GasConst<R> &c, R rho_L, R u_L, R v_L, R p_L,
                    R rho_R, R u_R, R v_R, R p_R, R F[4])
{
    R a_L, a_R, ppv;
    const int reg = hllc_classify(c, rho_L, u_L, p_L, rho_R, u_R, p_R, a_L, a_R, ppv);
    if (reg == PREG_VACUUM) {
        hllc_vacuum_flux(c, rho_L, u_L, v_L, p_L, a_L, rho_R, u_R, v_R, p_R, a_R, F);
        return DEV_OK;
    }
    R pg = ppv;
    if (reg == PREG_TRRS) pg = guess_p_trrs(c, u_L, p_L, a_L, u_R, p_R, a_R);
    else if (reg == PREG_TSRS) pg = guess_p_tsrs(c, rho_L, u_L, p_L, rho_R, u_R, p_R, ppv);
    return hllc_finish(c, rho_L, u_L, v_L, p_L, a_L, rho_R, u_R, v_R, p_R, a_R, pg, F);
}

/* HLLC flux, 1D form (energy density groups 0.5*u*u as (0.5*u)*u). */
template <class R>
HD int hllc_flux_1d(const GasConst<R> &c, R rho_L, R u_L, R p_L, R rho_R, R u_R, R p_R, R F[3])
{
    const R a_L = (rho_L > R(0)) ? sound_speed(c, rho_L, p_L) : R(0);
    const R a_R = (rho_R > R(0)) ? sound_speed(c, rho_R, p_R) : R(0);
    if (rho_L <= R(0) || rho_R <= R(0) || quot_le((a_L + a_R) * R(2), c.gp1, u_R - u_L)) {
        R s[4];
        solve_vacuum(c, rho_L, u_L, R(0), p_L, a_L, rho_R, u_R, R(0), p_R, a_R, R(0), s);
        const R E = s[0] * (R(0.5) * s[1] * s[1] + dv(s[3], s[0] * c.gm1));
        F[0] = s[0] * s[1];
        F[1] = s[0] * s[1] * s[1] + s[3];
        F[2] = s[1] * (E + s[3]);
        return DEV_OK;
    }
    const R ps = guess_p(c, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R);
    const R S_L = u_L - a_L * hllc_q(c, p_L, ps);
    const R S_R = u_R + a_R * hllc_q(c, p_R, ps);
    const R S_s = dv(p_R - p_L + rho_L * u_L * (S_L - u_L) - rho_R * u_R * (S_R - u_R),
                     rho_L * (S_L - u_L) - rho_R * (S_R - u_R));
    if (R(0) <= S_L) {
        const R E = rho_L * (R(0.5) * u_L * u_L + dv(p_L, rho_L * c.gm1));
        F[0] = rho_L * u_L;
        F[1] = rho_L * u_L * u_L + p_L;
        F[2] = u_L * (E + p_L);
        return DEV_OK;
    }
    if (S_L <= R(0) && R(0) <= S_s) {
        const R E = rho_L * (R(0.5) * u_L * u_L + dv(p_L, rho_L * c.gm1));
        const R fm = rho_L * u_L;
        const R rs = dv(rho_L * (S_L - u_L), S_L - S_s);
        const R es = rs * (dv(E, rho_L) + (S_s - u_L) * (S_s + dv(p_L, rho_L * (S_L - u_L))));
        F[0] = fm + S_L * (rs - rho_L);
        F[1] = (fm * u_L + p_L) + S_L * (rs * S_s - rho_L * u_L);
        F[2] = u_L * (E + p_L) + S_L * (es - E);
        return DEV_OK;
    }
    if (S_s <= R(0) && R(0) <= S_R) {
        const R E = rho_R * (R(0.5) * u_R * u_R + dv(p_R, rho_R * c.gm1));
        const R fm = rho_R * u_R;
        const R rs = dv(rho_R * (S_R - u_R), S_R - S_s);
        const R es = rs * (dv(E, rho_R) + (S_s - u_R) * (S_s + dv(p_R, rho_R * (S_R - u_R))));
        F[0] = fm + S_R * (rs - rho_R);
        F[1] = (fm * u_R + p_R) + S_R * (rs * S_s - rho_R * u_R);
        F[2] = u_R * (E + p_R) + S_R * (es - E);
        return DEV_OK;
    }
    if (S_R <= R(0)) {
        const R E = rho_R * (R(0.5) * u_R * u_R + dv(p_R, rho_R * c.gm1));
        F[0] = rho_R * u_R;
        F[1] = rho_R * u_R * u_R + p_R;
        F[2] = u_R * (E + p_R);
        return DEV_OK;
    }
    return DEV_ERR_HLLC_WAVE_SPEED;
}

/* ---------------------------------------------------------- exact solver */

template <class R>
HD R exact_fK(const GasConst<R> &c, R rho, R p, R a, R ps)
{
    if (ps > p) {
        const R A = dv(R(2), c.gp1 * rho);
        const R B = p * c.gm1_gp1;
        return (ps - p) * sq(dv(A, ps + B));
    }
    return dv(R(2) * a * (pw(dv(ps, p), c.gm1_2g) - R(1)), c.gm1);
}

/* Derivative; the shock branch's (B - p*) follows the reference
 * (src/riemann_solver_exact.c:550-556). */
template <class R>
HD R exact_dfK(const GasConst<R> &c, R rho, R p, R a, R ps)
{
    if (ps > p) {
        const R A = dv(R(2), c.gp1 * rho);
        const R B = p * c.gm1_gp1;
        return (R(1) - dv(R(0.5) * (ps - p), B - ps)) * sq(dv(A, B + ps));
    }
    return dv(pw(dv(ps, p), c.neg_gp1_2g), p * a);
}

template <class R>
HD R exact_f(const GasConst<R> &c, R rho_L, R u_L, R p_L, R a_L, R rho_R, R u_R, R p_R, R a_R, R ps)
{
    return exact_fK(c, rho_L, p_L, a_L, ps) + exact_fK(c, rho_R, p_R, a_R, ps) + (u_R - u_L);
}

/* Bisection iterations at which the reference warns when Settings.verbose
 * > 0 ("Bisection method did not converge after %d iterations", every 500
 * iterations, src/riemann_solver_exact.c:736-744): marks[k] counts the
 * solves that passed 500 (k + 1) iterations.  The caller prints the
 * warnings; a null pointer counts nothing. */
constexpr int kBisectionMarks = 10;

HD void note_bisection_mark(unsigned int *marks, int count)
{
    if (marks == nullptr || count % 500 != 0) return;
#if defined(__CUDA_ARCH__)
    atomicAdd(&marks[count / 500 - 1], 1u);
#else
    marks[count / 500 - 1] += 1u;
#endif
}

/* Newton-Raphson (<= 100 iterations) with a bracketed bisection fallback
 * (<= 5000 iterations): every loop is bounded. */
template <class R>
HD int exact_p_star(const GasConst<R> &c, R rho_L, R u_L, R p_L, R a_L,
                    R rho_R, R u_R, R p_R, R a_R, R *out, unsigned int *marks = nullptr)
{
    const R pg = guess_p(c, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R);
    bool bracket = false;
    R p_hi = pg;
    R f_hi = exact_f(c, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, p_hi);
    R p_lo = R(0), f_lo = R(0);
    R p0 = pg;
    for (int it = 0; it < 100; it++) {
        const R f = exact_f(c, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, p0);
        const R fp = exact_dfK(c, rho_L, p_L, a_L, p0) + exact_dfK(c, rho_R, p_R, a_R, p0);
        if (!bracket && f * f_hi < R(0)) {
            bracket = true;
            f_lo = f;
            p_lo = p0;
        }
        const R p1 = p0 - dv(f, fp);
        if (p1 < R(0)) break;
        if (ratio_below(R(2) * fabs(p1 - p0), p1 + p0, c.tol)) {
            *out = p1;
            return DEV_OK;
        }
        p0 = p1;
    }
    if (!bracket) {
        p_lo = R(0);
        f_lo = exact_f(c, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, p_lo);
        if (f_lo * f_hi >= R(0)) {
            p_hi *= R(10);
            const R dp = dv(p_hi - p_lo, R(100));
            for (int i = 0; i < 100; i++) {
                const R a = p_lo + R(i) * dp;
                const R b = p_lo + R(i + 1) * dp;
                const R fa = exact_f(c, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, a);
                const R fb = exact_f(c, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, b);
                if (fa * fb < R(0)) {
                    p_lo = a; f_lo = fa; p_hi = b; f_hi = fb;
                    break;
                }
            }
            if (f_lo * f_hi >= R(0)) return DEV_ERR_EXACT_BRACKET;
        }
    }
    for (int count = 1; count <= 5001; count++) {
        const R pm = R(0.5) * (p_lo + p_hi);
        if (p_hi - p_lo < c.tol) {
            *out = pm;
            return DEV_OK;
        }
        const R fm = exact_f(c, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, pm);
        if (fm * f_lo < R(0)) { p_hi = pm; f_hi = fm; }
        else { p_lo = pm; f_lo = fm; }
        note_bisection_mark(marks, count);
    }
    return DEV_ERR_EXACT_BISECTION;
}

template <class R>
HD void exact_sample(const GasConst<R> &c, R rho_L, R u_L, R p_L, R a_L,
                     R rho_R, R u_R, R p_R, R a_R, R us, R ps, R S, R o[3])
{
    if (S < us) {
        if (ps > p_L) {
            const R r = dv(ps, p_L);
            const R SL = u_L - a_L * sq(c.gp1_2g * r + c.gm1_2g);
            if (S < SL) { o[0] = rho_L; o[1] = u_L; o[2] = p_L; return; }
            const R k = c.gm1_gp1;
            o[0] = dv(rho_L * (r + k), k * r + R(1));
            o[1] = us;
            o[2] = ps;
            return;
        }
        const R SH = u_L - a_L;
        if (S < SH) { o[0] = rho_L; o[1] = u_L; o[2] = p_L; return; }
        const R as = a_L * pw(dv(ps, p_L), c.gm1_2g);
        if (S < us - as) {
            const R cm = pw((c.two_gp1 + (u_L - S) * dv(c.gm1, a_L * c.gp1)), c.two_gm1);
            o[0] = rho_L * cm;
            o[1] = c.two_gp1 * (a_L + R(0.5) * u_L * c.gm1 + S);
            o[2] = p_L * pw(cm, c.gamma);
            return;
        }
        o[0] = rho_L * pw(dv(ps, p_L), c.inv_g);
        o[1] = us;
        o[2] = ps;
        return;
    }
    if (ps > p_R) {
        const R r = dv(ps, p_R);
        const R SR = u_R + a_R * sq(dv(r * c.gp1, R(2) * c.gamma) + c.gm1_2g);
        if (S > SR) { o[0] = rho_R; o[1] = u_R; o[2] = p_R; return; }
        const R k = c.gm1_gp1;
        o[0] = dv(rho_R * (r + k), k * r + R(1));
        o[1] = us;
        o[2] = ps;
        return;
    }
    const R SH = u_R + a_R;
    if (S > SH) { o[0] = rho_R; o[1] = u_R; o[2] = p_R; return; }
    const R as = a_R * pw(dv(ps, p_R), c.gm1_2g);
    if (S > us + as) {
        const R cm = pw((c.two_gp1 - dv((u_R - S) * c.gm1, a_R * c.gp1)), c.two_gm1);
        o[0] = rho_R * cm;
        o[1] = c.two_gp1 * (-a_R + R(0.5) * u_R * c.gm1 + S);
        o[2] = p_R * pw(cm, c.gamma);
        return;
    }
    o[0] = rho_R * pw(dv(ps, p_R), c.inv_g);
    o[1] = us;
    o[2] = ps;
}

/* Exact solution sampled at x/t = S (src/riemann_solver_exact.c:332-469).
 * o = (rho, u, p).  On a p* failure o is zeroed and the error returned. */
template <class R>
HD int exact_solve_1d(const GasConst<R> &c, R rho_L, R u_L, R p_L, R rho_R, R u_R, R p_R, R S, R o[3], unsigned int *marks = nullptr)
{
    const R a_L = (rho_L > R(0)) ? sound_speed(c, rho_L, p_L) : R(0);
    const R a_R = (rho_R > R(0)) ? sound_speed(c, rho_R, p_R) : R(0);
    if (rho_L <= R(0) || rho_R <= R(0) || quot_le((a_L + a_R) * R(2), c.gp1, u_R - u_L)) {
        R s[4];
        solve_vacuum(c, rho_L, u_L, R(0), p_L, a_L, rho_R, u_R, R(0), p_R, a_R, S, s);
        o[0] = s[0]; o[1] = s[1]; o[2] = s[3];
        return DEV_OK;
    }
    R ps = R(0);
    const int rc = exact_p_star(c, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, &ps, marks);
    if (rc != DEV_OK) { o[0] = o[1] = o[2] = R(0); return rc; }
    const R us = R(0.5) * (u_L + u_R)
               + R(0.5) * (exact_fK(c, rho_R, p_R, a_R, ps) - exact_fK(c, rho_L, p_L, a_L, ps));
    exact_sample(c, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, us, ps, S, o);
    return DEV_OK;
}

/* Exact Godunov flux at x/t = S (src/riemann_solver_exact.c:471-510). */
template <class R>
HD int exact_flux_1d(const GasConst<R> &c, R rho_L, R u_L, R p_L, R rho_R, R u_R, R p_R, R S, R F[3],
                     unsigned int *marks = nullptr)
{
    R s[3];
    const int rc = exact_solve_1d(c, rho_L, u_L, p_L, rho_R, u_R, p_R, S, s, marks);
    F[0] = s[0] * s[1];
    F[1] = s[0] * s[1] * s[1] + s[2];
    F[2] = (s[2] * c.g_gm1 + R(0.5) * s[0] * s[1] * s[1]) * s[1];
    return rc;
}

/* ------------------------------------------------------------- predictor */

/*
 * Hancock half-step predictor of one cell along one direction.  q = (rho, n,
 * t, p) with n the velocity along the sweep; d = limited slopes of q;
 * d_rho_vel is the slope entering the density row: the reference uses the
 * slope of the x velocity in both sweeps (:688-693 and :988-993), so the
 * y sweep passes the x-velocity slope here, not d[1].  The literal "+ 0.0"
 * terms of the reference only turn -0.0 into +0.0 and are kept.
 * lo = extrapolated state at the cell's low face, hi = at its high face.
 */
template <class R>
HD void hancock_2d(R dtA, R dtA_rho, R rho, R n, R t, R p, R a,
                   const R d[4], R d_rho_vel, R lo[4], R hi[4])
{
    const R up = R(1) + dtA * n;
    const R um = R(1) - dtA * n;
    const R dr = dtA * rho;
    const R draa = dr * a * a * d[1];
    /* ((0 + 0) + y) + 0 == add_zero(y) and (0 + 0) - y == zero_minus(y): the
     * zero terms in closed form, the same values (x + 0 is idempotent) */
    lo[0] = rho + R(-0.5) * add_zero(up * d[0] + dr * d_rho_vel);
    lo[1] = n + R(-0.5) * (add_zero(up * d[1]) + dtA_rho * d[3]);
    lo[2] = t + R(-0.5) * add_zero(up * d[2]);
    lo[3] = p + R(-0.5) * (add_zero(draa) + up * d[3]);
    hi[0] = rho + R(0.5) * add_zero(um * d[0] - dr * d_rho_vel);
    hi[1] = n + R(0.5) * (add_zero(um * d[1]) - dtA_rho * d[3]);
    hi[2] = t + R(0.5) * add_zero(um * d[2]);
    hi[3] = p + R(0.5) * (zero_minus(draa) + um * d[3]);
}

/* 1D predictor (src/integrator_muscl_hancock.c:185-246). */
template <class R>
HD void hancock_1d(R dtA, R rho, R u, R p, R a, const R d[3], R lo[3], R hi[3])
{
    const R up = R(1) + dtA * u;
    const R um = R(1) - dtA * u;
    const R dr = dtA * rho;
    const R drd = dv(dtA, rho);
    lo[0] = rho + R(-0.5) * (up * d[0] + dr * d[1] + R(0));
    lo[1] = u + R(-0.5) * (R(0) + up * d[1] + drd * d[2]);
    lo[2] = p + R(-0.5) * (R(0) + dr * a * a * d[1] + up * d[2]);
    hi[0] = rho + R(0.5) * (um * d[0] - dr * d[1] + R(0));
    hi[1] = u + R(0.5) * (R(0) + um * d[1] - drd * d[2]);
    hi[2] = p + R(0.5) * (R(0) + -dtA * rho * a * a * d[1] + um * d[2]);
}

/* ------------------------------------------------------------ conversion */

/* U (volume totals) -> W, 2D (src/system.c:763-802). */
template <class R>
HD void cons_to_prim_2d(const GasConst<R> &c, R vol, R m, R mx, R my, R E, R w[4])
{
    w[0] = dv(m, vol);
    w[1] = dv(mx, m);
    w[2] = dv(my, m);
    w[3] = dv(c.gm1 * (E - R(0.5) * m * (w[1] * w[1] + w[2] * w[2])), vol);
}

/* FP32 state: the same conversion, except that where the kinetic energy is
 * more than half of the total energy (E - KE loses at least one bit to
 * cancellation, more as KE -> E) the pressure is recovered in FP64 from the
 * stored conserved values.  For FP64 state this is cons_to_prim_2d. */
template <class R>
HD void cons_to_prim_2d_guarded(const GasConst<R> &c, R vol, R m, R mx, R my, R E, R w[4])
{
    cons_to_prim_2d(c, vol, m, mx, my, E, w);
    if (sizeof(R) == 4) {
        const R ke = R(0.5) * m * (w[1] * w[1] + w[2] * w[2]);
        if (ke > R(0.5) * E) {
            const double md = (double) m, ud = (double) mx / md, vd = (double) my / md;
            const double pd = ((double) c.gm1) * ((double) E - 0.5 * md * (ud * ud + vd * vd)) / (double) vol;
            w[3] = (R) pd;
        }
    }
}

/* Ordered-bits encoding of a double, monotone for every non-NaN value, so a
 * device-wide maximum is one unsigned 64-bit atomicMax. */
HD unsigned long long ordered_bits(double x)
{
    unsigned long long b;
    memcpy(&b, &x, sizeof b);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

HD double from_ordered_bits(unsigned long long e)
{
    const unsigned long long b = (e >> 63) ? (e & 0x7fffffffffffffffull) : ~e;
    double x;
    memcpy(&x, &b, sizeof x);
    return x;
}

/* ---------------------------------------------------------------------- */
/* Source terms (src/source_term.c).  One cell's update each, shared by    */
/* the step kernels and the exported host functions.                       */
/* ---------------------------------------------------------------------- */

/* Rates of the cylindrical / spherical geometry source for density rho,
 * momentum density sm and energy density se; pf = -alpha V / r
 * (src/source_term.c:32-43). */
template <class R>
HD void geometry_rates(R pf, R gm1, R rho, R sm, R se, R &dm, R &dmom, R &de)
{
    const R p = gm1 * (se - dv(R(0.5) * sm * sm, rho));
    dm = pf * sm;
    dmom = dv(pf * sm * sm, rho);
    de = dv(pf * sm * (se + p), rho);
}

/* RK4 step of the geometry source on one cell's totals (m, mom, E) with
 * volume vol and density rho (src/source_term.c:91-165); pf as above. */
template <class R>
HD void geometry_source_rk4(R pf, R gm1, R vol, R dt, R rho, R &m, R &mom, R &E)
{
    R k1m, k1p, k1e, k2m, k2p, k2e, k3m, k3p, k3e, k4m, k4p, k4e;
    geometry_rates(pf, gm1, rho, dv(mom, vol), dv(E, vol), k1m, k1p, k1e);
    R tm = m + R(0.5) * dt * k1m, tp = mom + R(0.5) * dt * k1p, te = E + R(0.5) * dt * k1e;
    geometry_rates(pf, gm1, dv(tm, vol), dv(tp, vol), dv(te, vol), k2m, k2p, k2e);
    tm = m + R(0.5) * dt * k2m;
    tp = mom + R(0.5) * dt * k2p;
    te = E + R(0.5) * dt * k2e;
    geometry_rates(pf, gm1, dv(tm, vol), dv(tp, vol), dv(te, vol), k3m, k3p, k3e);
    tm = m + dt * k3m;
    tp = mom + dt * k3p;
    te = E + dt * k3e;
    geometry_rates(pf, gm1, dv(tm, vol), dv(tp, vol), dv(te, vol), k4m, k4p, k4e);
    m = m + dv(dt * (k1m + R(2) * k2m + R(2) * k3m + k4m), R(6));
    mom = mom + dv(dt * (k1p + R(2) * k2p + R(2) * k3p + k4p), R(6));
    E = E + dv(dt * (k1e + R(2) * k2e + R(2) * k3e + k4e), R(6));
}

/* The gravity kick on one cell's totals with pf = -dt g: the momentum
 * change pf m is exact (the mass does not change), the energy takes the RK4
 * sum (src/source_term.c:213-236). */
template <class R>
HD void gravity_kick(R pf, R mass, R &mom_y, R &E)
{
    const R km = pf * mass;
    const R k1 = pf * mom_y;
    const R k2 = pf * (mom_y + R(0.5) * km);
    const R k3 = k2;
    const R k4 = pf * (mom_y + km);
    mom_y = mom_y + km;
    E = E + dv(k1 + R(2) * k2 + R(2) * k3 + k4, R(6));
}

}  // namespace hydro

#endif
