/*
 * hydro_oracle.c -- TEST INFRASTRUCTURE ONLY (parity checker + "port" CPU
 * baseline).  Never linked into the product library.
 *
 * A CPU restatement of hydroFV's finite-volume step.  Every floating-point
 * expression keeps the reference's operand order and grouping so that, built
 * with -ffp-contract=off, it reproduces the reference bit for bit (the tests
 * pin this against oracle/_ref and tests/golden/).  Citations are
 * path:line in the reference project (alvinng4/hydroFV).
 *
 * Covered: MUSCL-Hancock 2D (src/integrator_muscl_hancock.c:385-1225) and 1D
 * (:26-383), Godunov first order 2D/1D (src/integrator_godunov_first_order.c),
 * HLLC 2D/1D (src/riemann_solver_hllc.c), exact solver 1D
 * (src/riemann_solver_exact.c), limiters (src/slope_limiter.c), built-in
 * boundary conditions (src/boundary.c:411-777), conversions
 * (src/system.c:735-802), CFL time step (src/utils.c:23-95).
 */
#include <math.h>
#include <stdbool.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "hydro_oracle.h"

enum { OK = 0, FAILURE = 1, VALUE_ERROR = 2, POINTER_ERROR = 3, MEMORY_ERROR = 4,
       NOT_IMPLEMENTED_ERROR = 6 };
/* Internal codes of the exact solver's two failures; public_code() and
 * solver_message() turn them into the reference's code and message. */
enum { ERR_EXACT_BRACKET = 101, ERR_EXACT_BISECTION = 102 };
enum { LIM_MINMOD = 1, LIM_VAN_LEER = 2, LIM_MC = 3 };
enum { BC_NONE = 1, BC_REFLECTIVE = 2, BC_TRANSMISSIVE = 3, BC_PERIODIC = 4, BC_CUSTOM = 5 };
enum { SOLVER_EXACT = 1, SOLVER_HLLC = 2 };

#define NEWTON_MAX_ITER 100      /* src/riemann_solver_exact.c:26 */
#define BRACKET_INTERVALS 100    /* src/riemann_solver_exact.c:27 */
#define BISECTION_MAX_ITER 5000  /* src/riemann_solver_exact.c:28 */

static void set_err(char *buf, int len, const char *msg)
{
    if (buf && len > 0) snprintf(buf, (size_t) len, "%s", msg);
}

/* The reference's return code for a solver failure: both exact-solver
 * failures raise FAILURE (src/riemann_solver_exact.c:702-707, :745-754), the
 * HLLC failure VALUE_ERROR (src/riemann_solver_hllc.c:372-375). */
static int public_code(int rc)
{
    return (rc == ERR_EXACT_BRACKET || rc == ERR_EXACT_BISECTION) ? FAILURE : rc;
}

/* The reference's message for a failed Riemann solve. */
static const char *solver_message(int rc)
{
    if (rc == ERR_EXACT_BRACKET) return "Failed to bracket the root for bisection method.";
    if (rc == ERR_EXACT_BISECTION)
        return "Bisection method did not converge after 5001 iterations for exact riemann solver.";
    return "Invalid wave speed for the HLLC riemann solver. Possible fix: use a smaller CFL.";
}

/* ---------------------------------------------------------------- numerics */

/* src/utils.c:23-26 */
static double sound_speed(double gamma, double rho, double p)
{
    return sqrt(gamma * p / rho);
}

/* src/slope_limiter.c:49-91 */
static double limit_slope(int flag, double a, double b)
{
    if (a * b <= 0.0) return 0.0;
    switch (flag)
    {
        case LIM_MINMOD:
            return (fabs(a) < fabs(b)) ? a : b;
        case LIM_VAN_LEER:
            return 2.0 * a * b / (a + b + 1e-10);
        default:
            if (a > 0) return fmin(0.5 * (a + b), 2.0 * fmin(fabs(a), fabs(b)));
            return -fmin(-0.5 * (a + b), 2.0 * fmin(fabs(a), fabs(b)));
    }
}

/* src/riemann_solver.c:144-152 */
static double coef_A(double gamma, double rho) { return 2.0 / ((gamma + 1.0) * rho); }
static double coef_B(double gamma, double p) { return p * ((gamma - 1.0) / (gamma + 1.0)); }

/* Star-pressure initial guess, src/riemann_solver.c:154-224. */
static double guess_p(double gamma, double rho_L, double u_L, double p_L, double a_L,
                      double rho_R, double u_R, double p_R, double a_R, double tol)
{
    const double p_min = (p_L > p_R) ? p_R : p_L;
    const double p_max = (p_L > p_R) ? p_L : p_R;
    const double ppv = 0.5 * (p_L + p_R) - 0.125 * (u_R - u_L) * (rho_L + rho_R) * (a_L + a_R);
    double pg;
    if (p_max / p_min <= 2.0 && (p_min <= ppv && ppv <= p_max))
    {
        pg = ppv;  /* PVRS */
    }
    else if (ppv < p_min)
    {
        /* two-rarefaction */
        const double h = 0.5 * (gamma - 1.0);
        pg = (a_L + a_R - h * (u_R - u_L))
           / (a_L / (pow(p_L, h / gamma)) + a_R / (pow(p_R, h / gamma)));
        pg = pow(pg, gamma / h);
    }
    else
    {
        /* two-shock seeded with PVRS */
        const double gL = sqrt(coef_A(gamma, rho_L) / (ppv + coef_B(gamma, p_L)));
        const double gR = sqrt(coef_A(gamma, rho_R) / (ppv + coef_B(gamma, p_R)));
        pg = (gL * p_L + gR * p_R - (u_R - u_L)) / (gL + gR);
    }
    if (pg < tol) pg = tol;
    return pg;
}

/*
 * Vacuum sampling, src/riemann_solver.c:230-733.  One routine serves 1D and
 * 2D: the tangential velocity is carried through unchanged (or zeroed in the
 * vacuum regime) exactly as the 2D samplers do.  The reference's branch
 * naming (rho_L <= 0 -> "right vacuum" sampler fed with the left state) and
 * the vacuum-generation front speeds 2a/(gamma-1) without the velocity term
 * are reproduced as written (:468-473, :655-660, :710-716).
 */
static void sample_right_vacuum(double gamma, double rho, double u, double v, double p,
                                double a, double S, double *o)
{
    if (S <= (u - a)) { o[0] = rho; o[1] = u; o[2] = v; o[3] = p; return; }
    const double front = u + 2.0 * a / (gamma - 1.0);
    if (S < front)
    {
        double tmp = 2.0 / (gamma + 1.0) + (u - S) * (gamma - 1.0) / ((gamma + 1.0) * a);
        tmp = pow(tmp, 2.0 / (gamma - 1.0));
        o[0] = rho * tmp;
        o[1] = (a + 0.5 * (gamma - 1.0) * u + S) * 2.0 / (gamma + 1.0);
        o[2] = v;
        o[3] = p * pow(tmp, gamma);
    }
    else { o[0] = 0.0; o[1] = 0.0; o[2] = 0.0; o[3] = 0.0; }
}

static void sample_left_vacuum(double gamma, double rho, double u, double v, double p,
                               double a, double S, double *o)
{
    if (S >= (u + a)) { o[0] = rho; o[1] = u; o[2] = v; o[3] = p; return; }
    const double front = u - 2.0 * a / (gamma - 1.0);
    if (S > front)
    {
        double tmp = 2.0 / (gamma + 1.0) - (u - S) * (gamma - 1.0) / ((gamma + 1.0) * a);
        tmp = pow(tmp, 2.0 / (gamma - 1.0));
        o[0] = rho * tmp;
        o[1] = (-a + 0.5 * (gamma - 1.0) * u + S) * 2.0 / (gamma + 1.0);
        o[2] = v;
        o[3] = p * pow(tmp, gamma);
    }
    else { o[0] = 0.0; o[1] = 0.0; o[2] = 0.0; o[3] = 0.0; }
}

static void solve_vacuum(double gamma,
                         double rho_L, double u_L, double v_L, double p_L, double a_L,
                         double rho_R, double u_R, double v_R, double p_R, double a_R,
                         double S, double *o)
{
    if (rho_L <= 0.0 && rho_R <= 0.0) { o[0] = o[1] = o[2] = o[3] = 0.0; return; }
    if (rho_L <= 0.0) { sample_right_vacuum(gamma, rho_L, u_L, v_L, p_L, a_L, S, o); return; }
    if (rho_R <= 0.0) { sample_left_vacuum(gamma, rho_R, u_R, v_R, p_R, a_R, S, o); return; }
    const double SL = 2.0 * a_L / (gamma - 1.0);
    const double SR = 2.0 * a_R / (gamma - 1.0);
    if (S <= SL) { sample_right_vacuum(gamma, rho_L, u_L, v_L, p_L, a_L, S, o); return; }
    if (SR <= S) { sample_left_vacuum(gamma, rho_R, u_R, v_R, p_R, a_R, S, o); return; }
    o[0] = o[1] = o[2] = o[3] = 0.0;
}

/* src/riemann_solver_hllc.c:30-40 */
static double hllc_q(double gamma, double p_X, double p_star)
{
    if (p_star <= p_X) return 1.0;
    return sqrt(1.0 + (0.5 + 0.5 / gamma) * (p_star / p_X - 1.0));
}

/*
 * HLLC flux, 2D form (src/riemann_solver_hllc.c:202-376).  u is the normal
 * velocity, v the tangential one; F = (mass, normal momentum, tangential
 * momentum, energy).
 */
static int hllc_2d(double gamma, double rho_L, double u_L, double v_L, double p_L,
                   double rho_R, double u_R, double v_R, double p_R, double tol, double *F)
{
    const double a_L = (rho_L > 0.0) ? sound_speed(gamma, rho_L, p_L) : 0.0;
    const double a_R = (rho_R > 0.0) ? sound_speed(gamma, rho_R, p_R) : 0.0;
    if (rho_L <= 0.0 || rho_R <= 0.0 || ((a_L + a_R) * 2.0 / (gamma + 1.0)) <= (u_R - u_L))
    {
        double s[4];
        solve_vacuum(gamma, rho_L, u_L, v_L, p_L, a_L, rho_R, u_R, v_R, p_R, a_R, 0.0, s);
        const double E = s[0] * (0.5 * (s[1] * s[1] + s[2] * s[2]) + s[3] / (s[0] * (gamma - 1.0)));
        F[0] = s[0] * s[1];
        F[1] = s[0] * s[1] * s[1] + s[3];
        F[2] = s[0] * s[1] * s[2];
        F[3] = s[1] * (E + s[3]);
        return OK;
    }
    const double ps = guess_p(gamma, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, tol);
    const double S_L = u_L - a_L * hllc_q(gamma, p_L, ps);
    const double S_R = u_R + a_R * hllc_q(gamma, p_R, ps);
    const double S_s = (p_R - p_L + rho_L * u_L * (S_L - u_L) - rho_R * u_R * (S_R - u_R))
                     / (rho_L * (S_L - u_L) - rho_R * (S_R - u_R));
    if (0.0 <= S_L)
    {
        const double E = rho_L * (0.5 * (u_L * u_L + v_L * v_L) + p_L / (rho_L * (gamma - 1.0)));
        F[0] = rho_L * u_L;
        F[1] = rho_L * u_L * u_L + p_L;
        F[2] = rho_L * u_L * v_L;
        F[3] = u_L * (E + p_L);
        return OK;
    }
    if (S_L <= 0.0 && 0.0 <= S_s)
    {
        const double E = rho_L * (0.5 * (u_L * u_L + v_L * v_L) + p_L / (rho_L * (gamma - 1.0)));
        const double fm = rho_L * u_L;
        const double fx = fm * u_L + p_L;
        const double fy = fm * v_L;
        const double fe = u_L * (E + p_L);
        const double rs = rho_L * (S_L - u_L) / (S_L - S_s);
        const double mxs = rs * S_s;
        const double mys = rs * v_L;
        const double es = rs * (E / rho_L + (S_s - u_L) * (S_s + p_L / (rho_L * (S_L - u_L))));
        F[0] = fm + S_L * (rs - rho_L);
        F[1] = fx + S_L * (mxs - rho_L * u_L);
        F[2] = fy + S_L * (mys - rho_L * v_L);
        F[3] = fe + S_L * (es - E);
        return OK;
    }
    if (S_s <= 0.0 && 0.0 <= S_R)
    {
        const double E = rho_R * (0.5 * (u_R * u_R + v_R * v_R) + p_R / (rho_R * (gamma - 1.0)));
        const double fm = rho_R * u_R;
        const double fx = fm * u_R + p_R;
        const double fy = fm * v_R;
        const double fe = u_R * (E + p_R);
        const double rs = rho_R * (S_R - u_R) / (S_R - S_s);
        const double mxs = rs * S_s;
        const double mys = rs * v_R;
        const double es = rs * (E / rho_R + (S_s - u_R) * (S_s + p_R / (rho_R * (S_R - u_R))));
        F[0] = fm + S_R * (rs - rho_R);
        F[1] = fx + S_R * (mxs - rho_R * u_R);
        F[2] = fy + S_R * (mys - rho_R * v_R);
        F[3] = fe + S_R * (es - E);
        return OK;
    }
    if (S_R <= 0.0)
    {
        const double E = rho_R * (0.5 * (u_R * u_R + v_R * v_R) + p_R / (rho_R * (gamma - 1.0)));
        F[0] = rho_R * u_R;
        F[1] = rho_R * u_R * u_R + p_R;
        F[2] = rho_R * u_R * v_R;
        F[3] = u_R * (E + p_R);
        return OK;
    }
    return VALUE_ERROR;  /* "Invalid wave speed for the HLLC riemann solver." :372-375 */
}

/* HLLC flux, 1D form (src/riemann_solver_hllc.c:42-200): note the 1D energy
 * density groups 0.5*u*u as (0.5*u)*u. */
static int hllc_1d(double gamma, double rho_L, double u_L, double p_L,
                   double rho_R, double u_R, double p_R, double tol, double *F)
{
    const double a_L = (rho_L > 0.0) ? sound_speed(gamma, rho_L, p_L) : 0.0;
    const double a_R = (rho_R > 0.0) ? sound_speed(gamma, rho_R, p_R) : 0.0;
    if (rho_L <= 0.0 || rho_R <= 0.0 || ((a_L + a_R) * 2.0 / (gamma + 1.0)) <= (u_R - u_L))
    {
        double s[4];
        solve_vacuum(gamma, rho_L, u_L, 0.0, p_L, a_L, rho_R, u_R, 0.0, p_R, a_R, 0.0, s);
        const double E = s[0] * (0.5 * s[1] * s[1] + s[3] / (s[0] * (gamma - 1.0)));
        F[0] = s[0] * s[1];
        F[1] = s[0] * s[1] * s[1] + s[3];
        F[2] = s[1] * (E + s[3]);
        return OK;
    }
    const double ps = guess_p(gamma, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, tol);
    const double S_L = u_L - a_L * hllc_q(gamma, p_L, ps);
    const double S_R = u_R + a_R * hllc_q(gamma, p_R, ps);
    const double S_s = (p_R - p_L + rho_L * u_L * (S_L - u_L) - rho_R * u_R * (S_R - u_R))
                     / (rho_L * (S_L - u_L) - rho_R * (S_R - u_R));
    if (0.0 <= S_L)
    {
        const double E = rho_L * (0.5 * u_L * u_L + p_L / (rho_L * (gamma - 1.0)));
        F[0] = rho_L * u_L;
        F[1] = rho_L * u_L * u_L + p_L;
        F[2] = u_L * (E + p_L);
        return OK;
    }
    if (S_L <= 0.0 && 0.0 <= S_s)
    {
        const double E = rho_L * (0.5 * u_L * u_L + p_L / (rho_L * (gamma - 1.0)));
        const double fm = rho_L * u_L;
        const double fx = fm * u_L + p_L;
        const double fe = u_L * (E + p_L);
        const double rs = rho_L * (S_L - u_L) / (S_L - S_s);
        const double ms = rs * S_s;
        const double es = rs * (E / rho_L + (S_s - u_L) * (S_s + p_L / (rho_L * (S_L - u_L))));
        F[0] = fm + S_L * (rs - rho_L);
        F[1] = fx + S_L * (ms - rho_L * u_L);
        F[2] = fe + S_L * (es - E);
        return OK;
    }
    if (S_s <= 0.0 && 0.0 <= S_R)
    {
        const double E = rho_R * (0.5 * u_R * u_R + p_R / (rho_R * (gamma - 1.0)));
        const double fm = rho_R * u_R;
        const double fx = fm * u_R + p_R;
        const double fe = u_R * (E + p_R);
        const double rs = rho_R * (S_R - u_R) / (S_R - S_s);
        const double ms = rs * S_s;
        const double es = rs * (E / rho_R + (S_s - u_R) * (S_s + p_R / (rho_R * (S_R - u_R))));
        F[0] = fm + S_R * (rs - rho_R);
        F[1] = fx + S_R * (ms - rho_R * u_R);
        F[2] = fe + S_R * (es - E);
        return OK;
    }
    if (S_R <= 0.0)
    {
        const double E = rho_R * (0.5 * u_R * u_R + p_R / (rho_R * (gamma - 1.0)));
        F[0] = rho_R * u_R;
        F[1] = rho_R * u_R * u_R + p_R;
        F[2] = u_R * (E + p_R);
        return OK;
    }
    return VALUE_ERROR;
}

/* ------------------------------------------------------ exact 1D solver */

/* src/riemann_solver_exact.c:512-536 */
static double exact_fK(double gamma, double rho, double p, double a, double ps)
{
    if (ps > p)
    {
        const double A = coef_A(gamma, rho);
        const double B = coef_B(gamma, p);
        return (ps - p) * sqrt(A / (ps + B));
    }
    return 2.0 * a * (pow((ps / p), (gamma - 1.0) / (2.0 * gamma)) - 1.0) / (gamma - 1.0);
}

/* src/riemann_solver_exact.c:538-565; the shock branch's (B - p*) is kept as
 * written in the reference. */
static double exact_dfK(double gamma, double rho, double p, double a, double ps)
{
    if (ps > p)
    {
        const double A = coef_A(gamma, rho);
        const double B = coef_B(gamma, p);
        return (1.0 - 0.5 * (ps - p) / (B - ps)) * sqrt(A / (B + ps));
    }
    return pow(ps / p, -0.5 * (gamma + 1.0) / gamma) / (p * a);
}

static double exact_f(double gamma, double rho_L, double u_L, double p_L, double a_L,
                      double rho_R, double u_R, double p_R, double a_R, double ps)
{
    return exact_fK(gamma, rho_L, p_L, a_L, ps) + exact_fK(gamma, rho_R, p_R, a_R, ps)
         + (u_R - u_L);
}

/* Newton-Raphson with bisection fallback, src/riemann_solver_exact.c:604-763. */
static int exact_p_star(double gamma, double rho_L, double u_L, double p_L, double a_L,
                        double rho_R, double u_R, double p_R, double a_R, double tol,
                        double *out)
{
    const double pg = guess_p(gamma, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, tol);
    bool bracket = false;
    double p_hi = pg;
    double f_hi = exact_f(gamma, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, p_hi);
    double p_lo = 0.0, f_lo = 0.0;
    double p0 = pg;
    for (int it = 0; it < NEWTON_MAX_ITER; it++)
    {
        const double f = exact_f(gamma, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, p0);
        const double fp = exact_dfK(gamma, rho_L, p_L, a_L, p0) + exact_dfK(gamma, rho_R, p_R, a_R, p0);
        if (!bracket && f * f_hi < 0.0)
        {
            bracket = true;
            f_lo = f;
            p_lo = p0;
        }
        const double p1 = p0 - f / fp;
        if (p1 < 0.0) break;
        if (2.0 * fabs(p1 - p0) / (p1 + p0) < tol)
        {
            *out = p1;
            return OK;
        }
        p0 = p1;
    }
    if (!bracket)
    {
        p_lo = 0.0;
        f_lo = exact_f(gamma, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, p_lo);
        if (f_lo * f_hi >= 0.0)
        {
            p_hi *= 10.0;
            const double dp = (p_hi - p_lo) / BRACKET_INTERVALS;
            for (int i = 0; i < BRACKET_INTERVALS; i++)
            {
                const double a = p_lo + i * dp;
                const double b = p_lo + (i + 1) * dp;
                const double fa = exact_f(gamma, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, a);
                const double fb = exact_f(gamma, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, b);
                if (fa * fb < 0.0)
                {
                    p_lo = a; f_lo = fa; p_hi = b; f_hi = fb;
                    break;
                }
            }
            if (f_lo * f_hi >= 0.0) return ERR_EXACT_BRACKET;
        }
    }
    int count = 0;
    for (;;)
    {
        const double pm = 0.5 * (p_lo + p_hi);
        if (p_hi - p_lo < tol)
        {
            *out = pm;
            return OK;
        }
        const double fm = exact_f(gamma, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, pm);
        if (fm * f_lo < 0.0) { p_hi = pm; f_hi = fm; }
        else { p_lo = pm; f_lo = fm; }
        count++;
        if (count > BISECTION_MAX_ITER) return ERR_EXACT_BISECTION;
    }
}

/* Wave-pattern sampling, src/riemann_solver_exact.c:765-1080. */
static void exact_sample(double gamma, double rho_L, double u_L, double p_L, double a_L,
                         double rho_R, double u_R, double p_R, double a_R,
                         double us, double ps, double S, double *o)
{
    if (S < us)
    {
        if (ps > p_L)
        {
            const double r = ps / p_L;
            const double SL = u_L - a_L * sqrt((gamma + 1.0) / (2.0 * gamma) * r + (gamma - 1.0) / (2.0 * gamma));
            if (S < SL) { o[0] = rho_L; o[1] = u_L; o[2] = p_L; return; }
            const double k = (gamma - 1.0) / (gamma + 1.0);
            o[0] = rho_L * (r + k) / (k * r + 1.0);
            o[1] = us;
            o[2] = ps;
            return;
        }
        const double SH = u_L - a_L;
        if (S < SH) { o[0] = rho_L; o[1] = u_L; o[2] = p_L; return; }
        const double as = a_L * pow(ps / p_L, (gamma - 1.0) / (2.0 * gamma));
        const double ST = us - as;
        if (S < ST)
        {
            const double c2 = 2.0 / (gamma + 1.0);
            const double cm = pow((c2 + (u_L - S) * ((gamma - 1.0) / (a_L * (gamma + 1.0)))), 2.0 / (gamma - 1.0));
            o[0] = rho_L * cm;
            o[1] = c2 * (a_L + 0.5 * u_L * (gamma - 1.0) + S);
            o[2] = p_L * pow(cm, gamma);
            return;
        }
        o[0] = rho_L * pow(ps / p_L, 1.0 / gamma);
        o[1] = us;
        o[2] = ps;
        return;
    }
    if (ps > p_R)
    {
        const double r = ps / p_R;
        const double SR = u_R + a_R * sqrt(r * (gamma + 1.0) / (2.0 * gamma) + (gamma - 1.0) / (2.0 * gamma));
        if (S > SR) { o[0] = rho_R; o[1] = u_R; o[2] = p_R; return; }
        const double k = (gamma - 1.0) / (gamma + 1.0);
        o[0] = rho_R * (r + k) / (k * r + 1.0);
        o[1] = us;
        o[2] = ps;
        return;
    }
    const double SH = u_R + a_R;
    if (S > SH) { o[0] = rho_R; o[1] = u_R; o[2] = p_R; return; }
    const double as = a_R * pow(ps / p_R, (gamma - 1.0) / (2.0 * gamma));
    const double ST = us + as;
    if (S > ST)
    {
        const double c2 = 2.0 / (gamma + 1.0);
        const double cm = pow((c2 - (u_R - S) * (gamma - 1.0) / (a_R * (gamma + 1.0))), 2.0 / (gamma - 1.0));
        o[0] = rho_R * cm;
        o[1] = c2 * (-a_R + 0.5 * u_R * (gamma - 1.0) + S);
        o[2] = p_R * pow(cm, gamma);
        return;
    }
    o[0] = rho_R * pow(ps / p_R, 1.0 / gamma);
    o[1] = us;
    o[2] = ps;
}

/* src/riemann_solver_exact.c:332-510 (flux form with speed S). */
static int exact_flux_1d(double gamma, double rho_L, double u_L, double p_L,
                         double rho_R, double u_R, double p_R, double tol, double S, double *F)
{
    const double a_L = (rho_L > 0.0) ? sound_speed(gamma, rho_L, p_L) : 0.0;
    const double a_R = (rho_R > 0.0) ? sound_speed(gamma, rho_R, p_R) : 0.0;
    double s[4];
    int rc = OK;
    if (rho_L <= 0.0 || rho_R <= 0.0 || ((a_L + a_R) * 2.0 / (gamma + 1.0)) <= (u_R - u_L))
    {
        solve_vacuum(gamma, rho_L, u_L, 0.0, p_L, a_L, rho_R, u_R, 0.0, p_R, a_R, S, s);
        s[2] = s[3];
    }
    else
    {
        double ps;
        rc = exact_p_star(gamma, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, tol, &ps);
        if (rc != OK)
        {
            /* The reference leaves sol_* unset here; report zeros. */
            F[0] = F[1] = F[2] = 0.0;
            return rc;
        }
        const double us = 0.5 * (u_L + u_R) + 0.5 * (exact_fK(gamma, rho_R, p_R, a_R, ps)
                                                    - exact_fK(gamma, rho_L, p_L, a_L, ps));
        exact_sample(gamma, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, us, ps, S, s);
    }
    F[0] = s[0] * s[1];
    F[1] = s[0] * s[1] * s[1] + s[2];
    F[2] = (s[2] * (gamma / (gamma - 1.0)) + 0.5 * s[0] * s[1] * s[1]) * s[1];
    return rc;
}

/* ------------------------------------------------------------ grid helpers */

static int parse_bc(const char *s)
{
    if (!s) return -1;
    if (!strcmp(s, "none")) return BC_NONE;
    if (!strcmp(s, "reflective")) return BC_REFLECTIVE;
    if (!strcmp(s, "transmissive")) return BC_TRANSMISSIVE;
    if (!strcmp(s, "periodic")) return BC_PERIODIC;
    if (!strcmp(s, "custom")) return BC_CUSTOM;
    return -1;
}

static int parse_limiter(const char *s)
{
    if (!s) return -1;
    if (!strcmp(s, "minmod")) return LIM_MINMOD;
    if (!strcmp(s, "van_leer")) return LIM_VAN_LEER;
    if (!strcmp(s, "monotonized_central")) return LIM_MC;
    return -1;
}

typedef struct
{
    int nx, ny, g, tx;           /* tx = nx + 2g (row length) */
    double gamma, dx, dy, A_x, A_y, vol;
    int lim, solver;
    double tol;
    int bc[4];                   /* x_min, x_max, y_min, y_max */
    OracleBcFn custom[4];        /* callbacks of custom sides (src/boundary.h:40-48) */
    double gravity;              /* System.gravity */
    double *W[4];                /* rho, u, v, p */
    double *U[4];                /* mass, mom_x, mom_y, energy */
} Grid;

/* src/system.c:763-802 over every padded cell (ghosts included). */
static void conserved_to_primitive_2d(Grid *G)
{
    const int ty = G->ny + 2 * G->g;
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < G->tx; i++)
    {
        for (int j = 0; j < ty; j++)
        {
            const int k = j * G->tx + i;
            const double m = G->U[0][k], mx = G->U[1][k], my = G->U[2][k], E = G->U[3][k];
            G->W[0][k] = m / G->vol;
            G->W[1][k] = mx / m;
            G->W[2][k] = my / m;
            G->W[3][k] = (G->gamma - 1.0) * (E - 0.5 * m * (G->W[1][k] * G->W[1][k] + G->W[2][k] * G->W[2][k])) / G->vol;
        }
    }
}

/* Built-in ghost fill on the primitives, src/boundary.c:513-777.  x sides over
 * interior rows, then y sides over interior columns; corners untouched.
 * Transmissive is a mirror copy, reflective additionally negates the normal
 * velocity, periodic copies from the opposite interior (done in the *_max
 * case, as the reference does). */
static void boundary_2d(Grid *G)
{
    const int g = G->g, nx = G->nx, ny = G->ny, tx = G->tx;
    double **W = G->W;
    for (int side = 0; side < 2; side++)
    {
        const int f = G->bc[side];
        if (f == BC_CUSTOM)
        {
            G->custom[side](W[0], W[1], W[2], W[3], g, nx, ny);
            continue;
        }
        if (f == BC_NONE || (f == BC_PERIODIC && side == 0)) continue;
        for (int k = 0; k < g; k++)
        {
            for (int j = g; j < g + ny; j++)
            {
                int dst, src;
                if (f == BC_PERIODIC)
                {
                    /* right ghost <- left interior, then left ghost <- right interior */
                    dst = j * tx + (g + nx + k); src = j * tx + (g + k);
                    for (int q = 0; q < 4; q++) W[q][dst] = W[q][src];
                    dst = j * tx + (g - 1 - k); src = j * tx + (g + nx - 1 - k);
                    for (int q = 0; q < 4; q++) W[q][dst] = W[q][src];
                    continue;
                }
                if (side == 0) { dst = j * tx + (g - 1 - k); src = j * tx + (g + k); }
                else { dst = j * tx + (g + nx + k); src = j * tx + (g + nx - 1 - k); }
                W[0][dst] = W[0][src];
                W[1][dst] = (f == BC_REFLECTIVE) ? -W[1][src] : W[1][src];
                W[2][dst] = W[2][src];
                W[3][dst] = W[3][src];
            }
        }
    }
    for (int side = 0; side < 2; side++)
    {
        const int f = G->bc[2 + side];
        if (f == BC_CUSTOM)
        {
            G->custom[2 + side](W[0], W[1], W[2], W[3], g, nx, ny);
            continue;
        }
        if (f == BC_NONE || (f == BC_PERIODIC && side == 0)) continue;
        for (int i = g; i < g + nx; i++)
        {
            for (int k = 0; k < g; k++)
            {
                int dst, src;
                if (f == BC_PERIODIC)
                {
                    dst = (g + ny + k) * tx + i; src = (g + k) * tx + i;
                    for (int q = 0; q < 4; q++) W[q][dst] = W[q][src];
                    dst = (g - 1 - k) * tx + i; src = (g + ny - 1 - k) * tx + i;
                    for (int q = 0; q < 4; q++) W[q][dst] = W[q][src];
                    continue;
                }
                if (side == 0) { dst = (g - 1 - k) * tx + i; src = (g + k) * tx + i; }
                else { dst = (g + ny + k) * tx + i; src = (g + ny - 1 - k) * tx + i; }
                W[0][dst] = W[0][src];
                W[1][dst] = W[1][src];
                W[2][dst] = (f == BC_REFLECTIVE) ? -W[2][src] : W[2][src];
                W[3][dst] = W[3][src];
            }
        }
    }
}

/* src/utils.c:55-95: max over interior cells of a+|u| and a+|v|. */
static double time_step_2d(const Grid *G, double cfl)
{
    double sx = -INFINITY, sy = -INFINITY;
    for (int i = G->g; i < G->g + G->nx; i++)
    {
        for (int j = G->g; j < G->g + G->ny; j++)
        {
            const int k = j * G->tx + i;
            const double a = sound_speed(G->gamma, G->W[0][k], G->W[3][k]);
            const double vx = fabs(G->W[1][k]);
            const double vy = fabs(G->W[2][k]);
            if (a + vx > sx) sx = a + vx;
            if (a + vy > sy) sy = a + vy;
        }
    }
    return cfl / (sx / G->dx + sy / G->dy);
}

/*
 * Hancock half-step predictor for one cell in one direction
 * (src/integrator_muscl_hancock.c:682-755 for x, :967-1041 for y).
 * q = (rho, n, t, p) with n the velocity along the sweep and t the other
 * one.  For the y sweep the reference's density row uses the limited slope
 * of the x velocity (:988-993, :1014-1019) -- reproduced through `d_rho_vel`,
 * which the caller sets to the slope of u in both sweeps.
 * Outputs: lo = state at the cell's low face, hi = state at its high face.
 */
static void hancock(double dtA, double rho, double n, double t, double p, double a,
                    const double d[4], double d_rho_vel, double *lo, double *hi)
{
    /* d = limited slopes of (rho, n, t, p) */
    const double up = 1.0 + dtA * n;
    const double um = 1.0 - dtA * n;
    const double l_rho = -0.5 * (up * d[0] + dtA * rho * d_rho_vel + 0.0 + 0.0);
    const double l_n = -0.5 * (0.0 + up * d[1] + 0.0 + (dtA / rho) * d[3]);
    const double l_t = -0.5 * (0.0 + 0.0 + up * d[2] + 0.0);
    const double l_p = -0.5 * (0.0 + dtA * rho * a * a * d[1] + 0.0 + up * d[3]);
    const double h_rho = 0.5 * (um * d[0] - dtA * rho * d_rho_vel + 0.0 + 0.0);
    const double h_n = 0.5 * (0.0 + um * d[1] + 0.0 - (dtA / rho) * d[3]);
    const double h_t = 0.5 * (0.0 + 0.0 + um * d[2] + 0.0);
    const double h_p = 0.5 * (0.0 + 0.0 - dtA * rho * a * a * d[1] + um * d[3]);
    lo[0] = rho + l_rho; lo[1] = n + l_n; lo[2] = t + l_t; lo[3] = p + l_p;
    hi[0] = rho + h_rho; hi[1] = n + h_n; hi[2] = t + h_t; hi[3] = p + h_p;
}

/*
 * One MUSCL-Hancock 2D step (src/integrator_muscl_hancock.c:552-1115).
 * Both sweeps read the same W; U is updated in place, x faces then y faces.
 * Returns OK or the first error code.
 */
static int mh2d_step(Grid *G, double dt)
{
    const int g = G->g, nx = G->nx, ny = G->ny, tx = G->tx;
    double **W = G->W, **U = G->U;
    int err = OK;

    #pragma omp parallel
    {
        double (*Lx)[4] = malloc(sizeof(double[4]) * (size_t) (nx + 1));
        double (*Rx)[4] = malloc(sizeof(double[4]) * (size_t) (nx + 1));
        double (*Ly)[4] = malloc(sizeof(double[4]) * (size_t) (ny + 1));
        double (*Ry)[4] = malloc(sizeof(double[4]) * (size_t) (ny + 1));
        int local_err = OK;

        /* x sweep, rows in parallel */
        #pragma omp for
        for (int j = g; j < g + ny; j++)
        {
            for (int i = 0; i < nx + 2; i++)
            {
                const int k = j * tx + (i + g - 1);
                const double rho = W[0][k], u = W[1][k], v = W[2][k], p = W[3][k];
                const double dtA = dt * G->A_x / G->vol;
                const double a = sound_speed(G->gamma, rho, p);
                double d[4];
                for (int q = 0; q < 4; q++)
                    d[q] = limit_slope(G->lim, W[q][k] - W[q][k - 1], W[q][k + 1] - W[q][k]);
                const double dd[4] = { d[0], d[1], d[2], d[3] };
                double lo[4], hi[4];
                hancock(dtA, rho, u, v, p, a, dd, d[1], lo, hi);
                if (i > 0) memcpy(Rx[i - 1], lo, sizeof lo);
                if (i < nx + 1) memcpy(Lx[i], hi, sizeof hi);
            }
            for (int i = 0; i < nx + 1; i++)
            {
                double F[4];
                const int rc = hllc_2d(G->gamma, Lx[i][0], Lx[i][1], Lx[i][2], Lx[i][3],
                                       Rx[i][0], Rx[i][1], Rx[i][2], Rx[i][3], G->tol, F);
                if (rc != OK) local_err = rc;
                const int kl = j * tx + (g + i - 1), kr = kl + 1;
                for (int q = 0; q < 4; q++)
                {
                    const double dq = F[q] * dt;
                    U[q][kl] -= dq * G->A_x;
                    U[q][kr] += dq * G->A_x;
                }
            }
        }

        /* y sweep, columns in parallel; the solver sees (rho, v, u, p) */
        #pragma omp for
        for (int i = g; i < g + nx; i++)
        {
            for (int j = 0; j < ny + 2; j++)
            {
                const int k = (j + g - 1) * tx + i;
                const double rho = W[0][k], u = W[1][k], v = W[2][k], p = W[3][k];
                const double dtA = dt * G->A_y / G->vol;
                const double a = sound_speed(G->gamma, rho, p);
                double d[4];
                for (int q = 0; q < 4; q++)
                    d[q] = limit_slope(G->lim, W[q][k] - W[q][k - tx], W[q][k + tx] - W[q][k]);
                /* reorder to (rho, n=v, t=u, p); density row uses slope of u */
                const double dd[4] = { d[0], d[2], d[1], d[3] };
                double lo[4], hi[4];
                hancock(dtA, rho, v, u, p, a, dd, d[1], lo, hi);
                if (j > 0) memcpy(Ry[j - 1], lo, sizeof lo);
                if (j < ny + 1) memcpy(Ly[j], hi, sizeof hi);
            }
            for (int j = 0; j < ny + 1; j++)
            {
                double F[4];
                const int rc = hllc_2d(G->gamma, Ly[j][0], Ly[j][1], Ly[j][2], Ly[j][3],
                                       Ry[j][0], Ry[j][1], Ry[j][2], Ry[j][3], G->tol, F);
                if (rc != OK) local_err = rc;
                /* F = (mass, mom_y, mom_x, energy) */
                const double Fq[4] = { F[0], F[2], F[1], F[3] };
                const int kb = (g + j - 1) * tx + i, kt = kb + tx;
                for (int q = 0; q < 4; q++)
                {
                    const double dq = Fq[q] * dt;
                    U[q][kb] -= dq * G->A_y;
                    U[q][kt] += dq * G->A_y;
                }
            }
        }
        #pragma omp critical
        {
            if (local_err != OK) err = local_err;
        }
        free(Lx); free(Rx); free(Ly); free(Ry);
    }
    return err;
}

/* One Godunov first-order 2D step (src/integrator_godunov_first_order.c:
 * 356-480): cell states are the Riemann data; dt*F*A grouping. */
static int godunov2d_step(Grid *G, double dt)
{
    const int g = G->g, nx = G->nx, ny = G->ny, tx = G->tx;
    double **W = G->W, **U = G->U;
    int err = OK;
    #pragma omp parallel for
    for (int j = g; j < g + ny; j++)
    {
        for (int i = g; i < g + nx + 1; i++)
        {
            const int kl = j * tx + (i - 1), kr = kl + 1;
            double F[4];
            const int rc = hllc_2d(G->gamma, W[0][kl], W[1][kl], W[2][kl], W[3][kl],
                                   W[0][kr], W[1][kr], W[2][kr], W[3][kr], G->tol, F);
            if (rc != OK)
            {
                #pragma omp critical
                err = rc;
            }
            for (int q = 0; q < 4; q++)
            {
                U[q][kl] -= dt * F[q] * G->A_x;
                U[q][kr] += dt * F[q] * G->A_x;
            }
        }
    }
    if (err != OK) return err;
    #pragma omp parallel for
    for (int i = g; i < g + nx; i++)
    {
        for (int j = g; j < g + ny + 1; j++)
        {
            const int kb = (j - 1) * tx + i, kt = kb + tx;
            double F[4];
            const int rc = hllc_2d(G->gamma, W[0][kb], W[2][kb], W[1][kb], W[3][kb],
                                   W[0][kt], W[2][kt], W[1][kt], W[3][kt], G->tol, F);
            if (rc != OK)
            {
                #pragma omp critical
                err = rc;
            }
            const double Fq[4] = { F[0], F[2], F[1], F[3] };
            for (int q = 0; q < 4; q++)
            {
                U[q][kb] -= dt * Fq[q] * G->A_y;
                U[q][kt] += dt * Fq[q] * G->A_y;
            }
        }
    }
    return err;
}

/* Gravity source (src/source_term.c:185-259): RK4 kick of the interior
 * momentum_y / energy after the step's conversion and boundary routine, then
 * the conversion and the boundary routine again. */
static void gravity_2d(Grid *G, double dt)
{
    if (G->gravity == 0.0) return;
    const int g = G->g;
    for (int i = g; i < g + G->nx; i++)
    {
        for (int j = g; j < g + G->ny; j++)
        {
            const int k = j * G->tx + i;
            const double m = G->U[0][k];
            const double my = G->U[2][k];
            const double pf = - dt * G->gravity;
            const double km = pf * m;
            const double k1 = pf * my;
            const double k2 = pf * (my + 0.5 * km);
            const double k3 = k2;
            const double k4 = pf * (my + km);
            G->U[2][k] += km;
            G->U[3][k] += (k1 + 2.0 * k2 + 2.0 * k3 + k4) / 6.0;
        }
    }
    conserved_to_primitive_2d(G);
    boundary_2d(G);
}

int oracle_run_2d(
    int nx, int ny, int g,
    double x_min, double x_max, double y_min, double y_max, double gamma,
    const char *integrator, const char *riemann_solver, const char *slope_limiter,
    const char *bc_x_min, const char *bc_x_max, const char *bc_y_min, const char *bc_y_max,
    double cfl, double tf, long long max_steps,
    double *rho, double *u, double *v, double *p,
    double *mass, double *mom_x, double *mom_y, double *energy,
    long long *num_steps, double *t, double *dt,
    char *errbuf, int errlen)
{
    return oracle_run_2d_ex(nx, ny, g, x_min, x_max, y_min, y_max, gamma, integrator, riemann_solver,
                            slope_limiter, bc_x_min, bc_x_max, bc_y_min, bc_y_max, cfl, tf, max_steps,
                            rho, u, v, p, mass, mom_x, mom_y, energy, num_steps, t, dt, errbuf, errlen,
                            0.0, NULL, NULL, NULL, NULL);
}

int oracle_run_2d_ex(
    int nx, int ny, int g,
    double x_min, double x_max, double y_min, double y_max, double gamma,
    const char *integrator, const char *riemann_solver, const char *slope_limiter,
    const char *bc_x_min, const char *bc_x_max, const char *bc_y_min, const char *bc_y_max,
    double cfl, double tf, long long max_steps,
    double *rho, double *u, double *v, double *p,
    double *mass, double *mom_x, double *mom_y, double *energy,
    long long *num_steps, double *t, double *dt,
    char *errbuf, int errlen,
    double gravity, OracleBcFn bc_fn_x_min, OracleBcFn bc_fn_x_max, OracleBcFn bc_fn_y_min,
    OracleBcFn bc_fn_y_max)
{
    set_err(errbuf, errlen, "");
    *num_steps = 0; *t = 0.0; *dt = 0.0;
    const int is_mh = integrator && !strcmp(integrator, "muscl_hancock_2d");
    const int is_god = integrator && !strcmp(integrator, "godunov_first_order_2d");
    if (!is_mh && !is_god) { set_err(errbuf, errlen, "Integrator not recognized."); return VALUE_ERROR; }
    if (!riemann_solver || strcmp(riemann_solver, "riemann_solver_hllc"))
    {
        set_err(errbuf, errlen, "Only HLLC Riemann solver is available for cartesian 2D.");
        return VALUE_ERROR;
    }
    Grid G;
    G.nx = nx; G.ny = ny; G.g = g; G.tx = nx + 2 * g;
    G.gamma = gamma;
    /* src/system.c:291-309, :365-529 */
    G.dx = (x_max - x_min) / (nx + 2 * g);
    G.dy = (y_max - y_min) / (ny + 2 * g);
    G.A_x = G.dy; G.A_y = G.dx; G.vol = G.dx * G.dy;
    G.lim = parse_limiter(slope_limiter);
    G.solver = SOLVER_HLLC;
    G.tol = 1e-6;  /* src/integrator.c:25 */
    G.bc[0] = parse_bc(bc_x_min); G.bc[1] = parse_bc(bc_x_max);
    G.bc[2] = parse_bc(bc_y_min); G.bc[3] = parse_bc(bc_y_max);
    if (G.lim < 0) { set_err(errbuf, errlen, "Slope limiter not recognized."); return VALUE_ERROR; }
    for (int s = 0; s < 4; s++)
        if (G.bc[s] < 0) { set_err(errbuf, errlen, "Boundary condition not recognized."); return VALUE_ERROR; }
    /* a periodic side needs a periodic opposite side: y pair, then x pair
     * (src/boundary.c:258-305) */
    if ((G.bc[2] == BC_PERIODIC || G.bc[3] == BC_PERIODIC) && G.bc[2] != G.bc[3])
    {
        set_err(errbuf, errlen, "Periodic boundary condition mismatch for y_min and y_max.");
        return VALUE_ERROR;
    }
    if ((G.bc[0] == BC_PERIODIC || G.bc[1] == BC_PERIODIC) && G.bc[0] != G.bc[1])
    {
        set_err(errbuf, errlen, "Periodic boundary condition mismatch for x_min and x_max.");
        return VALUE_ERROR;
    }
    G.custom[0] = bc_fn_x_min; G.custom[1] = bc_fn_x_max;
    G.custom[2] = bc_fn_y_min; G.custom[3] = bc_fn_y_max;
    for (int s = 0; s < 4; s++)
        if (G.bc[s] == BC_CUSTOM && !G.custom[s])
        {
            set_err(errbuf, errlen, "A custom boundary condition needs its callback.");
            return VALUE_ERROR;
        }
    G.gravity = gravity;
    G.W[0] = rho; G.W[1] = u; G.W[2] = v; G.W[3] = p;
    G.U[0] = mass; G.U[1] = mom_x; G.U[2] = mom_y; G.U[3] = energy;

    const double shrink = 0.2;   /* src/integrator.c:23-24 */
    const int shrink_steps = 10;
    const double t_end = (max_steps >= 0) ? INFINITY : tf;
    while (*t < t_end && (max_steps < 0 || *num_steps < max_steps))
    {
        double step = time_step_2d(&G, (*num_steps < shrink_steps) ? cfl * shrink : cfl);
        if (*t + step > t_end) step = t_end - *t;
        *dt = step;
        if (step == 0.0) { set_err(errbuf, errlen, "dt is zero."); return VALUE_ERROR; }
        const int rc = is_mh ? mh2d_step(&G, step) : godunov2d_step(&G, step);
        if (rc != OK)
        {
            set_err(errbuf, errlen, "Invalid wave speed for the HLLC riemann solver. Possible fix: use a smaller CFL.");
            return rc;
        }
        conserved_to_primitive_2d(&G);
        boundary_2d(&G);
        gravity_2d(&G, step);
        *t += step;
        (*num_steps)++;
    }
    return OK;
}

/* ------------------------------------------------------------------- 1D */

typedef struct
{
    int nx, g;
    double gamma, dx, tol;
    double *A, *V, *X;           /* surface_area_x (per cell index), volume, mid_points_x */
    double alpha;                /* 0 Cartesian, 1 cylindrical, 2 spherical */
    int lim, solver, bc[2];
    double *W[3], *U[3];
} Grid1;

/* src/system.c:318-356, :365-529 for the 1D coordinate systems. */
static void geometry_1d(Grid1 *G, double x_min, int coord)
{
    const int tot = G->nx + 2 * G->g;
    const double dx = G->dx;
    for (int i = 0; i < tot; i++) G->X[i] = x_min + (i + 0.5) * dx;
    for (int i = 0; i < tot + 1; i++)
    {
        const double r = x_min + i * dx;
        if (coord == 1) G->A[i] = 1.0;
        else if (coord == 2) G->A[i] = (i == 0) ? 0.0 : 2.0 * M_PI * r;
        else G->A[i] = 4.0 * M_PI * r * r;
    }
    for (int i = 0; i < tot; i++)
    {
        const double r_min = x_min + i * dx;
        const double r_max = x_min + (i + 1) * dx;
        if (coord == 1) G->V[i] = dx;
        else if (coord == 2) G->V[i] = M_PI * (r_max * r_max - r_min * r_min);
        else G->V[i] = (4.0 / 3.0) * M_PI * (r_max * r_max * r_max - r_min * r_min * r_min);
    }
}

/* src/system.c:735-761 */
static void conserved_to_primitive_1d(Grid1 *G)
{
    for (int i = 0; i < G->nx + 2 * G->g; i++)
    {
        const double m = G->U[0][i], mx = G->U[1][i], E = G->U[2][i];
        G->W[0][i] = m / G->V[i];
        G->W[1][i] = mx / m;
        G->W[2][i] = (G->gamma - 1.0) * (E - 0.5 * m * G->W[1][i] * G->W[1][i]) / G->V[i];
    }
}

/* src/system.c:866-883 */
static void primitive_to_conserved_1d(Grid1 *G)
{
    for (int i = 0; i < G->nx + 2 * G->g; i++)
    {
        const double rho = G->W[0][i], u = G->W[1][i], p = G->W[2][i], V = G->V[i];
        G->U[0][i] = rho * V;
        G->U[1][i] = G->U[0][i] * u;
        G->U[2][i] = V * (0.5 * rho * u * u + p / (G->gamma - 1.0));
    }
}

/* src/boundary.c:411-511 */
static void boundary_1d(Grid1 *G)
{
    const int g = G->g, n = G->nx;
    double **W = G->W;
    for (int side = 0; side < 2; side++)
    {
        const int f = G->bc[side];
        if (f == BC_NONE || (f == BC_PERIODIC && side == 0)) continue;
        for (int k = 0; k < g; k++)
        {
            if (f == BC_PERIODIC)
            {
                for (int q = 0; q < 3; q++) W[q][g + n + k] = W[q][g + k];
                for (int q = 0; q < 3; q++) W[q][g - 1 - k] = W[q][g + n - 1 - k];
                continue;
            }
            const int dst = (side == 0) ? g - 1 - k : g + n + k;
            const int src = (side == 0) ? g + k : g + n - 1 - k;
            W[0][dst] = W[0][src];
            W[1][dst] = (f == BC_REFLECTIVE) ? -W[1][src] : W[1][src];
            W[2][dst] = W[2][src];
        }
    }
}

/* src/utils.c:28-53 */
static double time_step_1d(const Grid1 *G, double cfl)
{
    double s = -INFINITY;
    for (int i = G->g; i < G->nx + G->g; i++)
    {
        const double a = sound_speed(G->gamma, G->W[0][i], G->W[2][i]);
        const double w = fabs(G->W[1][i]);
        if (a + w > s) s = a + w;
    }
    return cfl * G->dx / s;
}

static int flux_1d(const Grid1 *G, double rl, double ul, double pl, double rr, double ur, double pr, double *F)
{
    if (G->solver == SOLVER_EXACT) return exact_flux_1d(G->gamma, rl, ul, pl, rr, ur, pr, G->tol, 0.0, F);
    return hllc_1d(G->gamma, rl, ul, pl, rr, ur, pr, G->tol, F);
}

/* src/integrator_godunov_first_order.c:152-193 (serial order): the flux of
 * face i updates cell i-1 with surface_area_x[i-1] and cell i with
 * surface_area_x[i]. */
static int godunov1d_step(Grid1 *G, double dt)
{
    double **W = G->W, **U = G->U;
    for (int i = G->g; i < G->g + G->nx + 1; i++)
    {
        double F[3];
        const int rc = flux_1d(G, W[0][i - 1], W[1][i - 1], W[2][i - 1], W[0][i], W[1][i], W[2][i], F);
        if (rc != OK) return rc;
        for (int q = 0; q < 3; q++)
        {
            const double d = F[q] * dt;
            U[q][i - 1] -= d * G->A[i - 1];
            U[q][i] += d * G->A[i];
        }
    }
    return OK;
}

/* src/integrator_muscl_hancock.c:159-295 (serial order).  The reference does
 * not stop on a flux error here (the status is overwritten by the boundary
 * call at :309), so neither does the restatement. */
static int mh1d_step(Grid1 *G, double dt)
{
    const int n = G->nx, g = G->g;
    double **W = G->W, **U = G->U;
    double (*L)[3] = malloc(sizeof(double[3]) * (size_t) (n + 1));
    double (*R)[3] = malloc(sizeof(double[3]) * (size_t) (n + 1));
    if (!L || !R) { free(L); free(R); return MEMORY_ERROR; }
    for (int i = 0; i < n + 2; i++)
    {
        const int k = g + i - 1;
        const double rho = W[0][k], u = W[1][k], p = W[2][k];
        const double dtA = dt * G->A[k] / G->V[k];
        const double a = sound_speed(G->gamma, rho, p);
        double d[3];
        for (int q = 0; q < 3; q++)
            d[q] = limit_slope(G->lim, W[q][k] - W[q][k - 1], W[q][k + 1] - W[q][k]);
        const double l_rho = -0.5 * ((1.0 + dtA * u) * d[0] + dtA * rho * d[1] + 0.0);
        const double l_u = -0.5 * (0.0 + (1.0 + dtA * u) * d[1] + (dtA / rho) * d[2]);
        const double l_p = -0.5 * (0.0 + dtA * rho * a * a * d[1] + (1.0 + dtA * u) * d[2]);
        const double h_rho = 0.5 * ((1.0 - dtA * u) * d[0] - dtA * rho * d[1] + 0.0);
        const double h_u = 0.5 * (0.0 + (1.0 - dtA * u) * d[1] - (dtA / rho) * d[2]);
        const double h_p = 0.5 * (0.0 + -dtA * rho * a * a * d[1] + (1.0 - dtA * u) * d[2]);
        if (i > 0) { R[i - 1][0] = rho + l_rho; R[i - 1][1] = u + l_u; R[i - 1][2] = p + l_p; }
        if (i < n + 1) { L[i][0] = rho + h_rho; L[i][1] = u + h_u; L[i][2] = p + h_p; }
    }
    for (int i = 0; i < n + 1; i++)
    {
        double F[3] = { 0.0, 0.0, 0.0 };
        (void) flux_1d(G, L[i][0], L[i][1], L[i][2], R[i][0], R[i][1], R[i][2], F);
        const int k = g + i;
        for (int q = 0; q < 3; q++)
        {
            const double d = F[q] * dt;
            U[q][k - 1] -= d * G->A[k - 1];
            U[q][k] += d * G->A[k];
        }
    }
    free(L); free(R);
    return OK;
}

/* src/integrator_random_choice_1d.c:28-43 */
static double van_der_corput(long long n)
{
    double result = 0;
    const int base = 5;
    double bk = 1.0 / (double) base;
    while (n > 0)
    {
        const int a_i = (int) (n % base);
        const int A_i = (3 * a_i) % 5;
        result += A_i * bk;
        n /= base;
        bk /= (double) base;
    }
    return result;
}

/* src/riemann_solver_exact.c:332-469: the exact solution sampled at x/t = S. */
static int exact_state_1d(double gamma, double rho_L, double u_L, double p_L,
                          double rho_R, double u_R, double p_R, double tol, double S, double *o)
{
    const double a_L = (rho_L > 0.0) ? sound_speed(gamma, rho_L, p_L) : 0.0;
    const double a_R = (rho_R > 0.0) ? sound_speed(gamma, rho_R, p_R) : 0.0;
    double s[4];
    if (rho_L <= 0.0 || rho_R <= 0.0 || ((a_L + a_R) * 2.0 / (gamma + 1.0)) <= (u_R - u_L))
    {
        solve_vacuum(gamma, rho_L, u_L, 0.0, p_L, a_L, rho_R, u_R, 0.0, p_R, a_R, S, s);
        o[0] = s[0]; o[1] = s[1]; o[2] = s[3];
        return OK;
    }
    double ps;
    const int rc = exact_p_star(gamma, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, tol, &ps);
    if (rc != OK) return rc;
    const double us = 0.5 * (u_L + u_R) + 0.5 * (exact_fK(gamma, rho_R, p_R, a_R, ps)
                                                - exact_fK(gamma, rho_L, p_L, a_L, ps));
    exact_sample(gamma, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, us, ps, S, o);
    return OK;
}

/* One random-choice step (src/integrator_random_choice_1d.c:157-237), then
 * the boundary routine and W -> U. */
static int random_choice_step(Grid1 *G, double dt, long long step_index)
{
    const int n = G->nx, g = G->g, tot = n + 2 * g;
    double **W = G->W;
    const double theta = van_der_corput(step_index + 1);
    double *T = malloc(sizeof(double) * 3 * (size_t) tot);
    if (!T) return MEMORY_ERROR;
    for (int q = 0; q < 3; q++) memcpy(T + q * tot, W[q], sizeof(double) * (size_t) tot);
    int err = OK;
    for (int i = g; i < g + n + 1; i++)
    {
        const int left = theta <= 0.5;
        const int l = left ? i - 1 : i, r = left ? i : i + 1;
        const double speed = left ? theta * G->dx / dt : (theta - 1.0) * G->dx / dt;
        double o[3];
        const int rc = exact_state_1d(G->gamma, T[l], T[tot + l], T[2 * tot + l], T[r], T[tot + r], T[2 * tot + r],
                                      G->tol, speed, o);
        if (rc != OK) { err = rc; continue; }
        W[0][i] = o[0]; W[1][i] = o[1]; W[2][i] = o[2];
    }
    free(T);
    if (err != OK) return err;
    boundary_1d(G);
    primitive_to_conserved_1d(G);
    return OK;
}

/* Cylindrical / spherical source, RK4 (src/source_term.c:14-183), then
 * U -> W and the boundary routine. */
static void rates(double pf, double gamma, double rho, double sm, double se, double *dm, double *dp, double *de)
{
    const double p = (gamma - 1) * (se - 0.5 * sm * sm / rho);
    *dm = pf * sm;
    *dp = pf * sm * sm / rho;
    *de = pf * sm * (se + p) / rho;
}

static void geometry_source_1d(Grid1 *G, double dt)
{
    if (G->alpha == 0.0) return;
    double **U = G->U;
    for (int i = G->g; i < G->nx + G->g; i++)
    {
        const double V = G->V[i], m = U[0][i], mom = U[1][i], E = U[2][i], rho = G->W[0][i];
        const double pf = -G->alpha * V / G->X[i];
        double k1m, k1p, k1e, k2m, k2p, k2e, k3m, k3p, k3e, k4m, k4p, k4e;
        rates(pf, G->gamma, rho, mom / V, E / V, &k1m, &k1p, &k1e);
        double tm = m + 0.5 * dt * k1m, tp = mom + 0.5 * dt * k1p, te = E + 0.5 * dt * k1e;
        rates(pf, G->gamma, tm / V, tp / V, te / V, &k2m, &k2p, &k2e);
        tm = m + 0.5 * dt * k2m; tp = mom + 0.5 * dt * k2p; te = E + 0.5 * dt * k2e;
        rates(pf, G->gamma, tm / V, tp / V, te / V, &k3m, &k3p, &k3e);
        tm = m + dt * k3m; tp = mom + dt * k3p; te = E + dt * k3e;
        rates(pf, G->gamma, tm / V, tp / V, te / V, &k4m, &k4p, &k4e);
        U[0][i] += dt * (k1m + 2.0 * k2m + 2.0 * k3m + k4m) / 6.0;
        U[1][i] += dt * (k1p + 2.0 * k2p + 2.0 * k3p + k4p) / 6.0;
        U[2][i] += dt * (k1e + 2.0 * k2e + 2.0 * k3e + k4e) / 6.0;
    }
    conserved_to_primitive_1d(G);
    boundary_1d(G);
}

int oracle_run_1d(
    int nx, int g, double x_min, double x_max, double gamma,
    const char *integrator, const char *riemann_solver, const char *slope_limiter,
    const char *bc_x_min, const char *bc_x_max,
    double cfl, double tf, long long max_steps,
    double *rho, double *u, double *p,
    double *mass, double *mom_x, double *energy,
    long long *num_steps, double *t, double *dt,
    char *errbuf, int errlen)
{
    return oracle_run_1d_ex(nx, g, x_min, x_max, gamma, integrator, riemann_solver, slope_limiter,
                            bc_x_min, bc_x_max, cfl, tf, max_steps, rho, u, p, mass, mom_x, energy,
                            num_steps, t, dt, errbuf, errlen, "cartesian_1d");
}

int oracle_run_1d_ex(
    int nx, int g, double x_min, double x_max, double gamma,
    const char *integrator, const char *riemann_solver, const char *slope_limiter,
    const char *bc_x_min, const char *bc_x_max,
    double cfl, double tf, long long max_steps,
    double *rho, double *u, double *p,
    double *mass, double *mom_x, double *energy,
    long long *num_steps, double *t, double *dt,
    char *errbuf, int errlen, const char *coord_sys)
{
    set_err(errbuf, errlen, "");
    *num_steps = 0; *t = 0.0; *dt = 0.0;
    const int is_mh = integrator && !strcmp(integrator, "muscl_hancock_1d");
    const int is_god = integrator && !strcmp(integrator, "godunov_first_order_1d");
    const int is_rc = integrator && !strcmp(integrator, "random_choice_1d");
    if (!is_mh && !is_god && !is_rc) { set_err(errbuf, errlen, "Integrator not recognized."); return VALUE_ERROR; }
    int coord = 0;
    if (coord_sys && !strcmp(coord_sys, "cartesian_1d")) coord = 1;
    else if (coord_sys && !strcmp(coord_sys, "cylindrical_1d")) coord = 2;
    else if (coord_sys && !strcmp(coord_sys, "spherical_1d")) coord = 3;
    if (!coord) { set_err(errbuf, errlen, "Coordinate system not recognized."); return VALUE_ERROR; }
    Grid1 G;
    G.nx = nx; G.g = g; G.gamma = gamma;
    G.dx = (x_max - x_min) / (nx + 2 * g);
    G.tol = 1e-6;
    G.alpha = (coord == 2) ? 1.0 : (coord == 3) ? 2.0 : 0.0;
    G.lim = parse_limiter(slope_limiter);
    if (!riemann_solver) { set_err(errbuf, errlen, "Riemann solver is not set."); return POINTER_ERROR; }
    if (!strcmp(riemann_solver, "riemann_solver_exact")) G.solver = SOLVER_EXACT;
    else if (!strcmp(riemann_solver, "riemann_solver_hllc")) G.solver = SOLVER_HLLC;
    else { set_err(errbuf, errlen, "Riemann solver not recognized."); return VALUE_ERROR; }
    if (G.lim < 0) { set_err(errbuf, errlen, "Slope limiter not recognized."); return VALUE_ERROR; }
    G.bc[0] = parse_bc(bc_x_min); G.bc[1] = parse_bc(bc_x_max);
    if (G.bc[0] < 0 || G.bc[1] < 0) { set_err(errbuf, errlen, "Boundary condition not recognized."); return VALUE_ERROR; }
    if ((G.bc[0] == BC_PERIODIC || G.bc[1] == BC_PERIODIC) && G.bc[0] != G.bc[1])
    {
        /* src/boundary.c:290-305 */
        set_err(errbuf, errlen, "Periodic boundary condition mismatch for x_min and x_max.");
        return VALUE_ERROR;
    }
    const int tot = nx + 2 * g;
    double *geo = malloc(sizeof(double) * (size_t) (3 * tot + 1));
    if (!geo) { set_err(errbuf, errlen, "Memory allocation failed."); return MEMORY_ERROR; }
    G.A = geo; G.V = geo + tot + 1; G.X = geo + 2 * tot + 1;
    geometry_1d(&G, x_min, coord);
    G.W[0] = rho; G.W[1] = u; G.W[2] = p;
    G.U[0] = mass; G.U[1] = mom_x; G.U[2] = energy;

    int status = OK;
    const double t_end = (max_steps >= 0) ? INFINITY : tf;
    while (*t < t_end && (max_steps < 0 || *num_steps < max_steps))
    {
        double step = time_step_1d(&G, (*num_steps < 10) ? cfl * 0.2 : cfl);
        if (*t + step > t_end) step = t_end - *t;
        *dt = step;
        if (step == 0.0) { set_err(errbuf, errlen, "dt is zero."); status = VALUE_ERROR; break; }
        int rc;
        if (is_rc)
        {
            rc = random_choice_step(&G, step, *num_steps);
        }
        else
        {
            rc = is_mh ? mh1d_step(&G, step) : godunov1d_step(&G, step);
            if (rc == OK)
            {
                conserved_to_primitive_1d(&G);
                boundary_1d(&G);
            }
        }
        if (rc != OK) { set_err(errbuf, errlen, solver_message(rc)); status = public_code(rc); break; }
        geometry_source_1d(&G, step);
        *t += step;
        (*num_steps)++;
    }
    free(geo);
    return status;
}

/* ------------------------------------------------- source-term exports */

/* add_geometry_source_term (src/source_term.c:45-183) on a cylindrical_1d
 * (coord 2) or spherical_1d (coord 3) grid: W and U padded, in place;
 * transmissive / reflective / periodic sides as in the 1D runs. */
int oracle_geometry_source_1d(int coord, int nx, int g, double x_min, double x_max, double gamma,
                              double dt, const char *bc_x_min, const char *bc_x_max,
                              double *rho, double *u, double *p,
                              double *mass, double *mom_x, double *energy)
{
    if (coord != 2 && coord != 3) return VALUE_ERROR;
    Grid1 G;
    G.nx = nx; G.g = g; G.gamma = gamma;
    G.dx = (x_max - x_min) / (nx + 2 * g);
    G.tol = 1e-6;
    G.alpha = (coord == 2) ? 1.0 : 2.0;
    G.lim = LIM_MINMOD;
    G.solver = SOLVER_EXACT;
    G.bc[0] = parse_bc(bc_x_min); G.bc[1] = parse_bc(bc_x_max);
    if (G.bc[0] < 0 || G.bc[1] < 0) return VALUE_ERROR;
    const int tot = nx + 2 * g;
    double *geo = malloc(sizeof(double) * (size_t) (3 * tot + 1));
    if (!geo) return MEMORY_ERROR;
    G.A = geo; G.V = geo + tot + 1; G.X = geo + 2 * tot + 1;
    geometry_1d(&G, x_min, coord);
    G.W[0] = rho; G.W[1] = u; G.W[2] = p;
    G.U[0] = mass; G.U[1] = mom_x; G.U[2] = energy;
    geometry_source_1d(&G, dt);
    free(geo);
    return OK;
}

/* add_gravity_source_term_2d (src/source_term.c:185-259) on a Cartesian 2D
 * grid with built-in sides: W and U padded, in place. */
int oracle_gravity_source_2d(int nx, int ny, int g, double x_min, double x_max, double y_min,
                             double y_max, double gamma, double gravity, double dt,
                             const char *bc_x_min, const char *bc_x_max, const char *bc_y_min,
                             const char *bc_y_max,
                             double *rho, double *u, double *v, double *p,
                             double *mass, double *mom_x, double *mom_y, double *energy)
{
    Grid G;
    memset(&G, 0, sizeof G);
    G.nx = nx; G.ny = ny; G.g = g; G.tx = nx + 2 * g;
    G.gamma = gamma;
    G.dx = (x_max - x_min) / (nx + 2 * g);
    G.dy = (y_max - y_min) / (ny + 2 * g);
    G.A_x = G.dy; G.A_y = G.dx; G.vol = G.dx * G.dy;
    G.bc[0] = parse_bc(bc_x_min); G.bc[1] = parse_bc(bc_x_max);
    G.bc[2] = parse_bc(bc_y_min); G.bc[3] = parse_bc(bc_y_max);
    for (int s = 0; s < 4; s++)
        if (G.bc[s] < 0 || G.bc[s] == BC_CUSTOM) return VALUE_ERROR;
    G.gravity = gravity;
    G.W[0] = rho; G.W[1] = u; G.W[2] = v; G.W[3] = p;
    G.U[0] = mass; G.U[1] = mom_x; G.U[2] = mom_y; G.U[3] = energy;
    gravity_2d(&G, dt);
    return OK;
}

/* ------------------------------------------------------- pointwise exports */

int oracle_hllc_2d(double gamma, double rho_L, double u_L, double v_L, double p_L,
                   double rho_R, double u_R, double v_R, double p_R, double tol, double *out4)
{
    return hllc_2d(gamma, rho_L, u_L, v_L, p_L, rho_R, u_R, v_R, p_R, tol, out4);
}

int oracle_exact_flux_1d(double gamma, double rho_L, double u_L, double p_L,
                         double rho_R, double u_R, double p_R, double tol, double speed,
                         double *out3)
{
    return public_code(exact_flux_1d(gamma, rho_L, u_L, p_L, rho_R, u_R, p_R, tol, speed, out3));
}

int oracle_hllc_1d(double gamma, double rho_L, double u_L, double p_L,
                   double rho_R, double u_R, double p_R, double tol, double *out3)
{
    return hllc_1d(gamma, rho_L, u_L, p_L, rho_R, u_R, p_R, tol, out3);
}

/* solve_exact_1d (src/riemann_solver_exact.c:332-469): the state sampled at
 * x/t = speed, as (rho, u, p). */
int oracle_exact_1d(double gamma, double rho_L, double u_L, double p_L,
                    double rho_R, double u_R, double p_R, double tol, double speed, double *out3)
{
    return public_code(exact_state_1d(gamma, rho_L, u_L, p_L, rho_R, u_R, p_R, tol, speed, out3));
}

/* Which way solve_exact_1d ends: 0 solved, 1 "Failed to bracket the root"
 * (src/riemann_solver_exact.c:702-707), 2 bisection not converged
 * (:745-754); the message for the last two is copied into errbuf. */
int oracle_exact_status(double gamma, double rho_L, double u_L, double p_L,
                        double rho_R, double u_R, double p_R, double tol, char *errbuf, int errlen)
{
    double out3[3];
    const int rc = exact_state_1d(gamma, rho_L, u_L, p_L, rho_R, u_R, p_R, tol, 0.0, out3);
    set_err(errbuf, errlen, rc == OK ? "" : solver_message(rc));
    return rc == ERR_EXACT_BRACKET ? 1 : rc == ERR_EXACT_BISECTION ? 2 : 0;
}

double oracle_guess_p(double gamma, double rho_L, double u_L, double p_L, double a_L,
                      double rho_R, double u_R, double p_R, double a_R, double tol)
{
    return guess_p(gamma, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, tol);
}

int oracle_limit_slope(int limiter_flag, double a, double b, double *out)
{
    if (limiter_flag < 1 || limiter_flag > 3) return VALUE_ERROR;
    *out = limit_slope(limiter_flag, a, b);
    return OK;
}

int oracle_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
