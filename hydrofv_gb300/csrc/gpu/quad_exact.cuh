/*
 * quad_exact.cuh -- the exact Riemann solver with four lanes per problem
 * (the 1D kernel's exact solves, and the pointwise test entry points).
 *
 * Compiled with --fmad=false like the rest of the FP64 code: the same IEEE
 * operation sequence as exact_solve_1d / exact_flux_1d of numerics.cuh.
 */
#ifndef HYDRO_GPU_QUAD_EXACT_CUH
#define HYDRO_GPU_QUAD_EXACT_CUH

#include "numerics.cuh"

namespace hydro {

/*
 * The exact solver with four lanes per Riemann problem.
 *
 * A Newton step of the star pressure needs fK and dfK of both sides
 * (src/riemann_solver_exact.c:515-560), each a pow (rarefaction side) or a
 * divide and square root (shock side).  One thread per problem evaluates the
 * four in sequence, and a warp of 32 different problems runs every branch
 * any of them takes.  Here lane q of a quad evaluates one of them (q = 0, 1:
 * fK of the left / right side; q = 2, 3: dfK) and the quad exchanges them by
 * shuffles, so a Newton step costs about one pow.  Every lane then forms
 *   f = (fK_L + fK_R) + (u_R - u_L),   f' = dfK_L + dfK_R
 * in the reference's order and runs the same control flow, so the quad's
 * lanes stay together and the result is that of exact_p_star / exact_solve_1d
 * (numerics.cuh) bit for bit.
 */
struct Quad {
    unsigned mask;   /* the quad's four lanes */
    int base;        /* its first lane */
    int q;           /* this lane's role, 0..3 */
};

__device__ __forceinline__ Quad make_quad()
{
    const int lane = threadIdx.x & 31;
    Quad Q;
    Q.base = lane & ~3;
    Q.mask = 0xfu << Q.base;
    Q.q = lane & 3;
    return Q;
}

struct Sides {
    double rho_L, p_L, a_L, rho_R, p_R, a_R, du;
    double A_L, A_R;   /* 2 / ((gamma + 1) rho) of each side, the shock branch's A */
};

/* fK (q < 2) or dfK (q >= 2) of side q & 1 at p*, the same expressions as
 * exact_fK / exact_dfK; all four values come back in v[].  With `sample`
 * set, lanes 2, 3 compute pow(p* / p_K, 1 / gamma) of side K instead (the
 * star density factor of exact_sample's rarefaction branch, used only when
 * p* <= p_K), and pre[] receives, per side, pow(p* / p_K, (gamma - 1) / 2
 * gamma) from the fK lanes (the same value exact_sample's `as` needs) and
 * that density factor. */
static __device__ void quad_fdf(const Quad &Q, const GasConst<double> &c, const Sides &S, double ps, double v[4],
                         bool sample = false, double pre[4] = nullptr)
{
    const int side = Q.q & 1;
    const bool d = Q.q >= 2;
    const double p = side ? S.p_R : S.p_L;
    const double a = side ? S.a_R : S.a_L;
    double x, r = 0.0;
    if (ps > p) {
        const double A = side ? S.A_R : S.A_L;
        const double B = p * c.gm1_gp1;
        if (d) x = sample ? 0.0 : (1.0 - dv(0.5 * (ps - p), B - ps)) * sq(dv(A, B + ps));
        else x = (ps - p) * sq(dv(A, ps + B));
    } else {
        r = pw(dv(ps, p), d ? (sample ? c.inv_g : c.neg_gp1_2g) : c.gm1_2g);
        x = d ? (sample ? r : dv(r, p * a)) : dv(2.0 * a * (r - 1.0), c.gm1);
    }
#pragma unroll
    for (int k = 0; k < 4; k++) v[k] = __shfl_sync(Q.mask, x, Q.base + k);
    if (sample) {
        pre[0] = __shfl_sync(Q.mask, r, Q.base + 0);
        pre[1] = __shfl_sync(Q.mask, r, Q.base + 1);
        pre[2] = v[2];
        pre[3] = v[3];
    }
}

__device__ __forceinline__ double quad_f(const Quad &Q, const GasConst<double> &c, const Sides &S, double ps)
{
    double v[4];
    quad_fdf(Q, c, S, ps, v);
    return v[0] + v[1] + S.du;
}

/* exact_p_star (numerics.cuh) with the function evaluations shared by the quad. */
static __device__ int quad_p_star(const Quad &Q, const GasConst<double> &c, const Sides &S, double rho_L, double u_L,
                           double p_L, double a_L, double rho_R, double u_R, double p_R, double a_R, double *out,
                           unsigned int *marks)
{
    const double pg = guess_p(c, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R);
    bool bracket = false;
    double p_hi = pg;
    /* f(p_hi) and, for the first Newton step at p0 = p_hi, f'(p_hi) */
    double v[4];
    quad_fdf(Q, c, S, p_hi, v);
    double f_hi = v[0] + v[1] + S.du;
    double p_lo = 0.0, f_lo = 0.0;
    double p0 = pg;
    for (int it = 0; it < 100; it++) {
        if (it > 0) quad_fdf(Q, c, S, p0, v);
        const double f = v[0] + v[1] + S.du;
        const double fp = v[2] + v[3];
        if (!bracket && f * f_hi < 0.0) {
            bracket = true;
            f_lo = f;
            p_lo = p0;
        }
        const double p1 = p0 - dv(f, fp);
        if (p1 < 0.0) break;
        if (ratio_below(2.0 * fabs(p1 - p0), p1 + p0, c.tol)) {
            *out = p1;
            return DEV_OK;
        }
        p0 = p1;
    }
    if (!bracket) {
        p_lo = 0.0;
        f_lo = quad_f(Q, c, S, p_lo);
        if (f_lo * f_hi >= 0.0) {
            p_hi *= 10.0;
            const double dp = dv(p_hi - p_lo, 100.0);
            for (int i = 0; i < 100; i++) {
                const double a = p_lo + (double) i * dp;
                const double b = p_lo + (double) (i + 1) * dp;
                const double fa = quad_f(Q, c, S, a);
                const double fb = quad_f(Q, c, S, b);
                if (fa * fb < 0.0) {
                    p_lo = a; f_lo = fa; p_hi = b; f_hi = fb;
                    break;
                }
            }
            if (f_lo * f_hi >= 0.0) return DEV_ERR_EXACT_BRACKET;
        }
    }
    for (int count = 1; count <= 5001; count++) {
        const double pm = 0.5 * (p_lo + p_hi);
        if (p_hi - p_lo < c.tol) {
            *out = pm;
            return DEV_OK;
        }
        const double fm = quad_f(Q, c, S, pm);
        if (fm * f_lo < 0.0) { p_hi = pm; f_hi = fm; }
        else { p_lo = pm; f_lo = fm; }
        if (Q.q == 0) note_bisection_mark(marks, count);
    }
    return DEV_ERR_EXACT_BISECTION;
}

/* exact_sample (numerics.cuh) with pow(p* / p_K, (gamma - 1) / 2 gamma) and
 * pow(p* / p_K, 1 / gamma) of each side taken from pre[] (computed in
 * parallel by the quad, the same expressions): the same branches and
 * operations. */
static __device__ void quad_sample(const GasConst<double> &c, double rho_L, double u_L, double p_L, double a_L,
                            double rho_R, double u_R, double p_R, double a_R, double us, double ps,
                            double S, const double pre[4], double o[3])
{
    if (S < us) {
        if (ps > p_L) {
            const double r = dv(ps, p_L);
            const double SL = u_L - a_L * sq(c.gp1_2g * r + c.gm1_2g);
            if (S < SL) { o[0] = rho_L; o[1] = u_L; o[2] = p_L; return; }
            const double k = c.gm1_gp1;
            o[0] = dv(rho_L * (r + k), k * r + 1.0);
            o[1] = us;
            o[2] = ps;
            return;
        }
        const double SH = u_L - a_L;
        if (S < SH) { o[0] = rho_L; o[1] = u_L; o[2] = p_L; return; }
        const double as = a_L * pre[0];
        if (S < us - as) {
            const double cm = pw((c.two_gp1 + (u_L - S) * dv(c.gm1, a_L * c.gp1)), c.two_gm1);
            o[0] = rho_L * cm;
            o[1] = c.two_gp1 * (a_L + 0.5 * u_L * c.gm1 + S);
            o[2] = p_L * pw(cm, c.gamma);
            return;
        }
        o[0] = rho_L * pre[2];
        o[1] = us;
        o[2] = ps;
        return;
    }
    if (ps > p_R) {
        const double r = dv(ps, p_R);
        const double SR = u_R + a_R * sq(dv(r * c.gp1, 2.0 * c.gamma) + c.gm1_2g);
        if (S > SR) { o[0] = rho_R; o[1] = u_R; o[2] = p_R; return; }
        const double k = c.gm1_gp1;
        o[0] = dv(rho_R * (r + k), k * r + 1.0);
        o[1] = us;
        o[2] = ps;
        return;
    }
    const double SH = u_R + a_R;
    if (S > SH) { o[0] = rho_R; o[1] = u_R; o[2] = p_R; return; }
    const double as = a_R * pre[1];
    if (S > us + as) {
        const double cm = pw((c.two_gp1 - dv((u_R - S) * c.gm1, a_R * c.gp1)), c.two_gm1);
        o[0] = rho_R * cm;
        o[1] = c.two_gp1 * (-a_R + 0.5 * u_R * c.gm1 + S);
        o[2] = p_R * pw(cm, c.gamma);
        return;
    }
    o[0] = rho_R * pre[3];
    o[1] = us;
    o[2] = ps;
}

/* exact_solve_1d (numerics.cuh) on a quad: the state sampled at x/t = S. */
static __device__ int quad_exact_solve(const Quad &Q, const GasConst<double> &c, double rho_L, double u_L, double p_L,
                                double rho_R, double u_R, double p_R, double S, double o[3],
                                unsigned int *marks = nullptr)
{
    /* lanes 0, 2 the left side, 1, 3 the right: the sound speed (exact_solve_1d's
     * a_L, a_R) and the shock coefficient A of exact_fK / exact_dfK */
    const int side = Q.q & 1;
    const double rho_s = side ? rho_R : rho_L, p_s = side ? p_R : p_L;
    const double a_s = (rho_s > 0.0) ? sound_speed(c, rho_s, p_s) : 0.0;
    const double A_s = dv(2.0, c.gp1 * rho_s);
    const double a_L = __shfl_sync(Q.mask, a_s, Q.base), a_R = __shfl_sync(Q.mask, a_s, Q.base + 1);
    const double A_L = __shfl_sync(Q.mask, A_s, Q.base), A_R = __shfl_sync(Q.mask, A_s, Q.base + 1);
    if (rho_L <= 0.0 || rho_R <= 0.0 || quot_le((a_L + a_R) * 2.0, c.gp1, u_R - u_L)) {
        double s[4];
        solve_vacuum(c, rho_L, u_L, 0.0, p_L, a_L, rho_R, u_R, 0.0, p_R, a_R, S, s);
        o[0] = s[0]; o[1] = s[1]; o[2] = s[3];
        return DEV_OK;
    }
    const Sides Sd{ rho_L, p_L, a_L, rho_R, p_R, a_R, u_R - u_L, A_L, A_R };
    double ps = 0.0;
    const int rc = quad_p_star(Q, c, Sd, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, &ps, marks);
    if (rc != DEV_OK) { o[0] = o[1] = o[2] = 0.0; return rc; }
    double v[4], pre[4];
    quad_fdf(Q, c, Sd, ps, v, true, pre);
    const double us = 0.5 * (u_L + u_R) + 0.5 * (v[1] - v[0]);
    quad_sample(c, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, us, ps, S, pre, o);
    return DEV_OK;
}

/* exact_flux_1d (numerics.cuh) on a quad, at x/t = 0. */
static __device__ int quad_exact_flux(const Quad &Q, const GasConst<double> &c, double rl, double ul, double pl,
                               double rr, double ur, double pr, double F[3], unsigned int *marks = nullptr)
{
    double s[3];
    const int rc = quad_exact_solve(Q, c, rl, ul, pl, rr, ur, pr, 0.0, s, marks);
    F[0] = s[0] * s[1];
    F[1] = s[0] * s[1] * s[1] + s[2];
    F[2] = (s[2] * c.g_gm1 + 0.5 * s[0] * s[1] * s[1]) * s[1];
    return rc;
}

}  // namespace hydro

#endif
