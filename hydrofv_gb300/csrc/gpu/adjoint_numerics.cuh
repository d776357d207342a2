/*
 * adjoint_numerics.cuh -- hand-written reverse mode (vector-Jacobian
 * products) of the pointwise pieces of one MUSCL-Hancock + HLLC step, and
 * the branch codes that identify which piece of a piecewise-smooth function
 * an evaluation took.
 *
 * Each *_vjp function recomputes the primal intermediates it needs with the
 * same expressions as numerics.cuh (so its branch decisions are the
 * forward pass's, bit for bit) and then applies the transposed chain rule.
 * The tie conventions at kinks are the ones Dual uses in dual.cuh, so the
 * reverse code here is the exact transpose of the tangent-linear model run
 * through numerics.cuh:
 *
 *   limiters          src/slope_limiter.c:49-91
 *   Hancock predictor src/integrator_muscl_hancock.c:682-755, :967-1041
 *   sound speed       src/utils.c:23-26
 *   HLLC 2D           src/riemann_solver_hllc.c:202-376, guesses
 *                     src/riemann_solver.c:154-224, vacuum
 *                     src/riemann_solver.c:230-733
 *   U <-> W           src/system.c:763-802, :884-905
 */
#ifndef HYDRO_GPU_ADJOINT_NUMERICS_CUH
#define HYDRO_GPU_ADJOINT_NUMERICS_CUH

#include "numerics.cuh"

/* `#pragma unroll` for the device compiler only (the host compiler builds
 * these functions too, and does not know the pragma) */
#if defined(__CUDA_ARCH__)
#define HYDRO_UNROLL _Pragma("unroll")
#else
#define HYDRO_UNROLL
#endif

namespace hydro {

/* ---------------------------------------------------------------- limiter */

/* Slope d = L(a, b) with its partial derivatives and a branch code:
 * 0  a*b <= 0 (d = 0);
 * 1  minmod a / van Leer / MC centred 0.5(a+b);
 * 2  minmod b / MC 2|a| branch;  3  MC 2|b| branch. */
template <int LIM>
HD double limit_slope_partials(double a, double b, double &da, double &db, int &code)
{
#if defined(__CUDA_ARCH__)
    /* the branch decided on the bits, as the forward limiter decides it
     * (fx::product_nonpositive; minima of positive doubles on their bit
     * patterns); operands it does not decide take the code below */
    {
        const fx::u64 ua = fx::bits(a), ub = fx::bits(b);
        const int t = fx::product_nonpositive(ua, ub);
        if (t > 0) { da = 0.0; db = 0.0; code = 0; return 0.0; }
        if (t == 0 && LIM != LIM_VAN_LEER) {
            const fx::u64 aa = ua & ~fx::SIGN, ab = ub & ~fx::SIGN;
            if (LIM == LIM_MINMOD) {
                if (aa < ab) { da = 1.0; db = 0.0; code = 1; return a; }
                da = 0.0; db = 1.0; code = 2; return b;
            }
            const bool take_b = ab < aa;
            const double two = 2.0 * fx::from_bits(take_b ? ab : aa);
            const double avg = ((ua >> 63) ? -0.5 : 0.5) * (a + b);
            const fx::u64 ut = fx::bits(two), uv = fx::bits(avg);
            if (ut < uv) {
                if (take_b) { da = 0.0; db = 2.0; code = 3; }
                else { da = 2.0; db = 0.0; code = 2; }
                return fx::from_bits(ut | (ua & fx::SIGN));
            }
            da = 0.5; db = 0.5; code = 1;
            return fx::from_bits(uv | (ua & fx::SIGN));
        }
    }
#endif
    const double d = limit_slope<LIM>(a, b);
    if (a * b <= 0.0) { da = 0.0; db = 0.0; code = 0; return d; }
    if (LIM == LIM_MINMOD) {
        if (fabs(a) < fabs(b)) { da = 1.0; db = 0.0; code = 1; }
        else { da = 0.0; db = 1.0; code = 2; }
        return d;
    }
    if (LIM == LIM_VAN_LEER) {
        const double s = a + b + 1e-10;
        da = dv(2.0 * b - d, s);
        db = dv(2.0 * a - d, s);
        code = 1;
        return d;
    }
    /* MC: fmin(avg, 2 fmin(|a|, |b|)) (signs mirrored for a < 0); ties take
     * the first argument of each fmin. */
    const double fa = fabs(a), fb = fabs(b);
    const bool take_b = fb < fa;
    const double two = 2.0 * (take_b ? fb : fa);
    const double avg = (a > 0.0) ? 0.5 * (a + b) : -0.5 * (a + b);
    if (two < avg) {
        if (take_b) { da = 0.0; db = 2.0; code = 3; }
        else { da = 2.0; db = 0.0; code = 2; }
    } else {
        da = 0.5; db = 0.5; code = 1;
    }
    return d;
}

/* ------------------------------------------------------------ sound speed */

/* a = sqrt(gamma p / rho): rho_b += -a/(2 rho) a_b, p_b += a/(2 p) a_b. */
HD void sound_speed_vjp(double rho, double p, double a, double ab, double &rhob, double &pb)
{
    if (ab == 0.0) return;
    rhob -= ab * dv(0.5 * a, rho);
    pb += ab * dv(0.5 * a, p);
}

/* ------------------------------------------------------------- predictor */

/*
 * Reverse of hancock_2d.  Inputs are those of the forward call (with
 * dtA_rho = dtA / rho); lob / hib are the adjoints of the extrapolated
 * states.  Accumulates into rhob, nb, tb, pb, ab, the slope adjoints db[4]
 * and d_rho_velb (the slope that feeds the density row).
 */
HD void hancock_2d_vjp(double dtA, double dtA_rho, double rho, double inv_rho, double n, double a,
                       const double d[4], double d_rho_vel, const double lob[4],
                       const double hib[4], double &rhob, double &nb, double &tb, double &pb,
                       double &ab, double db[4], double &d_rho_velb)
{
    const double up = 1.0 + dtA * n;
    const double um = 1.0 - dtA * n;
    const double dr = dtA * rho;
    rhob += lob[0] + hib[0];
    nb += lob[1] + hib[1];
    tb += lob[2] + hib[2];
    pb += lob[3] + hib[3];
    const double upb = -0.5 * (lob[0] * d[0] + lob[1] * d[1] + lob[2] * d[2] + lob[3] * d[3]);
    const double umb = 0.5 * (hib[0] * d[0] + hib[1] * d[1] + hib[2] * d[2] + hib[3] * d[3]);
    nb += dtA * (upb - umb);
    const double s0 = lob[0] + hib[0];
    double drb = -0.5 * s0 * d_rho_vel;
    d_rho_velb += -0.5 * dr * s0;
    const double drab = -0.5 * (lob[3] + hib[3]);          /* adjoint of dr*a*a*d[1] */
    drb += drab * a * a * d[1];
    ab += drab * 2.0 * dr * a * d[1];
    db[1] += drab * dr * a * a;
    const double s1 = lob[1] + hib[1];
    const double dtA_rhob = -0.5 * d[3] * s1;
    db[3] += -0.5 * dtA_rho * s1;
    rhob += -dtA_rhob * dtA_rho * inv_rho;                 /* d(dtA/rho)/drho */
    rhob += drb * dtA;
    db[0] += -0.5 * up * lob[0] + 0.5 * um * hib[0];
    db[1] += -0.5 * up * lob[1] + 0.5 * um * hib[1];
    db[2] += -0.5 * up * lob[2] + 0.5 * um * hib[2];
    db[3] += -0.5 * up * lob[3] + 0.5 * um * hib[3];
}

/* ------------------------------------------------------------------ HLLC */

/* Primal intermediates of one HLLC face (same expressions as
 * hllc_classify / guess_p_* / hllc_finish). */
struct HllcFwd {
    double aL, aR, ppv, pg, ps, qL, qR, SL, SR, Ss;
    int reg;       /* PREG_* */
    int region;    /* 0 left, 1 left star, 2 right star, 3 right; -1 vacuum */
};

HD int hllc_fwd(const GasConst<double> &c, double rl, double ul, double pl, double rr, double ur,
                double pr, HllcFwd &s)
{
    s.reg = hllc_classify(c, rl, ul, pl, rr, ur, pr, s.aL, s.aR, s.ppv);
    s.region = -1;
    s.pg = s.ps = s.qL = s.qR = s.SL = s.SR = s.Ss = 0.0;
    if (s.reg == PREG_VACUUM) return DEV_OK;
    s.pg = s.ppv;
    if (s.reg == PREG_TRRS) s.pg = guess_p_trrs(c, ul, pl, s.aL, ur, pr, s.aR);
    else if (s.reg == PREG_TSRS) s.pg = guess_p_tsrs(c, rl, ul, pl, rr, ur, pr, s.ppv);
    s.ps = lt(s.pg, c.tol) ? c.tol : s.pg;
    s.qL = hllc_q(c, pl, s.ps);
    s.qR = hllc_q(c, pr, s.ps);
    s.SL = ul - s.aL * s.qL;
    s.SR = ur + s.aR * s.qR;
    s.Ss = dv(pr - pl + rl * ul * (s.SL - ul) - rr * ur * (s.SR - ur),
              rl * (s.SL - ul) - rr * (s.SR - ur));
    if (le(0.0, s.SL)) s.region = 0;
    else if (le(s.SL, 0.0) && le(0.0, s.Ss)) s.region = 1;
    else if (le(s.Ss, 0.0) && le(0.0, s.SR)) s.region = 2;
    else if (le(s.SR, 0.0)) s.region = 3;
    else return DEV_ERR_HLLC_WAVE_SPEED;
    return DEV_OK;
}

/* The intermediates of a non-vacuum face from the tape: sound speeds,
 * unfloored guess, regime and the finish's q_L, q_R and S* as the forward
 * pass computed them (the same values hllc_fwd_from_guess recomputes). */
HD int hllc_fwd_from_tape(const GasConst<double> &c, double rl, double ul, double pl, double rr, double ur,
                          double pr, double aL, double aR, double pg, int reg, double qL, double qR, double Ss,
                          HllcFwd &s)
{
    s.aL = aL;
    s.aR = aR;
    s.reg = reg;
    s.region = -1;
    s.ppv = 0.5 * (pl + pr) - 0.125 * (ur - ul) * (rl + rr) * (aL + aR);
    s.pg = pg;
    s.ps = s.qL = s.qR = s.SL = s.SR = s.Ss = 0.0;
    if (reg == PREG_VACUUM) return DEV_OK;
    s.ps = lt(s.pg, c.tol) ? c.tol : s.pg;
    s.qL = qL;
    s.qR = qR;
    s.SL = ul - s.aL * s.qL;
    s.SR = ur + s.aR * s.qR;
    s.Ss = Ss;
    if (le(0.0, s.SL)) s.region = 0;
    else if (le(s.SL, 0.0) && le(0.0, s.Ss)) s.region = 1;
    else if (le(s.Ss, 0.0) && le(0.0, s.SR)) s.region = 2;
    else if (le(s.SR, 0.0)) s.region = 3;
    else return DEV_ERR_HLLC_WAVE_SPEED;
    return DEV_OK;
}

/* Which sampler branch the vacuum flux takes (S = 0):
 * 0 zero state, 1 right-vacuum sampler on the left state, 2 left-vacuum
 * sampler on the right state; *sub: 0 data state, 1 fan, 2 vacuum. */
HD int vacuum_case(const GasConst<double> &c, double rl, double ul, double al, double rr,
                   double ur, double ar, int &sub)
{
    int which;
    if (rl <= 0.0 && rr <= 0.0) { sub = 0; return 0; }
    if (rl <= 0.0) which = 1;
    else if (rr <= 0.0) which = 2;
    else if (0.0 <= 2.0 * al / c.gm1) which = 1;
    else if (2.0 * ar / c.gm1 <= 0.0) which = 2;
    else { sub = 0; return 0; }
    if (which == 1) {
        if (0.0 <= ul - al) sub = 0;
        else sub = (0.0 < ul + 2.0 * al / c.gm1) ? 1 : 2;
    } else {
        if (0.0 >= ur + ar) sub = 0;
        else sub = (0.0 > ur - 2.0 * ar / c.gm1) ? 1 : 2;
    }
    return which;
}

/* Branch code of one face: regime, guess floor, shock/rarefaction side of
 * each wave speed, region; for vacuum faces the sampler branch. */
HD int hllc_code(const GasConst<double> &c, const HllcFwd &s, double rl, double ul, double pl,
                 double rr, double ur, double pr)
{
    if (s.reg == PREG_VACUUM) {
        int sub;
        const int which = vacuum_case(c, rl, ul, s.aL, rr, ur, s.aR, sub);
        return 0x100 | (which << 2) | sub;
    }
    return s.reg | ((s.pg < c.tol) << 2) | ((s.ps > pl) << 3) | ((s.ps > pr) << 4)
         | ((s.region & 3) << 5);
}

/* Reverse of a vacuum-sampler fan: o = (rho t, (+-a + h u)*2/(g+1), v, p t^gamma),
 * t = (2/(g+1) +- (u/((g+1) a)) (g-1))^(2/(g-1)) at S = 0. */
HD void vacuum_fan_vjp(const GasConst<double> &c, bool right, double rho, double u, double p,
                       double a, const double ob[4], double &rhob, double &ub, double &vb,
                       double &pb, double &ab)
{
    const double k = (u - 0.0) * c.gm1 / (c.gp1 * a);
    const double t0 = right ? (c.two_gp1 + k) : (c.two_gp1 - k);
    const double t = pw(t0, c.two_gm1);
    const double tg = pw(t, c.gamma);
    rhob += ob[0] * t;
    const double tb = ob[0] * rho + ob[3] * p * c.gamma * tg / t;
    pb += ob[3] * tg;
    ab += (right ? 1.0 : -1.0) * ob[1] * 2.0 / c.gp1;
    ub += ob[1] * c.half_gm1 * 2.0 / c.gp1;
    vb += ob[2];
    const double t0b = tb * c.two_gm1 * t / t0;
    const double kb = right ? t0b : -t0b;
    ub += kb * c.gm1 / (c.gp1 * a);
    ab += -kb * k / a;
}

/* The remaining intermediates of a face from its sound speeds, unfloored
 * guess and regime (what the tape keeps): the same expressions as
 * hllc_classify / hllc_finish. */
HD int hllc_fwd_from_guess(const GasConst<double> &c, double rl, double ul, double pl, double rr, double ur,
                           double pr, double aL, double aR, double pg, int reg, HllcFwd &s)
{
    s.aL = aL;
    s.aR = aR;
    s.reg = reg;
    s.region = -1;
    s.ppv = 0.5 * (pl + pr) - 0.125 * (ur - ul) * (rl + rr) * (aL + aR);
    s.pg = pg;
    s.ps = s.qL = s.qR = s.SL = s.SR = s.Ss = 0.0;
    if (reg == PREG_VACUUM) return DEV_OK;
    s.ps = lt(s.pg, c.tol) ? c.tol : s.pg;
    s.qL = hllc_q(c, pl, s.ps);
    s.qR = hllc_q(c, pr, s.ps);
    s.SL = ul - s.aL * s.qL;
    s.SR = ur + s.aR * s.qR;
    s.Ss = dv(pr - pl + rl * ul * (s.SL - ul) - rr * ur * (s.SR - ur),
              rl * (s.SL - ul) - rr * (s.SR - ur));
    if (le(0.0, s.SL)) s.region = 0;
    else if (le(s.SL, 0.0) && le(0.0, s.Ss)) s.region = 1;
    else if (le(s.Ss, 0.0) && le(0.0, s.SR)) s.region = 2;
    else if (le(s.SR, 0.0)) s.region = 3;
    else return DEV_ERR_HLLC_WAVE_SPEED;
    return DEV_OK;
}

/* Reverse of the vacuum / vacuum-generation flux (kept out of line: rare,
 * and its pow-heavy samplers would otherwise raise the register count of
 * every face). */
#ifdef __CUDACC__
static __host__ __device__ __noinline__
#else
static
#endif
void hllc_vacuum_vjp(const GasConst<double> &c, const double L[4], const double Rs[4], double aL, double aR,
                     const double Fb[4], double Lb[4], double Rb[4])
{
    const double rl = L[0], ul = L[1], vl = L[2], pl = L[3];
    const double rr = Rs[0], ur = Rs[1], vr = Rs[2], pr = Rs[3];
    double rLb = 0, uLb = 0, vLb = 0, pLb = 0, rRb = 0, uRb = 0, vRb = 0, pRb = 0, aLb = 0, aRb = 0;
    int sub;
    const int which = vacuum_case(c, rl, ul, aL, rr, ur, aR, sub);
    double o[4];
    solve_vacuum(c, rl, ul, vl, pl, aL, rr, ur, vr, pr, aR, 0.0, o);
    const double E = o[0] * (0.5 * (o[1] * o[1] + o[2] * o[2]) + o[3] / (o[0] * c.gm1));
    const double Eb = Fb[3] * o[1];
    double ob[4];
    ob[0] = Fb[0] * o[1] + Fb[1] * o[1] * o[1] + Fb[2] * o[1] * o[2] + Eb * 0.5 * (o[1] * o[1] + o[2] * o[2]);
    ob[1] = Fb[0] * o[0] + Fb[1] * 2.0 * o[0] * o[1] + Fb[2] * o[0] * o[2] + Fb[3] * (E + o[3])
          + Eb * o[0] * o[1];
    ob[2] = Fb[2] * o[0] * o[1] + Eb * o[0] * o[2];
    ob[3] = Fb[1] + Fb[3] * o[1] + Eb / c.gm1;
    if (which == 1) {
        if (sub == 0) { rLb += ob[0]; uLb += ob[1]; vLb += ob[2]; pLb += ob[3]; }
        else if (sub == 1) vacuum_fan_vjp(c, true, rl, ul, pl, aL, ob, rLb, uLb, vLb, pLb, aLb);
    } else if (which == 2) {
        if (sub == 0) { rRb += ob[0]; uRb += ob[1]; vRb += ob[2]; pRb += ob[3]; }
        else if (sub == 1) vacuum_fan_vjp(c, false, rr, ur, pr, aR, ob, rRb, uRb, vRb, pRb, aRb);
    }
    if (rl > 0.0) sound_speed_vjp(rl, pl, aL, aLb, rLb, pLb);
    if (rr > 0.0) sound_speed_vjp(rr, pr, aR, aRb, rRb, pRb);
    Lb[0] = rLb; Lb[1] = uLb; Lb[2] = vLb; Lb[3] = pLb;
    Rb[0] = rRb; Rb[1] = uRb; Rb[2] = vRb; Rb[3] = pRb;
}

/*
 * Reverse of hllc_flux_2d given the face's forward intermediates s.  L, Rs
 * = (rho, u_normal, u_tangential, p) of the left / right face states, Fb =
 * adjoint of the flux (mass, normal momentum, tangential momentum, energy).
 * With have_z the guess factors (z0, z1) are taken as given (from the tape)
 * instead of recomputed.  Writes Lb, Rb.
 */
HD void hllc_vjp_core(const GasConst<double> &c, const double L[4], const double Rs[4], const HllcFwd &s,
                      bool have_z, double z0, double z1, const double Fb[4], double Lb[4], double Rb[4])
{
    if (s.reg == PREG_VACUUM) {
        hllc_vacuum_vjp(c, L, Rs, s.aL, s.aR, Fb, Lb, Rb);
        return;
    }
    /* Only the forward intermediates in s decide branches; the reverse below
     * is derivatives only, so a quotient that appears several times is
     * formed once as a reciprocal (a derivative, not a bit-parity value). */
    const double rl = L[0], ul = L[1], vl = L[2], pl = L[3];
    const double rr = Rs[0], ur = Rs[1], vr = Rs[2], pr = Rs[3];
    const double inv_rl = rv(rl), inv_rr = rv(rr), inv_pl = rv(pl), inv_pr = rv(pr);
    const double inv_gm1 = c.inv_gm1;
    double rLb = 0, uLb = 0, vLb = 0, pLb = 0, rRb = 0, uRb = 0, vRb = 0, pRb = 0;
    double aLb = 0, aRb = 0;
    /* ---- region flux of the selected side K ---- */
    const bool left = s.region <= 1;
    const double rho = left ? rl : rr, u = left ? ul : ur, v = left ? vl : vr, p = left ? pl : pr;
    const double inv_rho = left ? inv_rl : inv_rr;
    const double E = 0.5 * rho * (u * u + v * v) + p * inv_gm1;
    const double fm = rho * u;
    double rhob = 0, ub = 0, vb = 0, pb = 0;
    double fmb = Fb[0] + Fb[1] * u + Fb[2] * v;
    ub += Fb[1] * fm + Fb[3] * (E + p);
    vb += Fb[2] * fm;
    pb += Fb[1] + Fb[3] * u;
    double Eb = Fb[3] * u;
    double SLb = 0, SRb = 0, Ssb = 0;
    if (s.region == 1 || s.region == 2) {
        const double S = left ? s.SL : s.SR;
        const double Ss = s.Ss;
        const double Smu = S - u, SmS = S - Ss;
        const double inv_SmS = rv(SmS);
        const double D = rho * Smu;
        const double inv_D = rv(D);
        const double rs = D * inv_SmS;
        const double pD = p * inv_D;
        const double Z = Ss + pD;
        const double Er = E * inv_rho;
        const double Y = Er + (Ss - u) * Z;
        const double es = rs * Y;
        double Sb = Fb[0] * (rs - rho) + Fb[1] * (rs * Ss - rho * u) + Fb[2] * (rs * v - rho * v)
                  + Fb[3] * (es - E);
        double rsb = S * (Fb[0] + Fb[1] * Ss + Fb[2] * v);
        Ssb += Fb[1] * S * rs;
        const double esb = Fb[3] * S;
        Eb += -Fb[3] * S;
        rhob += -S * (Fb[0] + Fb[1] * u + Fb[2] * v);
        ub += -Fb[1] * S * rho;
        vb += Fb[2] * S * (rs - rho);
        rsb += esb * Y;
        const double Yb = esb * rs;
        Eb += Yb * inv_rho;
        rhob += -Yb * Er * inv_rho;
        Ssb += Yb * Z;
        ub += -Yb * Z;
        const double Zb = Yb * (Ss - u);
        Ssb += Zb;
        pb += Zb * inv_D;
        const double Db = -Zb * pD * inv_D;
        /* rs = N / M, N = D = rho (S - u), M = S - Ss */
        const double Nb = rsb * inv_SmS + Db;
        const double Mb = -rsb * rs * inv_SmS;
        rhob += Nb * Smu;
        Sb += Nb * rho;
        ub += -Nb * rho;
        Sb += Mb;
        Ssb += -Mb;
        if (left) SLb += Sb;
        else SRb += Sb;
    }
    rhob += fmb * u;
    ub += fmb * rho;
    rhob += Eb * 0.5 * (u * u + v * v);
    ub += Eb * rho * u;
    vb += Eb * rho * v;
    pb += Eb * inv_gm1;
    if (left) { rLb += rhob; uLb += ub; vLb += vb; pLb += pb; }
    else { rRb += rhob; uRb += ub; vRb += vb; pRb += pb; }

    /* ---- S* ---- */
    if (!eq_zero(Ssb)) {
        const double dL = s.SL - ul, dR = s.SR - ur;
        const double Dd = rl * dL - rr * dR;
        const double Nnb = dv(Ssb, Dd);
        const double Ddb = -Nnb * s.Ss;
        pRb += Nnb;
        pLb -= Nnb;
        rLb += Nnb * ul * dL + Ddb * dL;
        uLb += Nnb * rl * (dL - ul) - Ddb * rl;
        SLb += (Nnb * ul + Ddb) * rl;
        rRb -= Nnb * ur * dR + Ddb * dR;
        uRb -= Nnb * rr * (dR - ur) - Ddb * rr;
        SRb -= (Nnb * ur + Ddb) * rr;
    }

    /* ---- wave speeds ---- */
    uLb += SLb;
    aLb -= SLb * s.qL;
    const double qLb = -SLb * s.aL;
    uRb += SRb;
    aRb += SRb * s.qR;
    const double qRb = SRb * s.aR;
    double psb = 0.0;
    if (lt(pl, s.ps)) {
        const double t = dv(qLb * (0.5 * c.q_coef), s.qL) * inv_pl;
        psb += t;
        pLb -= t * s.ps * inv_pl;
    }
    if (lt(pr, s.ps)) {
        const double t = dv(qRb * (0.5 * c.q_coef), s.qR) * inv_pr;
        psb += t;
        pRb -= t * s.ps * inv_pr;
    }
    const double pgb = lt(s.pg, c.tol) ? 0.0 : psb;

    /* ---- star-pressure guess ---- */
    double ppvb = 0.0;
    if (s.reg == PREG_PVRS) {
        ppvb += pgb;
    } else if (s.reg == PREG_TRRS) {
        const double zL = have_z ? z0 : pw(pl, c.half_gm1_g);
        const double zR = have_z ? z1 : pw(pr, c.half_gm1_g);
        const double izL = rv(zL), izR = rv(zR);
        const double num = s.aL + s.aR - c.half_gm1 * (ur - ul);
        const double den = s.aL * izL + s.aR * izR;
        /* pg = (num / den)^(1/hg): d pg = (pg / hg) (d num / num - d den / den) */
        const double k = pgb * c.g_half_gm1 * s.pg;
        const double numb = dv(k, num);
        const double denb = dv(-k, den);
        aLb += numb + denb * izL;
        aRb += numb + denb * izR;
        uRb -= numb * c.half_gm1;
        uLb += numb * c.half_gm1;
        /* den = aL zL^-1 + aR zR^-1, zK = pK^hg: d den / d pK = -aK hg zK^-1 / pK */
        pLb -= denb * s.aL * izL * c.half_gm1_g * inv_pl;
        pRb -= denb * s.aR * izR * c.half_gm1_g * inv_pr;
    } else {
        const double BL = s.ppv + pl * c.gm1_gp1, BR = s.ppv + pr * c.gm1_gp1;
        const double gL = have_z ? z0 : sq(dv(dv(2.0, c.gp1 * rl), BL));
        const double gR = have_z ? z1 : sq(dv(dv(2.0, c.gp1 * rr), BR));
        const double Nnb = dv(pgb, gL + gR);
        const double Ddb = -Nnb * s.pg;
        const double gLb = Nnb * pl + Ddb, gRb = Nnb * pr + Ddb;
        pLb += Nnb * gL;
        pRb += Nnb * gR;
        uRb -= Nnb;
        uLb += Nnb;
        const double hL = 0.5 * gLb * gL, hR = 0.5 * gRb * gR;
        rLb -= hL * inv_rl;
        rRb -= hR * inv_rr;
        const double BLb = dv(-hL, BL), BRb = dv(-hR, BR);
        ppvb += BLb + BRb;
        pLb += BLb * c.gm1_gp1;
        pRb += BRb * c.gm1_gp1;
    }
    if (!eq_zero(ppvb)) {
        pLb += 0.5 * ppvb;
        pRb += 0.5 * ppvb;
        const double du = ur - ul, sr = rl + rr, sa = s.aL + s.aR;
        const double w = -0.125 * ppvb;
        const double dub = w * sr * sa;
        const double srb = w * du * sa;
        const double sab = w * du * sr;
        uRb += dub;
        uLb -= dub;
        rLb += srb;
        rRb += srb;
        aLb += sab;
        aRb += sab;
    }
    /* a = sqrt(gamma p / rho): da = a/2 (dp/p - drho/rho) */
    const double hL = 0.5 * aLb * s.aL, hR = 0.5 * aRb * s.aR;
    rLb -= hL * inv_rl;
    pLb += hL * inv_pl;
    rRb -= hR * inv_rr;
    pRb += hR * inv_pr;
    Lb[0] = rLb; Lb[1] = uLb; Lb[2] = vLb; Lb[3] = pLb;
    Rb[0] = rRb; Rb[1] = uRb; Rb[2] = vRb; Rb[3] = pRb;
}

/* Reverse of hllc_flux_2d from the face states alone (forward intermediates
 * recomputed).  Returns DEV_OK or DEV_ERR_HLLC_WAVE_SPEED; *code (may be
 * NULL) receives the face's branch code. */
HD int hllc_vjp(const GasConst<double> &c, const double L[4], const double Rs[4], const double Fb[4],
                double Lb[4], double Rb[4], int *code)
{
    HllcFwd s;
    const int rc = hllc_fwd(c, L[0], L[1], L[3], Rs[0], Rs[1], Rs[3], s);
    if (code) *code = hllc_code(c, s, L[0], L[1], L[3], Rs[0], Rs[1], Rs[3]);
    if (rc != DEV_OK) {
        for (int q = 0; q < 4; q++) { Lb[q] = 0.0; Rb[q] = 0.0; }
        return rc;
    }
    hllc_vjp_core(c, L, Rs, s, false, 0.0, 0.0, Fb, Lb, Rb);
    return DEV_OK;
}

/* ------------------------------------------------------- cell recon */

/*
 * MUSCL-Hancock reconstruction of one cell along one direction, as the step
 * kernel does it: wm, w0, wp = (rho, vx, vy, p) of the cells below, at and
 * above along the sweep, a0 = sound speed of w0.  dir 0 (x): states in
 * (rho, vx, vy, p) order; dir 1 (y): (rho, vy, vx, p), and the density row
 * takes the x-velocity slope (src/integrator_muscl_hancock.c:988-993).
 * lo / hi = states at the cell's low / high face.
 */
template <int LIM, class R>
HD void recon_cell(int dir, R dtA, const R wm[4], const R w0[4], const R wp[4], R a0, R lo[4], R hi[4])
{
    R d[4];
    if (dir == 0) {
HYDRO_UNROLL
        for (int q = 0; q < 4; q++) d[q] = limit_slope<LIM>(w0[q] - wm[q], wp[q] - w0[q]);
        hancock_2d(dtA, dv(dtA, w0[0]), w0[0], w0[1], w0[2], w0[3], a0, d, d[1], lo, hi);
    } else {
        d[0] = limit_slope<LIM>(w0[0] - wm[0], wp[0] - w0[0]);
        const R dvx = limit_slope<LIM>(w0[1] - wm[1], wp[1] - w0[1]);
        d[1] = limit_slope<LIM>(w0[2] - wm[2], wp[2] - w0[2]);
        d[2] = dvx;
        d[3] = limit_slope<LIM>(w0[3] - wm[3], wp[3] - w0[3]);
        hancock_2d(dtA, dv(dtA, w0[0]), w0[0], w0[2], w0[1], w0[3], a0, d, dvx, lo, hi);
    }
}

/* Branch code of recon_cell: 2 bits per limiter call. */
template <int LIM>
HD int recon_code(const double wm[4], const double w0[4], const double wp[4])
{
    int code = 0;
HYDRO_UNROLL
    for (int q = 0; q < 4; q++) {
        double da, db;
        int c;
        limit_slope_partials<LIM>(w0[q] - wm[q], wp[q] - w0[q], da, db, c);
        code |= c << (2 * q);
    }
    return code;
}

/*
 * Reverse of recon_cell (a0 = sound speed of w0, folded back into w0;
 * inv_rho, inv_p = 1/rho, 1/p of w0).
 * Given lob / hib (sweep order), writes in storage order (rho, vx, vy, p):
 *   own  adjoint reaching w0 itself, including its share of the slopes;
 *   A    adjoint of the backward differences w0 - wm (wm receives -A);
 *   B    adjoint of the forward differences wp - w0 (wp receives +B).
 */
template <int LIM>
HD void recon_cell_vjp(int dir, double dtA, const double wm[4], const double w0[4], const double wp[4],
                       double a0, double inv_rho, double inv_p, const double lob[4], const double hib[4],
                       double own[4], double A[4], double B[4])
{
    double pa[4], pb[4], d[4];
    int code;
HYDRO_UNROLL
    for (int q = 0; q < 4; q++) d[q] = limit_slope_partials<LIM>(w0[q] - wm[q], wp[q] - w0[q], pa[q], pb[q], code);
    const int in_ = (dir == 0) ? 1 : 2;    /* storage index of the normal velocity */
    const int it_ = (dir == 0) ? 2 : 1;    /* storage index of the tangential velocity */
    double ds[4];                          /* slopes in sweep order */
    ds[0] = d[0];
    ds[1] = d[in_];
    ds[2] = d[it_];
    ds[3] = d[3];
    double rhob = 0, nb = 0, tb = 0, pbb = 0, ab = 0, dvxb = 0;
    double dsb[4] = { 0, 0, 0, 0 };
    hancock_2d_vjp(dtA, dtA * inv_rho, w0[0], inv_rho, w0[in_], a0, ds, d[1], lob, hib, rhob, nb, tb, pbb,
                   ab, dsb, dvxb);
    double db[4];                          /* slope adjoints, storage order */
    db[0] = dsb[0];
    db[in_] = dsb[1];
    db[it_] = dsb[2];
    db[3] = dsb[3];
    db[1] += dvxb;
    own[0] = rhob;
    own[in_] = nb;
    own[it_] = tb;
    own[3] = pbb;
    /* a = sqrt(gamma p / rho): da = a/2 (dp/p - drho/rho) */
    const double h = 0.5 * ab * a0;
    own[0] -= h * inv_rho;
    own[3] += h * inv_p;
HYDRO_UNROLL
    for (int q = 0; q < 4; q++) {
        A[q] = db[q] * pa[q];
        B[q] = db[q] * pb[q];
        own[q] += A[q] - B[q];
    }
}

/* ------------------------------------------------ forced-branch forward */

/*
 * The forward pieces with every branch decision given (a code recorded from
 * another evaluation) instead of taken: the map whose derivative the
 * adjoint computes, as a function that stays on one smooth piece.  With the
 * evaluation's own codes the values are bit for bit those of numerics.cuh.
 */
template <int LIM>
HD double limit_slope_forced(double a, double b, int code)
{
    if (code == 0) return 0.0;
    if (LIM == LIM_MINMOD) return (code == 1) ? a : b;
    if (LIM == LIM_VAN_LEER) return dv(2.0 * a * b, a + b + 1e-10);
    if (code == 1) return (a > 0.0) ? 0.5 * (a + b) : -(-0.5 * (a + b));
    return 2.0 * ((code == 2) ? a : b);
}

template <int LIM>
HD void recon_cell_forced(int dir, double dtA, const double wm[4], const double w0[4], const double wp[4],
                          double a0, int code, double lo[4], double hi[4])
{
    double d[4];
HYDRO_UNROLL
    for (int q = 0; q < 4; q++) d[q] = limit_slope_forced<LIM>(w0[q] - wm[q], wp[q] - w0[q], (code >> (2 * q)) & 3);
    if (dir == 0) {
        hancock_2d(dtA, dv(dtA, w0[0]), w0[0], w0[1], w0[2], w0[3], a0, d, d[1], lo, hi);
    } else {
        const double ds[4] = { d[0], d[2], d[1], d[3] };
        hancock_2d(dtA, dv(dtA, w0[0]), w0[0], w0[2], w0[1], w0[3], a0, ds, d[1], lo, hi);
    }
}

/* Vacuum flux (S = 0) with the sampler branch given. */
HD void vacuum_flux_forced(const GasConst<double> &c, double rl, double ul, double vl, double pl, double al,
                           double rr, double ur, double vr, double pr, double ar, int which, int sub,
                           double F[4])
{
    double s[4] = { 0.0, 0.0, 0.0, 0.0 };
    if (which != 0 && sub != 2) {
        const bool right = (which == 1);
        const double rho = right ? rl : rr, u = right ? ul : ur, v = right ? vl : vr, p = right ? pl : pr;
        const double a = right ? al : ar;
        if (sub == 0) {
            s[0] = rho; s[1] = u; s[2] = v; s[3] = p;
        } else if (right) {
            double tmp = c.two_gp1 + (u - 0.0) * c.gm1 / (c.gp1 * a);
            tmp = pw(tmp, c.two_gm1);
            s[0] = rho * tmp;
            s[1] = (a + c.half_gm1 * u + 0.0) * 2.0 / c.gp1;
            s[2] = v;
            s[3] = p * pw(tmp, c.gamma);
        } else {
            double tmp = c.two_gp1 - (u - 0.0) * c.gm1 / (c.gp1 * a);
            tmp = pw(tmp, c.two_gm1);
            s[0] = rho * tmp;
            s[1] = (-a + c.half_gm1 * u + 0.0) * 2.0 / c.gp1;
            s[2] = v;
            s[3] = p * pw(tmp, c.gamma);
        }
    }
    const double E = s[0] * (0.5 * (s[1] * s[1] + s[2] * s[2]) + s[3] / (s[0] * c.gm1));
    F[0] = s[0] * s[1];
    F[1] = s[0] * s[1] * s[1] + s[3];
    F[2] = s[0] * s[1] * s[2];
    F[3] = s[1] * (E + s[3]);
}

/* HLLC 2D flux with the branch code of hllc_code given. */
HD void hllc_flux_2d_forced(const GasConst<double> &c, double rl, double ul, double vl, double pl, double rr,
                            double ur, double vr, double pr, int code, double F[4])
{
    const double aL = (rl > 0.0) ? sound_speed(c, rl, pl) : 0.0;
    const double aR = (rr > 0.0) ? sound_speed(c, rr, pr) : 0.0;
    if (code & 0x100) {
        vacuum_flux_forced(c, rl, ul, vl, pl, aL, rr, ur, vr, pr, aR, (code >> 2) & 3, code & 3, F);
        return;
    }
    const int reg = code & 3;
    const double ppv = 0.5 * (pl + pr) - 0.125 * (ur - ul) * (rl + rr) * (aL + aR);
    double pg = ppv;
    if (reg == PREG_TRRS) pg = guess_p_trrs(c, ul, pl, aL, ur, pr, aR);
    else if (reg == PREG_TSRS) pg = guess_p_tsrs(c, rl, ul, pl, rr, ur, pr, ppv);
    const double ps = (code & 4) ? c.tol : pg;
    const double qL = (code & 8) ? sq(1.0 + c.q_coef * (dv(ps, pl) - 1.0)) : 1.0;
    const double qR = (code & 16) ? sq(1.0 + c.q_coef * (dv(ps, pr) - 1.0)) : 1.0;
    const double SL = ul - aL * qL;
    const double SR = ur + aR * qR;
    const double Ss = dv(pr - pl + rl * ul * (SL - ul) - rr * ur * (SR - ur), rl * (SL - ul) - rr * (SR - ur));
    const int region = (code >> 5) & 3;
    const bool left = region <= 1;
    const double rho = left ? rl : rr, u = left ? ul : ur, v = left ? vl : vr, p = left ? pl : pr;
    const double E = rho * (0.5 * (u * u + v * v) + dv(p, rho * c.gm1));
    const double fm = rho * u;
    F[0] = fm;
    F[1] = fm * u + p;
    F[2] = fm * v;
    F[3] = u * (E + p);
    if (region == 1 || region == 2) {
        const double S = left ? SL : SR;
        const double rs = dv(rho * (S - u), S - Ss);
        const double es = rs * (dv(E, rho) + (Ss - u) * (Ss + dv(p, rho * (S - u))));
        F[0] = fm + S * (rs - rho);
        F[1] = F[1] + S * (rs * Ss - rho * u);
        F[2] = F[2] + S * (rs * v - rho * v);
        F[3] = F[3] + S * (es - E);
    }
}

/* ------------------------------------------------------------ conversion */

/* Reverse of cons_to_prim_2d: wb (rho, u, v, p) -> Ub (m, mx, my, E), accumulated. */
HD void cons_to_prim_2d_vjp(const GasConst<double> &c, double vol, double m, double mx, double my,
                            const double wb[4], double Ub[4])
{
    const double w1 = dv(mx, m), w2 = dv(my, m);
    const double K = w1 * w1 + w2 * w2;
    const double Pb = dv(wb[3] * c.gm1, vol);
    Ub[3] += Pb;
    double mb = -0.5 * K * Pb + dv(wb[0], vol);
    const double w1b = wb[1] - m * w1 * Pb;
    const double w2b = wb[2] - m * w2 * Pb;
    Ub[1] += dv(w1b, m);
    Ub[2] += dv(w2b, m);
    mb += dv(-(w1b * w1 + w2b * w2), m);
    Ub[0] += mb;
}

/* Reverse of the 2D primitive -> conserved conversion (src/system.c:884-905):
 * Ub -> wb, accumulated. */
HD void prim_to_cons_2d_vjp(const GasConst<double> &c, double vol, const double w[4],
                            const double Ub[4], double wb[4])
{
    const double rho = w[0], u = w[1], v = w[2];
    const double m = rho * vol;
    const double mb = Ub[0] + Ub[1] * u + Ub[2] * v;
    wb[0] += mb * vol + Ub[3] * vol * 0.5 * (u * u + v * v);
    wb[1] += Ub[1] * m + Ub[3] * vol * rho * u;
    wb[2] += Ub[2] * m + Ub[3] * vol * rho * v;
    wb[3] += dv(Ub[3] * vol, c.gm1);
}

/* The same conversion forward, templated for the tangent-linear state. */
template <class R>
HD void prim_to_cons_2d(const GasConst<R> &c, R vol, const R w[4], R U[4])
{
    const R m = w[0] * vol;
    U[0] = m;
    U[1] = m * w[1];
    U[2] = m * w[2];
    U[3] = vol * (R(0.5) * w[0] * (w[1] * w[1] + w[2] * w[2]) + dv(w[3], c.gm1));
}

}  // namespace hydro

#endif
