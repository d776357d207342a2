/*
 * host_numerics.cu -- host builds of the pointwise numerics exported by the
 * hydroFV API (src/riemann_solver.h, src/riemann_solver_hllc.h,
 * src/riemann_solver_exact.h, src/slope_limiter.h).
 *
 * They are compiled from the same templates (numerics.cuh) the kernels use,
 * so a program calling, e.g., solve_flux_hllc_2d gets the GPU path's
 * arithmetic.  The time loop never calls them: launch_simulation runs on the
 * GPU.  Host code here is compiled with -ffp-contract=off.
 */
#include <cstdio>

#include "hydro.h"
#include "numerics.cuh"

using namespace hydro;

namespace {

ErrorStatus hllc_error()
{
    return WRAP_RAISE_ERROR(VALUE_ERROR,
                            "Invalid wave speed for the HLLC riemann solver. Possible fix: use a smaller CFL.");
}

ErrorStatus exact_error(int rc)
{
    if (rc == DEV_ERR_EXACT_BRACKET)
        return WRAP_RAISE_ERROR(FAILURE, "Failed to bracket the root for bisection method.");
    return WRAP_RAISE_ERROR(FAILURE,
                            "Bisection method did not converge after 5001 iterations for exact riemann solver.");
}

/* The reference's verbose warnings of one exact solve, in its order: one per
 * 500 bisection iterations (src/riemann_solver_exact.c:736-744). */
void bisection_warnings(const unsigned int marks[kBisectionMarks], int verbose)
{
    if (verbose <= 0) return;
    for (int k = 0; k < kBisectionMarks; k++)
        for (unsigned int n = 0; n < marks[k]; n++) {
            char buf[128];
            snprintf(buf, sizeof buf,
                     "Bisection method did not converge after %d iterations for exact riemann solver.",
                     500 * (k + 1));
            WRAP_RAISE_WARNING(buf);
        }
}

}  // namespace

extern "C" {

double riemann_A_L_or_R(const double gamma, const double rho_X)
{
    return 2.0 / ((gamma + 1.0) * rho_X);
}

double riemann_B_L_or_R(const double gamma, const double p_X)
{
    return p_X * ((gamma - 1.0) / (gamma + 1.0));
}

double guess_p(const double gamma, const double rho_L, const double u_L, const double p_L,
               const double a_L, const double rho_R, const double u_R, const double p_R,
               const double a_R, const double tol)
{
    const GasConst<double> c = make_gas_const<double>(gamma, tol);
    return hydro::guess_p(c, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R);
}

void solve_vacuum_1d(double *__restrict sol_rho, double *__restrict sol_u, double *__restrict sol_p,
                     const double gamma, const double rho_L, const double u_L, const double p_L,
                     const double a_L, const double rho_R, const double u_R, const double p_R,
                     const double a_R, const double speed)
{
    const GasConst<double> c = make_gas_const<double>(gamma, 1e-6);
    double s[4];
    solve_vacuum(c, rho_L, u_L, 0.0, p_L, a_L, rho_R, u_R, 0.0, p_R, a_R, speed, s);
    *sol_rho = s[0];
    *sol_u = s[1];
    *sol_p = s[3];
}

void solve_vacuum_2d(double *__restrict sol_rho, double *__restrict sol_u, double *__restrict sol_v,
                     double *__restrict sol_p, const double gamma, const double rho_L,
                     const double u_L, const double v_L, const double p_L, const double a_L,
                     const double rho_R, const double u_R, const double v_R, const double p_R,
                     const double a_R, const double speed)
{
    const GasConst<double> c = make_gas_const<double>(gamma, 1e-6);
    double s[4];
    solve_vacuum(c, rho_L, u_L, v_L, p_L, a_L, rho_R, u_R, v_R, p_R, a_R, speed, s);
    *sol_rho = s[0];
    *sol_u = s[1];
    *sol_v = s[2];
    *sol_p = s[3];
}

ErrorStatus solve_flux_hllc_1d(double *__restrict flux_mass, double *__restrict flux_momentum,
                               double *__restrict flux_energy, const double gamma,
                               const double rho_L, const double u_L, const double p_L,
                               const double rho_R, const double u_R, const double p_R,
                               const double tol)
{
    const GasConst<double> c = make_gas_const<double>(gamma, tol);
    double F[3];
    if (hllc_flux_1d(c, rho_L, u_L, p_L, rho_R, u_R, p_R, F) != DEV_OK) return hllc_error();
    *flux_mass = F[0];
    *flux_momentum = F[1];
    *flux_energy = F[2];
    return make_success_error_status();
}

ErrorStatus solve_flux_hllc_2d(double *__restrict flux_mass, double *__restrict flux_momentum_x,
                               double *__restrict flux_momentum_y, double *__restrict flux_energy,
                               const double gamma, const double rho_L, const double u_L,
                               const double v_L, const double p_L, const double rho_R,
                               const double u_R, const double v_R, const double p_R,
                               const double tol)
{
    const GasConst<double> c = make_gas_const<double>(gamma, tol);
    double F[4];
    if (hllc_flux_2d(c, rho_L, u_L, v_L, p_L, rho_R, u_R, v_R, p_R, F) != DEV_OK) return hllc_error();
    *flux_mass = F[0];
    *flux_momentum_x = F[1];
    *flux_momentum_y = F[2];
    *flux_energy = F[3];
    return make_success_error_status();
}

ErrorStatus solve_exact_1d(double *sol_rho, double *sol_u, double *sol_p, const double gamma,
                           const double rho_L, const double u_L, const double p_L,
                           const double rho_R, const double u_R, const double p_R,
                           const double tol, const double speed, const int verbose)
{
    const GasConst<double> c = make_gas_const<double>(gamma, tol);
    double o[3];
    unsigned int marks[kBisectionMarks] = {};
    const int rc = exact_solve_1d(c, rho_L, u_L, p_L, rho_R, u_R, p_R, speed, o, marks);
    bisection_warnings(marks, verbose);
    if (rc != DEV_OK) return exact_error(rc);
    *sol_rho = o[0];
    *sol_u = o[1];
    *sol_p = o[2];
    return make_success_error_status();
}

ErrorStatus solve_flux_exact_1d(double *flux_mass, double *flux_momentum, double *flux_energy,
                                const double gamma, const double rho_L, const double u_L,
                                const double p_L, const double rho_R, const double u_R,
                                const double p_R, const double tol, const double speed,
                                const int verbose)
{
    const GasConst<double> c = make_gas_const<double>(gamma, tol);
    double F[3];
    unsigned int marks[kBisectionMarks] = {};
    const int rc = exact_flux_1d(c, rho_L, u_L, p_L, rho_R, u_R, p_R, speed, F, marks);
    bisection_warnings(marks, verbose);
    *flux_mass = F[0];
    *flux_momentum = F[1];
    *flux_energy = F[2];
    if (rc != DEV_OK) return exact_error(rc);
    return make_success_error_status();
}

ErrorStatus solve_flux_1d(IntegratorParam *__restrict ip, Settings *__restrict settings,
                          double *__restrict flux_mass, double *__restrict flux_momentum,
                          double *__restrict flux_energy, const double gamma, const double rho_L,
                          const double u_L, const double p_L, const double rho_R,
                          const double u_R, const double p_R)
{
    switch (ip->riemann_solver_flag_) {
    case RIEMANN_SOLVER_EXACT:
        return WRAP_TRACEBACK(solve_flux_exact_1d(flux_mass, flux_momentum, flux_energy, gamma,
                                                  rho_L, u_L, p_L, rho_R, u_R, p_R, ip->tol, 0.0,
                                                  settings ? settings->verbose : 0));
    case RIEMANN_SOLVER_HLLC:
        return WRAP_TRACEBACK(solve_flux_hllc_1d(flux_mass, flux_momentum, flux_energy, gamma,
                                                 rho_L, u_L, p_L, rho_R, u_R, p_R, ip->tol));
    default:
        return WRAP_RAISE_ERROR(VALUE_ERROR, "Riemann solver flag not recognized.");
    }
}

ErrorStatus solve_flux_2d(IntegratorParam *__restrict ip, Settings *__restrict settings,
                          double *__restrict flux_mass, double *__restrict flux_momentum_x,
                          double *__restrict flux_momentum_y, double *__restrict flux_energy,
                          const double gamma, const double rho_L, const double u_L,
                          const double v_L, const double p_L, const double rho_R,
                          const double u_R, const double v_R, const double p_R)
{
    (void) settings;
    switch (ip->riemann_solver_flag_) {
    case RIEMANN_SOLVER_EXACT:
        return WRAP_RAISE_ERROR(VALUE_ERROR, "Only HLLC Riemann solver is available for cartesian 2D.");
    case RIEMANN_SOLVER_HLLC:
        return WRAP_TRACEBACK(solve_flux_hllc_2d(flux_mass, flux_momentum_x, flux_momentum_y,
                                                 flux_energy, gamma, rho_L, u_L, v_L, p_L, rho_R,
                                                 u_R, v_R, p_R, ip->tol));
    default:
        return WRAP_RAISE_ERROR(VALUE_ERROR, "Riemann solver flag not recognized.");
    }
}

ErrorStatus limit_slope(double *__restrict limited_slope,
                        const IntegratorParam *__restrict ip, const double slope_L,
                        const double slope_R)
{
    switch (ip->slope_limiter_flag_) {
    case SLOPE_LIMITER_MINMOD:
        *limited_slope = hydro::limit_slope<LIM_MINMOD>(slope_L, slope_R);
        break;
    case SLOPE_LIMITER_VAN_LEER:
        *limited_slope = hydro::limit_slope<LIM_VAN_LEER>(slope_L, slope_R);
        break;
    case SLOPE_LIMITER_MONOTONIZED_CENTRAL:
        *limited_slope = hydro::limit_slope<LIM_MC>(slope_L, slope_R);
        break;
    default:
        return WRAP_RAISE_ERROR(VALUE_ERROR, "Limiter not recognized.");
    }
    return make_success_error_status();
}

}  // extern "C"
