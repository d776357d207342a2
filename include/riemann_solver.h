/*
 * riemann_solver.h -- Riemann-solver selection and pointwise helpers
 * (reference: src/riemann_solver.h).  The pointwise functions are host
 * builds of the same numerics the GPU kernels use.
 */
#ifndef RIEMANN_SOLVER_H
#define RIEMANN_SOLVER_H

#include "hydro.h"
#include "riemann_solver_exact.h"
#include "riemann_solver_hllc.h"

#ifdef __cplusplus
extern "C" {
#endif

#define RIEMANN_SOLVER_EXACT 1
#define RIEMANN_SOLVER_HLLC 2

ErrorStatus get_riemann_solver_flag(IntegratorParam *__restrict integrator_param);

ErrorStatus solve_flux_1d(
    IntegratorParam *__restrict integrator_param,
    Settings *__restrict settings,
    double *__restrict flux_mass,
    double *__restrict flux_momentum,
    double *__restrict flux_energy,
    const double gamma,
    const double rho_L,
    const double u_L,
    const double p_L,
    const double rho_R,
    const double u_R,
    const double p_R
);

ErrorStatus solve_flux_2d(
    IntegratorParam *__restrict integrator_param,
    Settings *__restrict settings,
    double *__restrict flux_mass,
    double *__restrict flux_momentum_x,
    double *__restrict flux_momentum_y,
    double *__restrict flux_energy,
    const double gamma,
    const double rho_L,
    const double u_L,
    const double v_L,
    const double p_L,
    const double rho_R,
    const double u_R,
    const double v_R,
    const double p_R
);

double riemann_A_L_or_R(const double gamma, const double rho_X);
double riemann_B_L_or_R(const double gamma, const double p_X);

double guess_p(
    const double gamma,
    const double rho_L,
    const double u_L,
    const double p_L,
    const double a_L,
    const double rho_R,
    const double u_R,
    const double p_R,
    const double a_R,
    const double tol
);

void solve_vacuum_1d(
    double *__restrict sol_rho,
    double *__restrict sol_u,
    double *__restrict sol_p,
    const double gamma,
    const double rho_L,
    const double u_L,
    const double p_L,
    const double a_L,
    const double rho_R,
    const double u_R,
    const double p_R,
    const double a_R,
    const double speed
);

void solve_vacuum_2d(
    double *__restrict sol_rho,
    double *__restrict sol_u,
    double *__restrict sol_v,
    double *__restrict sol_p,
    const double gamma,
    const double rho_L,
    const double u_L,
    const double v_L,
    const double p_L,
    const double a_L,
    const double rho_R,
    const double u_R,
    const double v_R,
    const double p_R,
    const double a_R,
    const double speed
);

#ifdef __cplusplus
}
#endif

#endif
