/*
 * riemann_solver_exact.h -- exact Riemann solver, 1D (reference:
 * src/riemann_solver_exact.h).
 */
#ifndef RIEMANN_SOLVER_EXACT_H
#define RIEMANN_SOLVER_EXACT_H

#include "hydro.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Sample the exact solution at x/t = speed. */
ErrorStatus solve_exact_1d(
    double *__restrict sol_rho,
    double *__restrict sol_u,
    double *__restrict sol_p,
    const double gamma,
    const double rho_L,
    const double u_L,
    const double p_L,
    const double rho_R,
    const double u_R,
    const double p_R,
    const double tol,
    const double speed,
    const int verbose
);

/* Godunov flux of the exact solution at x/t = speed. */
ErrorStatus solve_flux_exact_1d(
    double *__restrict flux_mass,
    double *__restrict flux_momentum,
    double *__restrict flux_energy,
    const double gamma,
    const double rho_L,
    const double u_L,
    const double p_L,
    const double rho_R,
    const double u_R,
    const double p_R,
    const double tol,
    const double speed,
    const int verbose
);

#ifdef __cplusplus
}
#endif

#endif
