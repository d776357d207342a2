/*
 * riemann_solver_hllc.h -- HLLC flux (reference: src/riemann_solver_hllc.h).
 */
#ifndef RIEMANN_SOLVER_HLLC_H
#define RIEMANN_SOLVER_HLLC_H

#include "hydro.h"

#ifdef __cplusplus
extern "C" {
#endif

ErrorStatus solve_flux_hllc_1d(
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
    const double tol
);

ErrorStatus solve_flux_hllc_2d(
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
    const double p_R,
    const double tol
);

#ifdef __cplusplus
}
#endif

#endif
