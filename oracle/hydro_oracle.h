/*
 * hydro_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the hydroFV finite-volume step, used as the parity
 * checker for the GPU library and as the "port" CPU baseline.  It is never
 * linked into, loaded by, or called from the product library.
 *
 * The flat entry points take the same arguments as oracle/ref_harness.c so the
 * tests can run the restatement and the unmodified reference side by side.
 * Return codes follow the reference's error codes (src/error.h:15-22).
 */
#ifndef HYDRO_ORACLE_H
#define HYDRO_ORACLE_H

int oracle_run_2d(
    int nx, int ny, int g,
    double x_min, double x_max, double y_min, double y_max, double gamma,
    const char *integrator, const char *riemann_solver, const char *slope_limiter,
    const char *bc_x_min, const char *bc_x_max, const char *bc_y_min, const char *bc_y_max,
    double cfl, double tf, long long max_steps,
    double *rho, double *u, double *v, double *p,
    double *mass, double *mom_x, double *mom_y, double *energy,
    long long *num_steps, double *t, double *dt,
    char *errbuf, int errlen);

/* Custom boundary callback, as in BoundaryConditionParam (src/boundary.h:40-48). */
typedef void (*OracleBcFn)(double *density, double *velocity_x, double *velocity_y, double *pressure,
                           int num_ghost_cells_side, int num_cells_x, int num_cells_y);

/* oracle_run_2d plus the gravity source and custom-side callbacks. */
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
    OracleBcFn bc_fn_y_max);

int oracle_run_1d(
    int nx, int g, double x_min, double x_max, double gamma,
    const char *integrator, const char *riemann_solver, const char *slope_limiter,
    const char *bc_x_min, const char *bc_x_max,
    double cfl, double tf, long long max_steps,
    double *rho, double *u, double *p,
    double *mass, double *mom_x, double *energy,
    long long *num_steps, double *t, double *dt,
    char *errbuf, int errlen);

/* oracle_run_1d on a "cartesian_1d", "cylindrical_1d" or "spherical_1d"
 * grid, with the random-choice integrator as well. */
int oracle_run_1d_ex(
    int nx, int g, double x_min, double x_max, double gamma,
    const char *integrator, const char *riemann_solver, const char *slope_limiter,
    const char *bc_x_min, const char *bc_x_max,
    double cfl, double tf, long long max_steps,
    double *rho, double *u, double *p,
    double *mass, double *mom_x, double *energy,
    long long *num_steps, double *t, double *dt,
    char *errbuf, int errlen, const char *coord_sys);

int oracle_hllc_2d(double gamma, double rho_L, double u_L, double v_L, double p_L,
                   double rho_R, double u_R, double v_R, double p_R, double tol, double *out4);
int oracle_exact_flux_1d(double gamma, double rho_L, double u_L, double p_L,
                         double rho_R, double u_R, double p_R, double tol, double speed,
                         double *out3);
int oracle_hllc_1d(double gamma, double rho_L, double u_L, double p_L,
                   double rho_R, double u_R, double p_R, double tol, double *out3);
int oracle_exact_1d(double gamma, double rho_L, double u_L, double p_L,
                    double rho_R, double u_R, double p_R, double tol, double speed, double *out3);
double oracle_guess_p(double gamma, double rho_L, double u_L, double p_L, double a_L,
                      double rho_R, double u_R, double p_R, double a_R, double tol);
int oracle_limit_slope(int limiter_flag, double a, double b, double *out);
/* 0 solved, 1 bracket failure, 2 bisection not converged (message in errbuf). */
int oracle_exact_status(double gamma, double rho_L, double u_L, double p_L,
                        double rho_R, double u_R, double p_R, double tol, char *errbuf, int errlen);

/* The source terms on their own (src/source_term.c:45-259): the RK4 update,
 * then U -> W and the ghost fill, in place on padded arrays.  coord: 2
 * cylindrical_1d, 3 spherical_1d. */
int oracle_geometry_source_1d(int coord, int nx, int g, double x_min, double x_max, double gamma,
                              double dt, const char *bc_x_min, const char *bc_x_max,
                              double *rho, double *u, double *p,
                              double *mass, double *mom_x, double *energy);
int oracle_gravity_source_2d(int nx, int ny, int g, double x_min, double x_max, double y_min,
                             double y_max, double gamma, double gravity, double dt,
                             const char *bc_x_min, const char *bc_x_max, const char *bc_y_min,
                             const char *bc_y_max,
                             double *rho, double *u, double *v, double *p,
                             double *mass, double *mom_x, double *mom_y, double *energy);

/* Number of OpenMP threads the 2D loops use (for the CPU-baseline report). */
int oracle_num_threads(void);

#endif
