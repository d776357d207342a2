/*
 * ref_harness.c -- TEST INFRASTRUCTURE ONLY (never linked into the product).
 *
 * Links against the reference hydroFV sources (src/*.c except storing.c, which
 * needs HDF5) to build oracle/_ref/libhydro_ref_{omp,serial}.so.  It supplies
 * the three storing entry points the reference integrators call, and turns
 * them into a fixed-step-count stop: with is_storing = true and a vanishing
 * storing interval, the integrators call store_snapshot() after every step
 * (src/integrator_muscl_hancock.c:1147-1154,
 * src/integrator_godunov_first_order.c:225-232); the stub returns FAILURE once
 * num_steps reaches the requested count, so the integrator unwinds with the
 * state after exactly that many steps left in the System arrays.
 *
 * Exposes one flat C function per dimensionality so the Python test harness
 * can drive the unmodified reference through its own public API
 * (launch_simulation, src/hydro.h:53-61).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "hydro.h"
#include "source_term.h"

static long long g_stop_after_steps = -1;
static int g_verbose = 0;

/* Settings.verbose of the runs and solves that follow (the reference's
 * exact solver warns every 500 bisection iterations when it is > 0). */
void ref_set_verbose(int verbose)
{
    g_verbose = verbose;
}

StoringParam get_new_storing_param(void)
{
    StoringParam p;
    memset(&p, 0, sizeof(p));
    p.storing_interval = -1.0;
    return p;
}

ErrorStatus finalize_storing_param(StoringParam *__restrict storing_param)
{
    (void) storing_param;
    return make_success_error_status();
}

ErrorStatus store_snapshot(
    const BoundaryConditionParam *__restrict boundary_condition_param,
    const System *__restrict system,
    const IntegratorParam *__restrict integrator_param,
    const SimulationStatus *__restrict simulation_status,
    StoringParam *__restrict storing_param
)
{
    (void) boundary_condition_param;
    (void) system;
    (void) integrator_param;
    storing_param->store_count_++;
    if (g_stop_after_steps >= 0 && simulation_status->num_steps >= g_stop_after_steps)
    {
        ErrorStatus e = make_success_error_status();
        e.return_code = FAILURE;  /* sentinel: requested step count reached */
        return e;
    }
    return make_success_error_status();
}

/* Copy the traceback (if any) into errbuf and release it. */
static int finish(ErrorStatus e, char *errbuf, int errlen, int fixed_stop)
{
    if (errbuf && errlen > 0)
    {
        errbuf[0] = '\0';
        if (e.traceback)
        {
            snprintf(errbuf, (size_t) errlen, "%s", e.traceback);
        }
    }
    /* the step-count sentinel is the one FAILURE without a traceback */
    const int sentinel = fixed_stop && e.return_code == FAILURE && !e.traceback;
    free_traceback(&e);
    return sentinel ? 0 : e.return_code;
}

/*
 * Run a 2D Cartesian problem.  W (rho, u, v, p) and U (mass, mom_x, mom_y,
 * energy) are padded (nx+2g)*(ny+2g) row-major arrays; both are inputs and are
 * overwritten with the final state.  bc[] = {x_min, x_max, y_min, y_max}.
 * max_steps < 0 runs to tf.  Returns the reference's return_code (0 = OK).
 */
typedef void (*RefBcFn)(double *, double *, double *, double *, int, int, int);

/* ref_run_2d plus System.gravity and the callbacks of custom sides. */
int ref_run_2d_ex(
    int nx, int ny, int g,
    double x_min, double x_max, double y_min, double y_max, double gamma,
    const char *integrator, const char *riemann_solver, const char *slope_limiter,
    const char *bc_x_min, const char *bc_x_max, const char *bc_y_min, const char *bc_y_max,
    double cfl, double tf, long long max_steps,
    double *rho, double *u, double *v, double *p,
    double *mass, double *mom_x, double *mom_y, double *energy,
    long long *num_steps, double *t, double *dt,
    char *errbuf, int errlen,
    double gravity, RefBcFn fn_x_min, RefBcFn fn_x_max, RefBcFn fn_y_min, RefBcFn fn_y_max
)
{
    System system = get_new_system_struct();
    system.coord_sys = "cartesian_2d";
    system.gamma = gamma;
    system.x_min = x_min;
    system.x_max = x_max;
    system.y_min = y_min;
    system.y_max = y_max;
    system.num_cells_x = nx;
    system.num_cells_y = ny;
    system.num_ghost_cells_side = g;
    system.gravity = gravity;
    ErrorStatus e = system_init(&system);
    if (e.return_code != SUCCESS)
    {
        return finish(e, errbuf, errlen, 0);
    }
    const size_t n = (size_t) (nx + 2 * g) * (size_t) (ny + 2 * g);
    memcpy(system.density_, rho, n * sizeof(double));
    memcpy(system.velocity_x_, u, n * sizeof(double));
    memcpy(system.velocity_y_, v, n * sizeof(double));
    memcpy(system.pressure_, p, n * sizeof(double));
    memcpy(system.mass_, mass, n * sizeof(double));
    memcpy(system.momentum_x_, mom_x, n * sizeof(double));
    memcpy(system.momentum_y_, mom_y, n * sizeof(double));
    memcpy(system.energy_, energy, n * sizeof(double));

    BoundaryConditionParam bcp = get_new_boundary_condition_param();
    bcp.boundary_condition_x_min = bc_x_min;
    bcp.boundary_condition_x_max = bc_x_max;
    bcp.boundary_condition_y_min = bc_y_min;
    bcp.boundary_condition_y_max = bc_y_max;
    bcp.set_boundary_condition_cartesian_2d_x_min = fn_x_min;
    bcp.set_boundary_condition_cartesian_2d_x_max = fn_x_max;
    bcp.set_boundary_condition_cartesian_2d_y_min = fn_y_min;
    bcp.set_boundary_condition_cartesian_2d_y_max = fn_y_max;

    IntegratorParam ip = get_new_integrator_param();
    ip.integrator = (char *) integrator;
    ip.riemann_solver = (char *) riemann_solver;
    ip.slope_limiter = (char *) slope_limiter;
    ip.cfl = cfl;

    StoringParam sp = get_new_storing_param();
    if (max_steps >= 0)
    {
        sp.is_storing = true;
        sp.storing_interval = 1e-300;
    }
    g_stop_after_steps = max_steps;

    Settings settings = { .verbose = g_verbose, .no_progress_bar = true };
    SimulationParam simp = { .tf = (max_steps >= 0) ? 1e300 : tf };
    SimulationStatus st = { 0, 0.0, 0.0 };

    e = launch_simulation(&bcp, &system, &ip, &sp, &settings, &simp, &st);

    memcpy(rho, system.density_, n * sizeof(double));
    memcpy(u, system.velocity_x_, n * sizeof(double));
    memcpy(v, system.velocity_y_, n * sizeof(double));
    memcpy(p, system.pressure_, n * sizeof(double));
    memcpy(mass, system.mass_, n * sizeof(double));
    memcpy(mom_x, system.momentum_x_, n * sizeof(double));
    memcpy(mom_y, system.momentum_y_, n * sizeof(double));
    memcpy(energy, system.energy_, n * sizeof(double));
    *num_steps = st.num_steps;
    *t = st.t;
    *dt = st.dt;
    free_system_memory(&system);
    return finish(e, errbuf, errlen, max_steps >= 0);
}

int ref_run_2d(
    int nx, int ny, int g,
    double x_min, double x_max, double y_min, double y_max, double gamma,
    const char *integrator, const char *riemann_solver, const char *slope_limiter,
    const char *bc_x_min, const char *bc_x_max, const char *bc_y_min, const char *bc_y_max,
    double cfl, double tf, long long max_steps,
    double *rho, double *u, double *v, double *p,
    double *mass, double *mom_x, double *mom_y, double *energy,
    long long *num_steps, double *t, double *dt,
    char *errbuf, int errlen
)
{
    return ref_run_2d_ex(nx, ny, g, x_min, x_max, y_min, y_max, gamma, integrator, riemann_solver,
                         slope_limiter, bc_x_min, bc_x_max, bc_y_min, bc_y_max, cfl, tf, max_steps,
                         rho, u, v, p, mass, mom_x, mom_y, energy, num_steps, t, dt, errbuf, errlen,
                         0.0, NULL, NULL, NULL, NULL);
}

/* Run a 1D Cartesian problem; arrays are padded to nx+2g. */
int ref_run_1d_ex(
    int nx, int g, double x_min, double x_max, double gamma,
    const char *integrator, const char *riemann_solver, const char *slope_limiter,
    const char *bc_x_min, const char *bc_x_max,
    double cfl, double tf, long long max_steps,
    double *rho, double *u, double *p,
    double *mass, double *mom_x, double *energy,
    long long *num_steps, double *t, double *dt,
    char *errbuf, int errlen, const char *coord_sys
);

int ref_run_1d(
    int nx, int g, double x_min, double x_max, double gamma,
    const char *integrator, const char *riemann_solver, const char *slope_limiter,
    const char *bc_x_min, const char *bc_x_max,
    double cfl, double tf, long long max_steps,
    double *rho, double *u, double *p,
    double *mass, double *mom_x, double *energy,
    long long *num_steps, double *t, double *dt,
    char *errbuf, int errlen
)
{
    return ref_run_1d_ex(nx, g, x_min, x_max, gamma, integrator, riemann_solver, slope_limiter, bc_x_min,
                         bc_x_max, cfl, tf, max_steps, rho, u, p, mass, mom_x, energy, num_steps, t, dt,
                         errbuf, errlen, "cartesian_1d");
}

/* ref_run_1d on a cartesian_1d, cylindrical_1d or spherical_1d grid. */
int ref_run_1d_ex(
    int nx, int g, double x_min, double x_max, double gamma,
    const char *integrator, const char *riemann_solver, const char *slope_limiter,
    const char *bc_x_min, const char *bc_x_max,
    double cfl, double tf, long long max_steps,
    double *rho, double *u, double *p,
    double *mass, double *mom_x, double *energy,
    long long *num_steps, double *t, double *dt,
    char *errbuf, int errlen, const char *coord_sys
)
{
    System system = get_new_system_struct();
    system.coord_sys = coord_sys;
    system.gamma = gamma;
    system.x_min = x_min;
    system.x_max = x_max;
    system.num_cells_x = nx;
    system.num_ghost_cells_side = g;
    ErrorStatus e = system_init(&system);
    if (e.return_code != SUCCESS)
    {
        return finish(e, errbuf, errlen, 0);
    }
    const size_t n = (size_t) (nx + 2 * g);
    memcpy(system.density_, rho, n * sizeof(double));
    memcpy(system.velocity_x_, u, n * sizeof(double));
    memcpy(system.pressure_, p, n * sizeof(double));
    memcpy(system.mass_, mass, n * sizeof(double));
    memcpy(system.momentum_x_, mom_x, n * sizeof(double));
    memcpy(system.energy_, energy, n * sizeof(double));

    BoundaryConditionParam bcp = get_new_boundary_condition_param();
    bcp.boundary_condition_x_min = bc_x_min;
    bcp.boundary_condition_x_max = bc_x_max;

    IntegratorParam ip = get_new_integrator_param();
    ip.integrator = (char *) integrator;
    ip.riemann_solver = (char *) riemann_solver;
    ip.slope_limiter = (char *) slope_limiter;
    ip.cfl = cfl;

    StoringParam sp = get_new_storing_param();
    if (max_steps >= 0)
    {
        sp.is_storing = true;
        sp.storing_interval = 1e-300;
    }
    g_stop_after_steps = max_steps;

    Settings settings = { .verbose = g_verbose, .no_progress_bar = true };
    SimulationParam simp = { .tf = (max_steps >= 0) ? 1e300 : tf };
    SimulationStatus st = { 0, 0.0, 0.0 };

    e = launch_simulation(&bcp, &system, &ip, &sp, &settings, &simp, &st);

    memcpy(rho, system.density_, n * sizeof(double));
    memcpy(u, system.velocity_x_, n * sizeof(double));
    memcpy(p, system.pressure_, n * sizeof(double));
    memcpy(mass, system.mass_, n * sizeof(double));
    memcpy(mom_x, system.momentum_x_, n * sizeof(double));
    memcpy(energy, system.energy_, n * sizeof(double));
    *num_steps = st.num_steps;
    *t = st.t;
    *dt = st.dt;
    free_system_memory(&system);
    return finish(e, errbuf, errlen, max_steps >= 0);
}

/* Pointwise known-answer helpers: thin pass-throughs to exported reference
 * functions (src/riemann_solver_hllc.h:32-61, src/riemann_solver_exact.h:37-87,
 * src/riemann_solver.h:144-186, src/slope_limiter.h:24-47). */
int ref_hllc_2d(double gamma, double rho_L, double u_L, double v_L, double p_L,
                double rho_R, double u_R, double v_R, double p_R, double tol, double *out4)
{
    ErrorStatus e = solve_flux_hllc_2d(&out4[0], &out4[1], &out4[2], &out4[3], gamma,
                                       rho_L, u_L, v_L, p_L, rho_R, u_R, v_R, p_R, tol);
    int rc = e.return_code;
    free_traceback(&e);
    return rc;
}

int ref_exact_flux_1d(double gamma, double rho_L, double u_L, double p_L,
                      double rho_R, double u_R, double p_R, double tol, double speed, double *out3)
{
    ErrorStatus e = solve_flux_exact_1d(&out3[0], &out3[1], &out3[2], gamma,
                                        rho_L, u_L, p_L, rho_R, u_R, p_R, tol, speed, g_verbose);
    int rc = e.return_code;
    free_traceback(&e);
    return rc;
}

int ref_hllc_1d(double gamma, double rho_L, double u_L, double p_L,
                double rho_R, double u_R, double p_R, double tol, double *out3)
{
    ErrorStatus e = solve_flux_hllc_1d(&out3[0], &out3[1], &out3[2], gamma,
                                       rho_L, u_L, p_L, rho_R, u_R, p_R, tol);
    int rc = e.return_code;
    free_traceback(&e);
    return rc;
}

int ref_exact_1d(double gamma, double rho_L, double u_L, double p_L,
                 double rho_R, double u_R, double p_R, double tol, double speed, double *out3)
{
    ErrorStatus e = solve_exact_1d(&out3[0], &out3[1], &out3[2], gamma,
                                   rho_L, u_L, p_L, rho_R, u_R, p_R, tol, speed, g_verbose);
    int rc = e.return_code;
    free_traceback(&e);
    return rc;
}

/* solve_exact_1d's way out, as oracle_exact_status: 0 solved, 1 bracket
 * failure, 2 bisection not converged, told apart by the reference's own
 * traceback text, which is copied into errbuf. */
int ref_exact_status(double gamma, double rho_L, double u_L, double p_L,
                     double rho_R, double u_R, double p_R, double tol, char *errbuf, int errlen)
{
    double out3[3];
    ErrorStatus e = solve_exact_1d(&out3[0], &out3[1], &out3[2], gamma,
                                   rho_L, u_L, p_L, rho_R, u_R, p_R, tol, 0.0, g_verbose);
    int kind = 0;
    if (errbuf && errlen > 0) errbuf[0] = '\0';
    if (e.return_code != SUCCESS)
    {
        kind = (e.traceback && strstr(e.traceback, "Failed to bracket")) ? 1 : 2;
        if (errbuf && errlen > 0 && e.traceback) snprintf(errbuf, (size_t) errlen, "%s", e.traceback);
    }
    free_traceback(&e);
    return kind;
}

/* The reference's own add_geometry_source_term / add_gravity_source_term_2d
 * on a System set up by its system_init, arrays copied in and out (same
 * argument order as the oracle's source-term exports). */
int ref_geometry_source_1d(int coord, int nx, int g, double x_min, double x_max, double gamma,
                           double dt, const char *bc_x_min, const char *bc_x_max,
                           double *rho, double *u, double *p,
                           double *mass, double *mom_x, double *energy)
{
    System system = get_new_system_struct();
    system.coord_sys = (coord == 2) ? "cylindrical_1d" : "spherical_1d";
    system.gamma = gamma;
    system.x_min = x_min;
    system.x_max = x_max;
    system.num_cells_x = nx;
    system.num_ghost_cells_side = g;
    ErrorStatus e = system_init(&system);
    if (e.return_code != SUCCESS) return finish(e, NULL, 0, 0);
    const size_t n = (size_t) (nx + 2 * g);
    double *fields[6] = { system.density_, system.velocity_x_, system.pressure_,
                          system.mass_, system.momentum_x_, system.energy_ };
    double *arrays[6] = { rho, u, p, mass, mom_x, energy };
    for (int q = 0; q < 6; q++) memcpy(fields[q], arrays[q], n * sizeof(double));
    BoundaryConditionParam bcp = get_new_boundary_condition_param();
    bcp.boundary_condition_x_min = bc_x_min;
    bcp.boundary_condition_x_max = bc_x_max;
    e = finalize_boundary_condition_param(&system, &bcp);
    if (e.return_code == SUCCESS) e = add_geometry_source_term(&bcp, &system, dt);
    for (int q = 0; q < 6; q++) memcpy(arrays[q], fields[q], n * sizeof(double));
    free_system_memory(&system);
    return finish(e, NULL, 0, 0);
}

int ref_gravity_source_2d(int nx, int ny, int g, double x_min, double x_max, double y_min,
                          double y_max, double gamma, double gravity, double dt,
                          const char *bc_x_min, const char *bc_x_max, const char *bc_y_min,
                          const char *bc_y_max,
                          double *rho, double *u, double *v, double *p,
                          double *mass, double *mom_x, double *mom_y, double *energy)
{
    System system = get_new_system_struct();
    system.coord_sys = "cartesian_2d";
    system.gamma = gamma;
    system.x_min = x_min;
    system.x_max = x_max;
    system.y_min = y_min;
    system.y_max = y_max;
    system.num_cells_x = nx;
    system.num_cells_y = ny;
    system.num_ghost_cells_side = g;
    system.gravity = gravity;
    ErrorStatus e = system_init(&system);
    if (e.return_code != SUCCESS) return finish(e, NULL, 0, 0);
    const size_t n = (size_t) (nx + 2 * g) * (size_t) (ny + 2 * g);
    double *fields[8] = { system.density_, system.velocity_x_, system.velocity_y_, system.pressure_,
                          system.mass_, system.momentum_x_, system.momentum_y_, system.energy_ };
    double *arrays[8] = { rho, u, v, p, mass, mom_x, mom_y, energy };
    for (int q = 0; q < 8; q++) memcpy(fields[q], arrays[q], n * sizeof(double));
    BoundaryConditionParam bcp = get_new_boundary_condition_param();
    bcp.boundary_condition_x_min = bc_x_min;
    bcp.boundary_condition_x_max = bc_x_max;
    bcp.boundary_condition_y_min = bc_y_min;
    bcp.boundary_condition_y_max = bc_y_max;
    e = finalize_boundary_condition_param(&system, &bcp);
    if (e.return_code == SUCCESS) e = add_gravity_source_term_2d(&bcp, &system, dt);
    for (int q = 0; q < 8; q++) memcpy(arrays[q], fields[q], n * sizeof(double));
    free_system_memory(&system);
    return finish(e, NULL, 0, 0);
}

double ref_guess_p(double gamma, double rho_L, double u_L, double p_L, double a_L,
                   double rho_R, double u_R, double p_R, double a_R, double tol)
{
    return guess_p(gamma, rho_L, u_L, p_L, a_L, rho_R, u_R, p_R, a_R, tol);
}

int ref_limit_slope(int limiter_flag, double a, double b, double *out)
{
    IntegratorParam ip = get_new_integrator_param();
    ip.slope_limiter_flag_ = limiter_flag;
    ErrorStatus e = limit_slope(out, &ip, a, b);
    int rc = e.return_code;
    free_traceback(&e);
    return rc;
}
