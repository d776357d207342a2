/*
 * params.c -- integrator / Riemann-solver / slope-limiter parameters and the
 * launch entry point.
 *
 * Defaults, name tables, checks and messages follow src/integrator.c:16-106,
 * src/riemann_solver.c:23-45, src/slope_limiter.c:18-47 and
 * src/hydro.c:29-265.  integrator_launch_simulation dispatches to the GPU
 * integrators in integrate_gpu.c.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "hydro.h"
#include "host_internal.h"

IntegratorParam get_new_integrator_param(void)
{
    IntegratorParam p;
    memset(&p, 0, sizeof p);
    p.integrator = NULL;
    p.riemann_solver = NULL;
    p.slope_limiter = NULL;
    p.cfl = 0.5;
    p.cfl_initial_shrink_factor = 0.2;
    p.cfl_initial_shrink_num_steps = 10;
    p.tol = 1e-6;
    p.integrator_flag_ = -1;
    p.riemann_solver_flag_ = -1;
    p.slope_limiter_flag_ = -1;
    return p;
}

static ErrorStatus get_integrator_flag(IntegratorParam *p)
{
    static const struct { const char *name; int flag; } table[] = {
        { "random_choice_1d", INTEGRATOR_RANDOM_CHOICE_1D },
        { "godunov_first_order_1d", INTEGRATOR_GODUNOV_FIRST_ORDER_1D },
        { "godunov_first_order_2d", INTEGRATOR_GODUNOV_FIRST_ORDER_2D },
        { "muscl_hancock_1d", INTEGRATOR_MUSCL_HANCOCK_1D },
        { "muscl_hancock_2d", INTEGRATOR_MUSCL_HANCOCK_2D },
    };
    if (!p->integrator)
    {
        return WRAP_RAISE_ERROR(POINTER_ERROR, "Integrator is not set.");
    }
    for (size_t k = 0; k < sizeof table / sizeof table[0]; k++)
    {
        if (strcmp(p->integrator, table[k].name) == 0)
        {
            p->integrator_flag_ = table[k].flag;
            return make_success_error_status();
        }
    }
    return WRAP_RAISE_ERROR(VALUE_ERROR, "Integrator not recognized.");
}

ErrorStatus get_riemann_solver_flag(IntegratorParam *__restrict p)
{
    if (!p->riemann_solver)
    {
        return WRAP_RAISE_ERROR(POINTER_ERROR, "Riemann solver is not set.");
    }
    if (strcmp(p->riemann_solver, "riemann_solver_exact") == 0)
    {
        p->riemann_solver_flag_ = RIEMANN_SOLVER_EXACT;
        return make_success_error_status();
    }
    if (strcmp(p->riemann_solver, "riemann_solver_hllc") == 0)
    {
        p->riemann_solver_flag_ = RIEMANN_SOLVER_HLLC;
        return make_success_error_status();
    }
    return WRAP_RAISE_ERROR(VALUE_ERROR, "Riemann solver not recognized.");
}

ErrorStatus get_slope_limiter_flag(IntegratorParam *__restrict p)
{
    if (!p || !p->slope_limiter)
    {
        return WRAP_RAISE_ERROR(POINTER_ERROR, "Integrator parameter or slope limiter is NULL.");
    }
    if (strcmp(p->slope_limiter, "minmod") == 0)
        p->slope_limiter_flag_ = SLOPE_LIMITER_MINMOD;
    else if (strcmp(p->slope_limiter, "van_leer") == 0)
        p->slope_limiter_flag_ = SLOPE_LIMITER_VAN_LEER;
    else if (strcmp(p->slope_limiter, "monotonized_central") == 0)
        p->slope_limiter_flag_ = SLOPE_LIMITER_MONOTONIZED_CENTRAL;
    else
        return WRAP_RAISE_ERROR(VALUE_ERROR, "Slope limiter not recognized.");
    return make_success_error_status();
}

ErrorStatus finalize_integrator_param(IntegratorParam *__restrict p)
{
    ErrorStatus e = get_integrator_flag(p);
    if (e.return_code != SUCCESS) return e;
    e = get_riemann_solver_flag(p);
    if (e.return_code != SUCCESS) return e;
    e = get_slope_limiter_flag(p);
    if (e.return_code != SUCCESS) return e;
    if (p->cfl <= 0.0)
        return WRAP_RAISE_ERROR(VALUE_ERROR, "CFL number must be positive.");
    if (p->cfl_initial_shrink_factor <= 0.0)
        return WRAP_RAISE_ERROR(VALUE_ERROR, "CFL initial shrink factor must be positive.");
    if (p->cfl_initial_shrink_num_steps <= 0)
        return WRAP_RAISE_ERROR(VALUE_ERROR, "CFL initial shrink number of steps must be positive.");
    if (p->tol <= 0.0)
        return WRAP_RAISE_ERROR(VALUE_ERROR, "Tolerance must be positive.");
    return make_success_error_status();
}

ErrorStatus integrator_launch_simulation(
    BoundaryConditionParam *__restrict bcp,
    System *__restrict system,
    IntegratorParam *__restrict ip,
    StoringParam *__restrict sp,
    Settings *__restrict settings,
    SimulationParam *__restrict simp,
    SimulationStatus *__restrict status
)
{
    switch (ip->integrator_flag_)
    {
        case INTEGRATOR_RANDOM_CHOICE_1D:
            return WRAP_TRACEBACK(random_choice_1d(bcp, system, ip, sp, settings, simp, status));
        case INTEGRATOR_GODUNOV_FIRST_ORDER_1D:
            return WRAP_TRACEBACK(godunov_first_order_1d(bcp, system, ip, sp, settings, simp, status));
        case INTEGRATOR_GODUNOV_FIRST_ORDER_2D:
            return WRAP_TRACEBACK(godunov_first_order_2d(bcp, system, ip, sp, settings, simp, status));
        case INTEGRATOR_MUSCL_HANCOCK_1D:
            return WRAP_TRACEBACK(muscl_hancock_1d(bcp, system, ip, sp, settings, simp, status));
        case INTEGRATOR_MUSCL_HANCOCK_2D:
            return WRAP_TRACEBACK(muscl_hancock_2d(bcp, system, ip, sp, settings, simp, status));
        default:
            return WRAP_RAISE_ERROR(VALUE_ERROR, "Integrator flag not recognized.");
    }
}

ErrorStatus hydro_final_check(const System *system, const IntegratorParam *ip)
{
    char msg[512];
    const int flag = ip->integrator_flag_;
    switch (flag)
    {
        case INTEGRATOR_RANDOM_CHOICE_1D:
        case INTEGRATOR_GODUNOV_FIRST_ORDER_1D:
        case INTEGRATOR_GODUNOV_FIRST_ORDER_2D:
        case INTEGRATOR_GODUNOV_FIRST_ORDER_3D:
            if (system->num_ghost_cells_side < 1)
                return WRAP_RAISE_ERROR(VALUE_ERROR, "Number of ghost cells must be at least 1.");
            break;
        case INTEGRATOR_MUSCL_HANCOCK_1D:
        case INTEGRATOR_MUSCL_HANCOCK_2D:
            if (system->num_ghost_cells_side < 2)
                return WRAP_RAISE_ERROR(VALUE_ERROR, "Number of ghost cells must be at least 2.");
            break;
        default:
            return WRAP_RAISE_ERROR(VALUE_ERROR, "Integrator flag not recognized.");
    }
    const int cs = system->coord_sys_flag_;
    if (flag == INTEGRATOR_RANDOM_CHOICE_1D || flag == INTEGRATOR_GODUNOV_FIRST_ORDER_1D ||
        flag == INTEGRATOR_MUSCL_HANCOCK_1D)
    {
        if (cs != COORD_SYS_CARTESIAN_1D && cs != COORD_SYS_CYLINDRICAL_1D && cs != COORD_SYS_SPHERICAL_1D)
        {
            snprintf(msg, sizeof msg,
                     "Wrong coordinate system. Supported coordinate system for integrator \"%s\": "
                     "\"cartesian_1d\", \"cylindrical_1d\" and \"spherical_1d\", got: \"%s\"",
                     ip->integrator, system->coord_sys);
            return WRAP_RAISE_ERROR(VALUE_ERROR, msg);
        }
    }
    else if (flag == INTEGRATOR_GODUNOV_FIRST_ORDER_2D || flag == INTEGRATOR_MUSCL_HANCOCK_2D)
    {
        if (cs != COORD_SYS_CARTESIAN_2D)
        {
            snprintf(msg, sizeof msg,
                     "Wrong coordinate system. Supported coordinate system for integrator \"%s\": "
                     "\"cartesian_2d\", got: \"%s\"", ip->integrator, system->coord_sys);
            return WRAP_RAISE_ERROR(VALUE_ERROR, msg);
        }
    }
    else if (flag == INTEGRATOR_GODUNOV_FIRST_ORDER_3D && cs != COORD_SYS_CARTESIAN_3D)
    {
        snprintf(msg, sizeof msg,
                 "Wrong coordinate system. Supported coordinate system for integrator \"%s\": "
                 "\"cartesian_3d\", got: \"%s\"", ip->integrator, system->coord_sys);
        return WRAP_RAISE_ERROR(VALUE_ERROR, msg);
    }
    if (flag == INTEGRATOR_RANDOM_CHOICE_1D && ip->riemann_solver_flag_ != RIEMANN_SOLVER_EXACT)
    {
        snprintf(msg, sizeof msg,
                 "Supported Riemann solver for random choice method 1D: \"riemann_solver_exact\", got: \"%s\"",
                 ip->riemann_solver);
        return WRAP_RAISE_ERROR(VALUE_ERROR, msg);
    }
    return make_success_error_status();
}

ErrorStatus launch_simulation(
    BoundaryConditionParam *__restrict bcp,
    System *__restrict system,
    IntegratorParam *__restrict ip,
    StoringParam *__restrict sp,
    Settings *__restrict settings,
    SimulationParam *__restrict simp,
    SimulationStatus *__restrict status
)
{
    ErrorStatus e = WRAP_TRACEBACK(finalize_boundary_condition_param(system, bcp));
    if (e.return_code != SUCCESS) return e;
    e = WRAP_TRACEBACK(finalize_integrator_param(ip));
    if (e.return_code != SUCCESS) return e;
    e = WRAP_TRACEBACK(finalize_storing_param(sp));
    if (e.return_code != SUCCESS) return e;
    e = WRAP_TRACEBACK(hydro_final_check(system, ip));
    if (e.return_code != SUCCESS) return e;
    return WRAP_TRACEBACK(integrator_launch_simulation(bcp, system, ip, sp, settings, simp, status));
}

/* Device error codes of the GPU kernels (hydro::DEV_ERR_*). */
ErrorStatus hydro_device_error_status(int code)
{
    switch (code)
    {
        case 1:  /* src/riemann_solver_hllc.c:372-375 */
            return WRAP_RAISE_ERROR(VALUE_ERROR,
                                    "Invalid wave speed for the HLLC riemann solver. Possible fix: use a smaller CFL.");
        case 2:  /* src/integrator_muscl_hancock.c:545-549 */
            return WRAP_RAISE_ERROR(VALUE_ERROR, "dt is zero.");
        case 3:  /* src/riemann_solver_exact.c:702-707 */
            return WRAP_RAISE_ERROR(FAILURE, "Failed to bracket the root for bisection method.");
        case 4:  /* src/riemann_solver_exact.c:745-754 */
            return WRAP_RAISE_ERROR(FAILURE,
                                    "Bisection method did not converge after 5001 iterations for exact riemann solver.");
        case 5:
            return WRAP_RAISE_ERROR(FAILURE, "A bounded device-side wait timed out.");
        default:
            return WRAP_RAISE_ERROR(UNKNOWN_ERROR, "Unknown device error.");
    }
}
