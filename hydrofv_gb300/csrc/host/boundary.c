/*
 * boundary.c -- boundary-condition names, validation and the host ghost
 * fill used during problem set-up.
 *
 * Follows src/boundary.c: names "none" / "reflective" / "transmissive" /
 * "periodic" / "custom" (:51-389), periodic must be set on both sides of an
 * axis, custom needs a callback (:250-389).  The host fill (:411-777) works on
 * the primitive arrays only: x sides over interior rows, then y sides over
 * interior columns, corners untouched; transmissive is a mirror copy,
 * reflective a mirror with the normal velocity negated, periodic copies the
 * opposite interior (both sides handled in the *_max case).  On the GPU the
 * same ghost values are produced by index remapping inside the step kernel.
 */
#include <stdio.h>
#include <string.h>

#include "hydro.h"

BoundaryConditionParam get_new_boundary_condition_param(void)
{
    BoundaryConditionParam p;
    memset(&p, 0, sizeof p);
    p.boundary_condition_flag_x_min_ = -1;
    p.boundary_condition_flag_x_max_ = -1;
    p.boundary_condition_flag_y_min_ = -1;
    p.boundary_condition_flag_y_max_ = -1;
    p.boundary_condition_flag_z_min_ = -1;
    p.boundary_condition_flag_z_max_ = -1;
    return p;
}

static int bc_flag(const char *name)
{
    if (strcmp(name, "none") == 0) return BOUNDARY_CONDITION_NONE;
    if (strcmp(name, "reflective") == 0) return BOUNDARY_CONDITION_REFLECTIVE;
    if (strcmp(name, "transmissive") == 0) return BOUNDARY_CONDITION_TRANSMISSIVE;
    if (strcmp(name, "periodic") == 0) return BOUNDARY_CONDITION_PERIODIC;
    if (strcmp(name, "custom") == 0) return BOUNDARY_CONDITION_CUSTOM;
    return -1;
}

/* Resolve both sides of one axis; axis is 'x', 'y' or 'z'. */
static ErrorStatus resolve_axis(char axis, const char *lo, const char *hi, int *flag_lo, int *flag_hi)
{
    char msg[96];
    if (!lo || !hi)
    {
        snprintf(msg, sizeof msg, "Boundary condition for %c_min or %c_max is NULL.", axis, axis);
        return WRAP_RAISE_ERROR(POINTER_ERROR, msg);
    }
    *flag_lo = bc_flag(lo);
    if (*flag_lo < 0)
    {
        snprintf(msg, sizeof msg, "Boundary condition for %c_min is not recognized.", axis);
        return WRAP_RAISE_ERROR(VALUE_ERROR, msg);
    }
    *flag_hi = bc_flag(hi);
    if (*flag_hi < 0)
    {
        snprintf(msg, sizeof msg, "Boundary condition for %c_max is not recognized.", axis);
        return WRAP_RAISE_ERROR(VALUE_ERROR, msg);
    }
    return make_success_error_status();
}

static ErrorStatus check_periodic(char axis, int lo, int hi)
{
    if ((lo == BOUNDARY_CONDITION_PERIODIC || hi == BOUNDARY_CONDITION_PERIODIC) && lo != hi)
    {
        char msg[96];
        snprintf(msg, sizeof msg, "Periodic boundary condition mismatch for %c_min and %c_max.", axis, axis);
        return WRAP_RAISE_ERROR(VALUE_ERROR, msg);
    }
    return make_success_error_status();
}

ErrorStatus finalize_boundary_condition_param(
    const System *__restrict system,
    BoundaryConditionParam *__restrict p
)
{
    ErrorStatus e;
    const int flag = system->coord_sys_flag_;
    const int is3d = flag == COORD_SYS_CARTESIAN_3D;
    const int is2d = flag == COORD_SYS_CARTESIAN_2D || is3d;
    const int is1d = flag == COORD_SYS_CARTESIAN_1D || flag == COORD_SYS_CYLINDRICAL_1D ||
                     flag == COORD_SYS_SPHERICAL_1D;
    if (!is1d && !is2d)
    {
        return WRAP_RAISE_ERROR(VALUE_ERROR, "Coordinate system flag not recognized.");
    }
    if (is3d)
    {
        e = resolve_axis('z', p->boundary_condition_z_min, p->boundary_condition_z_max,
                         &p->boundary_condition_flag_z_min_, &p->boundary_condition_flag_z_max_);
        if (e.return_code != SUCCESS) return e;
    }
    if (is2d)
    {
        e = resolve_axis('y', p->boundary_condition_y_min, p->boundary_condition_y_max,
                         &p->boundary_condition_flag_y_min_, &p->boundary_condition_flag_y_max_);
        if (e.return_code != SUCCESS) return e;
    }
    e = resolve_axis('x', p->boundary_condition_x_min, p->boundary_condition_x_max,
                     &p->boundary_condition_flag_x_min_, &p->boundary_condition_flag_x_max_);
    if (e.return_code != SUCCESS) return e;

    if (is3d)
    {
        e = check_periodic('z', p->boundary_condition_flag_z_min_, p->boundary_condition_flag_z_max_);
        if (e.return_code != SUCCESS) return e;
    }
    if (is2d)
    {
        e = check_periodic('y', p->boundary_condition_flag_y_min_, p->boundary_condition_flag_y_max_);
        if (e.return_code != SUCCESS) return e;
    }
    e = check_periodic('x', p->boundary_condition_flag_x_min_, p->boundary_condition_flag_x_max_);
    if (e.return_code != SUCCESS) return e;

    if (is1d)
    {
        if (p->boundary_condition_flag_x_min_ == BOUNDARY_CONDITION_CUSTOM && !p->set_boundary_condition_1d_x_min)
            return WRAP_RAISE_ERROR(POINTER_ERROR, "Custom boundary condition pointer for x_min is NULL.");
        if (p->boundary_condition_flag_x_max_ == BOUNDARY_CONDITION_CUSTOM && !p->set_boundary_condition_1d_x_max)
            return WRAP_RAISE_ERROR(POINTER_ERROR, "Custom boundary condition pointer for x_max is NULL.");
    }
    else if (!is3d)
    {
        if (p->boundary_condition_flag_x_min_ == BOUNDARY_CONDITION_CUSTOM && !p->set_boundary_condition_cartesian_2d_x_min)
            return WRAP_RAISE_ERROR(POINTER_ERROR, "Custom boundary condition pointer for x_min is NULL.");
        if (p->boundary_condition_flag_x_max_ == BOUNDARY_CONDITION_CUSTOM && !p->set_boundary_condition_cartesian_2d_x_max)
            return WRAP_RAISE_ERROR(POINTER_ERROR, "Custom boundary condition pointer for x_max is NULL.");
        if (p->boundary_condition_flag_y_min_ == BOUNDARY_CONDITION_CUSTOM && !p->set_boundary_condition_cartesian_2d_y_min)
            return WRAP_RAISE_ERROR(POINTER_ERROR, "Custom boundary condition pointer for y_min is NULL.");
        if (p->boundary_condition_flag_y_max_ == BOUNDARY_CONDITION_CUSTOM && !p->set_boundary_condition_cartesian_2d_y_max)
            return WRAP_RAISE_ERROR(POINTER_ERROR, "Custom boundary condition pointer for y_max is NULL.");
    }
    else
    {
        return WRAP_RAISE_ERROR(NOT_IMPLEMENTED_ERROR, "Custom boundary condition for 3D is not implemented.");
    }
    return make_success_error_status();
}

ErrorStatus set_boundary_condition_1d(
    const BoundaryConditionParam *__restrict p,
    double *__restrict density,
    double *__restrict velocity_x,
    double *__restrict pressure,
    const int g,
    const int n
)
{
    const int flags[2] = { p->boundary_condition_flag_x_min_, p->boundary_condition_flag_x_max_ };
    for (int side = 0; side < 2; side++)
    {
        switch (flags[side])
        {
            case BOUNDARY_CONDITION_NONE:
                break;
            case BOUNDARY_CONDITION_REFLECTIVE:
            case BOUNDARY_CONDITION_TRANSMISSIVE:
            {
                const double sign = (flags[side] == BOUNDARY_CONDITION_REFLECTIVE) ? -1.0 : 1.0;
                for (int k = 0; k < g; k++)
                {
                    const int dst = side == 0 ? g - 1 - k : g + n + k;
                    const int src = side == 0 ? g + k : g + n - 1 - k;
                    density[dst] = density[src];
                    velocity_x[dst] = (sign < 0.0) ? -velocity_x[src] : velocity_x[src];
                    pressure[dst] = pressure[src];
                }
                break;
            }
            case BOUNDARY_CONDITION_PERIODIC:
                if (side == 1)
                {
                    for (int k = 0; k < g; k++)
                    {
                        density[g + n + k] = density[g + k];
                        velocity_x[g + n + k] = velocity_x[g + k];
                        pressure[g + n + k] = pressure[g + k];
                        density[g - 1 - k] = density[g + n - 1 - k];
                        velocity_x[g - 1 - k] = velocity_x[g + n - 1 - k];
                        pressure[g - 1 - k] = pressure[g + n - 1 - k];
                    }
                }
                break;
            case BOUNDARY_CONDITION_CUSTOM:
                if (side == 0) p->set_boundary_condition_1d_x_min(density, velocity_x, pressure, g, n);
                else p->set_boundary_condition_1d_x_max(density, velocity_x, pressure, g, n);
                break;
            default:
                return WRAP_RAISE_ERROR(VALUE_ERROR, side == 0 ? "Boundary condition flag not recognized for x_min."
                                                                : "Boundary condition flag not recognized for x_max.");
        }
    }
    return make_success_error_status();
}

/* Copy one ghost cell of the four primitive fields; neg selects the velocity
 * component to negate (0 none, 1 x, 2 y). */
static inline void copy_cell(double *rho, double *u, double *v, double *p, long long dst, long long src, int neg)
{
    rho[dst] = rho[src];
    u[dst] = (neg == 1) ? -u[src] : u[src];
    v[dst] = (neg == 2) ? -v[src] : v[src];
    p[dst] = p[src];
}

ErrorStatus set_boundary_condition_cartesian_2d(
    const BoundaryConditionParam *__restrict p,
    double *__restrict rho,
    double *__restrict u,
    double *__restrict v,
    double *__restrict pr,
    const int g,
    const int nx,
    const int ny
)
{
    const long long tx = nx + 2 * g;
    static const char *const names[4] = { "x_min", "x_max", "y_min", "y_max" };
    const int flags[4] = { p->boundary_condition_flag_x_min_, p->boundary_condition_flag_x_max_,
                           p->boundary_condition_flag_y_min_, p->boundary_condition_flag_y_max_ };
    for (int side = 0; side < 4; side++)
    {
        const int f = flags[side];
        const int is_x = side < 2, is_max = side & 1;
        switch (f)
        {
            case BOUNDARY_CONDITION_NONE:
                break;
            case BOUNDARY_CONDITION_REFLECTIVE:
            case BOUNDARY_CONDITION_TRANSMISSIVE:
            case BOUNDARY_CONDITION_PERIODIC:
            {
                if (f == BOUNDARY_CONDITION_PERIODIC && !is_max) break;
                const int neg = (f == BOUNDARY_CONDITION_REFLECTIVE) ? (is_x ? 1 : 2) : 0;
                const int span = is_x ? ny : nx;
                for (int k = 0; k < g; k++)
                {
                    for (int m = g; m < g + span; m++)
                    {
                        if (is_x)
                        {
                            const long long row = (long long) m * tx;
                            if (f == BOUNDARY_CONDITION_PERIODIC)
                            {
                                copy_cell(rho, u, v, pr, row + g + nx + k, row + g + k, 0);
                                copy_cell(rho, u, v, pr, row + g - 1 - k, row + g + nx - 1 - k, 0);
                            }
                            else if (!is_max)
                                copy_cell(rho, u, v, pr, row + g - 1 - k, row + g + k, neg);
                            else
                                copy_cell(rho, u, v, pr, row + g + nx + k, row + g + nx - 1 - k, neg);
                        }
                        else
                        {
                            if (f == BOUNDARY_CONDITION_PERIODIC)
                            {
                                copy_cell(rho, u, v, pr, (g + ny + k) * tx + m, (g + k) * tx + m, 0);
                                copy_cell(rho, u, v, pr, (g - 1 - k) * tx + m, (g + ny - 1 - k) * tx + m, 0);
                            }
                            else if (!is_max)
                                copy_cell(rho, u, v, pr, (g - 1 - k) * tx + m, (g + k) * tx + m, neg);
                            else
                                copy_cell(rho, u, v, pr, (g + ny + k) * tx + m, (g + ny - 1 - k) * tx + m, neg);
                        }
                    }
                }
                break;
            }
            case BOUNDARY_CONDITION_CUSTOM:
            {
                set_boundary_condition_cartesian_2d_func fn =
                    side == 0 ? p->set_boundary_condition_cartesian_2d_x_min :
                    side == 1 ? p->set_boundary_condition_cartesian_2d_x_max :
                    side == 2 ? p->set_boundary_condition_cartesian_2d_y_min :
                                p->set_boundary_condition_cartesian_2d_y_max;
                fn(rho, u, v, pr, g, nx, ny);
                break;
            }
            default:
            {
                char msg[64];
                snprintf(msg, sizeof msg, "Boundary condition flag not recognized for %s.", names[side]);
                return WRAP_RAISE_ERROR(VALUE_ERROR, msg);
            }
        }
    }
    return make_success_error_status();
}

ErrorStatus set_boundary_condition(
    const BoundaryConditionParam *__restrict p,
    System *__restrict s
)
{
    switch (s->coord_sys_flag_)
    {
        case COORD_SYS_CARTESIAN_1D:
        case COORD_SYS_CYLINDRICAL_1D:
        case COORD_SYS_SPHERICAL_1D:
            return WRAP_TRACEBACK(set_boundary_condition_1d(p, s->density_, s->velocity_x_, s->pressure_,
                                                            s->num_ghost_cells_side, s->num_cells_x));
        case COORD_SYS_CARTESIAN_2D:
            return WRAP_TRACEBACK(set_boundary_condition_cartesian_2d(
                p, s->density_, s->velocity_x_, s->velocity_y_, s->pressure_,
                s->num_ghost_cells_side, s->num_cells_x, s->num_cells_y));
        default:
            return WRAP_RAISE_ERROR(VALUE_ERROR, "Coordinate system flag not recognized.");
    }
}
