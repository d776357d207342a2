/*
 * system.c -- System construction, geometry and host-side conversions.
 *
 * Semantics follow the reference (src/system.c): dx = (x_max - x_min) /
 * (N + 2G), i.e. the ghost cells lie inside [x_min, x_max] (:291-309); mid
 * points over the padded range (:318-356); 2D face areas A_x = dy, A_y = dx
 * and volume dx*dy (:365-529); conserved arrays are volume totals
 * (:849-917).  These routines run on the host during problem set-up; the
 * time loop itself never calls them.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "common.h"
#include "error.h"
#include "system.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

System get_new_system_struct(void)
{
    System s;
    memset(&s, 0, sizeof s);
    s.coord_sys = NULL;
    s.gamma = -1.0;
    s.gravity = 0.0;
    s.x_min = s.x_max = s.y_min = s.y_max = s.z_min = s.z_max = -1.0;
    s.num_cells_x = s.num_cells_y = s.num_cells_z = -1;
    s.num_ghost_cells_side = -1;
    s.coord_sys_flag_ = -1;
    s.dx_ = s.dy_ = s.dz_ = -1.0;
    return s;
}

static ErrorStatus coord_sys_flag(System *system)
{
    static const struct { const char *name; int flag; } table[] = {
        { "cartesian_1d", COORD_SYS_CARTESIAN_1D },
        { "cartesian_2d", COORD_SYS_CARTESIAN_2D },
        { "cartesian_3d", COORD_SYS_CARTESIAN_3D },
        { "cylindrical_1d", COORD_SYS_CYLINDRICAL_1D },
        { "spherical_1d", COORD_SYS_SPHERICAL_1D },
    };
    if (!system->coord_sys)
    {
        return WRAP_RAISE_ERROR(POINTER_ERROR, "Coordinate system pointer is NULL.");
    }
    for (size_t k = 0; k < sizeof table / sizeof table[0]; k++)
    {
        if (strcmp(system->coord_sys, table[k].name) == 0)
        {
            system->coord_sys_flag_ = table[k].flag;
            return make_success_error_status();
        }
    }
    return WRAP_RAISE_ERROR(VALUE_ERROR, "Coordinate system not recognized.");
}

static ErrorStatus value_errorf(const char *file, int line, const char *func, const char *fmt, ...)
    __attribute__((format(printf, 4, 5)));

#include <stdarg.h>
static ErrorStatus value_errorf(const char *file, int line, const char *func, const char *fmt, ...)
{
    char msg[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(msg, sizeof msg, fmt, ap);
    va_end(ap);
    return raise_error(VALUE_ERROR, msg, file, line, func);
}
#define VALUE_ERRORF(...) value_errorf(__FILE__, __LINE__, __func__, __VA_ARGS__)

/* Input checks of src/system.c:73-233. */
static ErrorStatus check_input(const System *s)
{
    if (!s->coord_sys)
    {
        return WRAP_RAISE_ERROR(VALUE_ERROR, "Coordinate system pointer is NULL.");
    }
    if (s->gamma < 1.0)
    {
        return VALUE_ERRORF("Gamma must be greater than 1. Got: %.3g", s->gamma);
    }
    const struct { const void *p; const char *msg; } arrays[] = {
        { s->density_, "Density array pointer (system->density_) is not NULL." },
        { s->velocity_x_, "Velocity (x-component) array pointer (system->velocity_x_) is not NULL." },
        { s->velocity_y_, "Velocity (y-component) array pointer (system->velocity_y_) is not NULL." },
        { s->velocity_z_, "Velocity (z-component) array pointer (system->velocity_z_) is not NULL." },
        { s->pressure_, "Pressure array pointer (system->pressure_) is not NULL." },
        { s->mass_, "Mass array pointer (system->mass_) is not NULL." },
        { s->momentum_x_, "Momentum (x-component) array pointer (system->momentum_x_) is not NULL." },
        { s->momentum_y_, "Momentum (y-component) array pointer (system->momentum_y_) is not NULL." },
        { s->momentum_z_, "Momentum (z-component) array pointer (system->momentum_z_) is not NULL." },
        { s->energy_, "Energy array pointer (system->energy_) is not NULL." },
        { s->mid_points_x_, "Mid points x array pointer (system->mid_points_x_) is not NULL." },
        { s->mid_points_y_, "Mid points y array pointer (system->mid_points_y_) is not NULL." },
        { s->mid_points_z_, "Mid points z array pointer (system->mid_points_z_) is not NULL." },
        { s->surface_area_x_, "Surface area x array pointer (system->surface_area_x_) is not NULL." },
        { s->surface_area_y_, "Surface area y array pointer (system->surface_area_y_) is not NULL." },
        { s->surface_area_z_, "Surface area z array pointer (system->surface_area_z_) is not NULL." },
        { s->volume_, "Volume array pointer (system->volume_) is not NULL." },
    };
    for (size_t k = 0; k < sizeof arrays / sizeof arrays[0]; k++)
    {
        if (arrays[k].p)
        {
            return WRAP_RAISE_ERROR(POINTER_ERROR, arrays[k].msg);
        }
    }
    if (s->num_ghost_cells_side < 1)
    {
        return VALUE_ERRORF("Number of ghost cells per side must be at least 1. Got: %d",
                            s->num_ghost_cells_side);
    }
    const int flag = s->coord_sys_flag_;
    if (flag == COORD_SYS_CARTESIAN_3D)
    {
        if (s->num_cells_z < 1)
            return VALUE_ERRORF("Number of cells in z-direction must be positive. Got: %d", s->num_cells_z);
        if (s->z_min >= s->z_max)
            return VALUE_ERRORF("z_min must be less than z_max. Got: z_min = %.3g, z_max = %.3g", s->z_min, s->z_max);
    }
    if (flag == COORD_SYS_CARTESIAN_3D || flag == COORD_SYS_CARTESIAN_2D)
    {
        if (s->num_cells_y < 1)
            return VALUE_ERRORF("Number of cells in y-direction must be positive. Got: %d", s->num_cells_y);
        if (s->y_min >= s->y_max)
            return VALUE_ERRORF("y_min must be less than y_max. Got: y_min = %.3g, y_max = %.3g", s->y_min, s->y_max);
    }
    if (flag < COORD_SYS_CARTESIAN_1D || flag > COORD_SYS_SPHERICAL_1D)
    {
        return WRAP_RAISE_ERROR(VALUE_ERROR, "Coordinate system flag not recognized.");
    }
    if (s->num_cells_x < 1)
        return VALUE_ERRORF("Number of cells in x-direction must be positive. Got: %d", s->num_cells_x);
    if (s->x_min >= s->x_max)
        return VALUE_ERRORF("x_min must be less than x_max. Got: x_min = %.3g, x_max = %.3g", s->x_min, s->x_max);
    return make_success_error_status();
}

static void release_arrays(System *s)
{
    double **arrays[] = {
        &s->density_, &s->velocity_x_, &s->velocity_y_, &s->velocity_z_, &s->pressure_,
        &s->mass_, &s->momentum_x_, &s->momentum_y_, &s->momentum_z_, &s->energy_,
        &s->mid_points_x_, &s->mid_points_y_, &s->mid_points_z_,
        &s->surface_area_x_, &s->surface_area_y_, &s->surface_area_z_, &s->volume_,
    };
    for (size_t k = 0; k < sizeof arrays / sizeof arrays[0]; k++)
    {
        free(*arrays[k]);
        *arrays[k] = NULL;
    }
}

/* Geometry of src/system.c:291-529. */
static void init_geometry(System *s)
{
    const int g = s->num_ghost_cells_side;
    const int tx = s->num_cells_x + 2 * g;
    const int flag = s->coord_sys_flag_;
    if (flag == COORD_SYS_CARTESIAN_3D)
        s->dz_ = (s->z_max - s->z_min) / (s->num_cells_z + 2 * g);
    if (flag == COORD_SYS_CARTESIAN_3D || flag == COORD_SYS_CARTESIAN_2D)
        s->dy_ = (s->y_max - s->y_min) / (s->num_cells_y + 2 * g);
    s->dx_ = (s->x_max - s->x_min) / (s->num_cells_x + 2 * g);

    if (flag == COORD_SYS_CARTESIAN_3D)
    {
        const int tz = s->num_cells_z + 2 * g;
        for (int i = 0; i < tz; i++) s->mid_points_z_[i] = s->z_min + (i + 0.5) * s->dz_;
    }
    if (flag == COORD_SYS_CARTESIAN_3D || flag == COORD_SYS_CARTESIAN_2D)
    {
        const int ty = s->num_cells_y + 2 * g;
        for (int i = 0; i < ty; i++) s->mid_points_y_[i] = s->y_min + (i + 0.5) * s->dy_;
    }
    for (int i = 0; i < tx; i++) s->mid_points_x_[i] = s->x_min + (i + 0.5) * s->dx_;

    switch (flag)
    {
        case COORD_SYS_CARTESIAN_1D:
            for (int i = 0; i < tx + 1; i++) s->surface_area_x_[i] = 1.0;
            for (int i = 0; i < tx; i++) s->volume_[i] = s->dx_;
            break;
        case COORD_SYS_CYLINDRICAL_1D:
            for (int i = 1; i < tx + 1; i++)
            {
                const double r = s->x_min + i * s->dx_;
                s->surface_area_x_[i] = 2.0 * M_PI * r;
            }
            for (int i = 0; i < tx; i++)
            {
                const double r0 = s->x_min + i * s->dx_;
                const double r1 = s->x_min + (i + 1) * s->dx_;
                s->volume_[i] = M_PI * (r1 * r1 - r0 * r0);
            }
            break;
        case COORD_SYS_SPHERICAL_1D:
            for (int i = 0; i < tx + 1; i++)
            {
                const double r = s->x_min + i * s->dx_;
                s->surface_area_x_[i] = 4.0 * M_PI * r * r;
            }
            for (int i = 0; i < tx; i++)
            {
                const double r0 = s->x_min + i * s->dx_;
                const double r1 = s->x_min + (i + 1) * s->dx_;
                s->volume_[i] = (4.0 / 3.0) * M_PI * (r1 * r1 * r1 - r0 * r0 * r0);
            }
            break;
        case COORD_SYS_CARTESIAN_2D:
        {
            const int ty = s->num_cells_y + 2 * g;
            for (int i = 0; i < tx; i++) s->surface_area_x_[i] = s->dy_;
            for (int j = 0; j < ty; j++) s->surface_area_y_[j] = s->dx_;
            const double v = s->dx_ * s->dy_;
            for (long long k = 0; k < (long long) tx * ty; k++) s->volume_[k] = v;
            break;
        }
        case COORD_SYS_CARTESIAN_3D:
        {
            const int ty = s->num_cells_y + 2 * g;
            const int tz = s->num_cells_z + 2 * g;
            for (int i = 0; i < tx; i++) s->surface_area_x_[i] = s->dy_ * s->dz_;
            for (int i = 0; i < ty; i++) s->surface_area_y_[i] = s->dx_ * s->dz_;
            for (int i = 0; i < tz; i++) s->surface_area_z_[i] = s->dx_ * s->dy_;
            const double v = s->dx_ * s->dy_ * s->dz_;
            for (long long k = 0; k < (long long) tx * ty * tz; k++) s->volume_[k] = v;
            break;
        }
        default:
            break;
    }
}

ErrorStatus system_init(System *__restrict system)
{
    ErrorStatus e = WRAP_TRACEBACK(coord_sys_flag(system));
    if (e.return_code != SUCCESS) return e;
    e = WRAP_TRACEBACK(check_input(system));
    if (e.return_code != SUCCESS) return e;

    const int g = system->num_ghost_cells_side;
    const int flag = system->coord_sys_flag_;
    const long long tx = system->num_cells_x + 2LL * g;
    const long long ty = (flag == COORD_SYS_CARTESIAN_2D || flag == COORD_SYS_CARTESIAN_3D)
                             ? system->num_cells_y + 2LL * g : 1;
    const long long tz = (flag == COORD_SYS_CARTESIAN_3D) ? system->num_cells_z + 2LL * g : 1;
    const long long total = tx * ty * tz;
    /* The reference indexes with 32-bit int (src/system.c:550-572). */
    if (total > 2147483647LL)
    {
        return WRAP_RAISE_ERROR(VALUE_ERROR, "Total number of cells exceeds the 32-bit index range.");
    }
    const size_t n = (size_t) total;

    system->density_ = calloc(n, sizeof(double));
    system->pressure_ = calloc(n, sizeof(double));
    system->mass_ = calloc(n, sizeof(double));
    system->energy_ = calloc(n, sizeof(double));
    system->volume_ = malloc(n * sizeof(double));
    system->velocity_x_ = calloc(n, sizeof(double));
    system->momentum_x_ = calloc(n, sizeof(double));
    system->mid_points_x_ = malloc((size_t) tx * sizeof(double));
    system->surface_area_x_ = malloc((size_t) (tx + 1) * sizeof(double));
    int ok = system->density_ && system->pressure_ && system->mass_ && system->energy_ &&
             system->volume_ && system->velocity_x_ && system->momentum_x_ &&
             system->mid_points_x_ && system->surface_area_x_;
    if (ty > 1 || flag == COORD_SYS_CARTESIAN_2D || flag == COORD_SYS_CARTESIAN_3D)
    {
        system->velocity_y_ = calloc(n, sizeof(double));
        system->momentum_y_ = calloc(n, sizeof(double));
        system->mid_points_y_ = malloc((size_t) ty * sizeof(double));
        system->surface_area_y_ = malloc((size_t) (ty + 1) * sizeof(double));
        ok = ok && system->velocity_y_ && system->momentum_y_ && system->mid_points_y_ &&
             system->surface_area_y_;
    }
    if (flag == COORD_SYS_CARTESIAN_3D)
    {
        system->velocity_z_ = calloc(n, sizeof(double));
        system->momentum_z_ = calloc(n, sizeof(double));
        system->mid_points_z_ = malloc((size_t) tz * sizeof(double));
        system->surface_area_z_ = malloc((size_t) (tz + 1) * sizeof(double));
        ok = ok && system->velocity_z_ && system->momentum_z_ && system->mid_points_z_ &&
             system->surface_area_z_;
    }
    if (!ok)
    {
        release_arrays(system);
        return WRAP_RAISE_ERROR(MEMORY_ERROR, "Memory allocation failed.");
    }
    init_geometry(system);
    return make_success_error_status();
}

void free_system_memory(System *__restrict system)
{
    release_arrays(system);
}

/* src/system.c:735-761 */
void convert_conserved_to_primitive_1d(
    const int num_cells_x,
    const int num_ghost_cells_side,
    const double gamma,
    const double *__restrict volume,
    const double *__restrict mass,
    const double *__restrict momentum_x,
    const double *__restrict energy,
    double *__restrict density,
    double *__restrict velocity_x,
    double *__restrict pressure
)
{
    for (int i = 0; i < num_cells_x + 2 * num_ghost_cells_side; i++)
    {
        const double m = mass[i];
        density[i] = m / volume[i];
        velocity_x[i] = momentum_x[i] / m;
        pressure[i] = (gamma - 1.0) * (energy[i] - 0.5 * m * velocity_x[i] * velocity_x[i]) / volume[i];
    }
}

/* src/system.c:763-802 */
void convert_conserved_to_primitive_2d(
    const int num_cells_x,
    const int num_cells_y,
    const int num_ghost_cells_side,
    const double gamma,
    const double *__restrict volume,
    const double *__restrict mass,
    const double *__restrict momentum_x,
    const double *__restrict momentum_y,
    const double *__restrict energy,
    double *__restrict density,
    double *__restrict velocity_x,
    double *__restrict velocity_y,
    double *__restrict pressure
)
{
    const long long n = (long long) (num_cells_x + 2 * num_ghost_cells_side)
                      * (num_cells_y + 2 * num_ghost_cells_side);
    for (long long k = 0; k < n; k++)
    {
        const double m = mass[k];
        density[k] = m / volume[k];
        velocity_x[k] = momentum_x[k] / m;
        velocity_y[k] = momentum_y[k] / m;
        pressure[k] = (gamma - 1.0) * (energy[k] - 0.5 * m * (velocity_x[k] * velocity_x[k]
                                                             + velocity_y[k] * velocity_y[k])) / volume[k];
    }
}

ErrorStatus convert_conserved_to_primitive(System *__restrict system)
{
    switch (system->coord_sys_flag_)
    {
        case COORD_SYS_CARTESIAN_1D:
        case COORD_SYS_CYLINDRICAL_1D:
        case COORD_SYS_SPHERICAL_1D:
            convert_conserved_to_primitive_1d(system->num_cells_x, system->num_ghost_cells_side,
                                              system->gamma, system->volume_, system->mass_,
                                              system->momentum_x_, system->energy_, system->density_,
                                              system->velocity_x_, system->pressure_);
            return make_success_error_status();
        case COORD_SYS_CARTESIAN_2D:
            convert_conserved_to_primitive_2d(system->num_cells_x, system->num_cells_y,
                                              system->num_ghost_cells_side, system->gamma,
                                              system->volume_, system->mass_, system->momentum_x_,
                                              system->momentum_y_, system->energy_, system->density_,
                                              system->velocity_x_, system->velocity_y_, system->pressure_);
            return make_success_error_status();
        case COORD_SYS_CARTESIAN_3D:
            return WRAP_RAISE_ERROR(NOT_IMPLEMENTED_ERROR, "");
        default:
            return WRAP_RAISE_ERROR(VALUE_ERROR, "Coordinate system flag not recognized.");
    }
}

/* src/system.c:849-917 */
ErrorStatus convert_primitive_to_conserved(System *__restrict system)
{
    const int g = system->num_ghost_cells_side;
    const double gamma = system->gamma;
    switch (system->coord_sys_flag_)
    {
        case COORD_SYS_CARTESIAN_1D:
        case COORD_SYS_CYLINDRICAL_1D:
        case COORD_SYS_SPHERICAL_1D:
            for (int i = 0; i < system->num_cells_x + 2 * g; i++)
            {
                const double rho = system->density_[i];
                const double u = system->velocity_x_[i];
                const double vol = system->volume_[i];
                system->mass_[i] = rho * vol;
                system->momentum_x_[i] = system->mass_[i] * u;
                system->energy_[i] = vol * (0.5 * rho * u * u + system->pressure_[i] / (gamma - 1.0));
            }
            return make_success_error_status();
        case COORD_SYS_CARTESIAN_2D:
        {
            const long long n = (long long) (system->num_cells_x + 2 * g) * (system->num_cells_y + 2 * g);
            for (long long k = 0; k < n; k++)
            {
                const double rho = system->density_[k];
                const double u = system->velocity_x_[k];
                const double v = system->velocity_y_[k];
                const double vol = system->volume_[k];
                system->mass_[k] = rho * vol;
                system->momentum_x_[k] = system->mass_[k] * u;
                system->momentum_y_[k] = system->mass_[k] * v;
                system->energy_[k] = vol * (0.5 * rho * (u * u + v * v) + system->pressure_[k] / (gamma - 1.0));
            }
            return make_success_error_status();
        }
        case COORD_SYS_CARTESIAN_3D:
            return WRAP_RAISE_ERROR(NOT_IMPLEMENTED_ERROR, "");
        default:
            return WRAP_RAISE_ERROR(VALUE_ERROR, "Coordinate system flag not recognized.");
    }
}
