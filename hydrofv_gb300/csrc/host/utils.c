/*
 * utils.c -- wall clock, sound speed and host CFL time step
 * (src/utils.c:16-95).  The GPU integrators compute the CFL maxima inside
 * the step kernel; these host versions serve set-up code and the exported API.
 */
#include <math.h>
#include <time.h>

#include "hydro.h"

double hydro_get_current_time(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double) ts.tv_sec + (double) ts.tv_nsec / 1.0e9;
}

double get_sound_speed(const double gamma, const double rho, const double p)
{
    return sqrt(gamma * p / rho);
}

double get_time_step_1d(const System *__restrict s, const double cfl)
{
    double smax = -INFINITY;
    for (int i = s->num_ghost_cells_side; i < s->num_cells_x + s->num_ghost_cells_side; i++)
    {
        const double a = get_sound_speed(s->gamma, s->density_[i], s->pressure_[i]);
        const double w = fabs(s->velocity_x_[i]);
        if (a + w > smax) smax = a + w;
    }
    return cfl * s->dx_ / smax;
}

double get_time_step_2d(const System *__restrict s, const double cfl)
{
    const int g = s->num_ghost_cells_side;
    const long long tx = s->num_cells_x + 2 * g;
    double sx = -INFINITY, sy = -INFINITY;
    for (int j = g; j < g + s->num_cells_y; j++)
    {
        for (int i = g; i < g + s->num_cells_x; i++)
        {
            const long long k = j * tx + i;
            const double a = get_sound_speed(s->gamma, s->density_[k], s->pressure_[k]);
            const double ax = a + fabs(s->velocity_x_[k]);
            const double ay = a + fabs(s->velocity_y_[k]);
            if (ax > sx) sx = ax;
            if (ay > sy) sy = ay;
        }
    }
    return cfl / (sx / s->dx_ + sy / s->dy_);
}
