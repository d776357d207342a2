/*
 * system.h -- the hydrodynamic system and its host arrays (reference:
 * src/system.h).  All arrays are padded with num_ghost_cells_side ghost cells
 * per side, row-major with index j * (num_cells_x + 2G) + i.  Conserved
 * arrays hold volume-integrated totals (mass = rho * volume, ...).
 */
#ifndef SYSTEM_H
#define SYSTEM_H

#include "common.h"

#ifdef __cplusplus
extern "C" {
#endif

#define COORD_SYS_CARTESIAN_1D 1
#define COORD_SYS_CARTESIAN_2D 2
#define COORD_SYS_CARTESIAN_3D 3
#define COORD_SYS_CYLINDRICAL_1D 4
#define COORD_SYS_SPHERICAL_1D 5

typedef struct System
{
    const char *coord_sys;
    double gamma;
    double gravity;
    double x_min;
    double x_max;
    double y_min;
    double y_max;
    double z_min;
    double z_max;
    int num_cells_x;
    int num_cells_y;
    int num_cells_z;
    int num_ghost_cells_side;

    int coord_sys_flag_;
    double dx_;
    double dy_;
    double dz_;
    double *density_;
    double *velocity_x_;
    double *velocity_y_;
    double *velocity_z_;
    double *pressure_;
    double *mass_;
    double *momentum_x_;
    double *momentum_y_;
    double *momentum_z_;
    double *energy_;
    double *mid_points_x_;
    double *mid_points_y_;
    double *mid_points_z_;
    double *surface_area_x_;
    double *surface_area_y_;
    double *surface_area_z_;
    double *volume_;
} System;

/* A System with every field unset (src/system.c:23-64). */
System get_new_system_struct(void);

/* Validate inputs, allocate the host arrays and fill the geometry
 * (src/system.c:531-712). */
ErrorStatus system_init(System *__restrict system);

/* Release the arrays allocated by system_init (src/system.c:714-733). */
void free_system_memory(System *__restrict system);

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
);

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
);

ErrorStatus convert_conserved_to_primitive(System *__restrict system);
ErrorStatus convert_primitive_to_conserved(System *__restrict system);

#ifdef __cplusplus
}
#endif

#endif
