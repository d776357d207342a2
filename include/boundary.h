/*
 * boundary.h -- boundary-condition selection and host ghost fill
 * (reference: src/boundary.h).
 */
#ifndef BOUNDARY_H
#define BOUNDARY_H

#include "common.h"
#include "system.h"

#ifdef __cplusplus
extern "C" {
#endif

/* User ghost-fill callbacks operating on the host primitive arrays. */
typedef void (*set_boundary_condition_1d_func)(
    double *__restrict density,
    double *__restrict velocity_x,
    double *__restrict pressure,
    const int num_ghost_cells_side,
    const int num_cells_x
);

typedef void (*set_boundary_condition_cartesian_2d_func)(
    double *__restrict density,
    double *__restrict velocity_x,
    double *__restrict velocity_y,
    double *__restrict pressure,
    const int num_ghost_cells_side,
    const int num_cells_x,
    const int num_cells_y
);

typedef struct BoundaryConditionParam
{
    const char *boundary_condition_x_min;
    const char *boundary_condition_x_max;
    const char *boundary_condition_y_min;
    const char *boundary_condition_y_max;
    const char *boundary_condition_z_min;
    const char *boundary_condition_z_max;
    set_boundary_condition_1d_func set_boundary_condition_1d_x_min;
    set_boundary_condition_1d_func set_boundary_condition_1d_x_max;
    set_boundary_condition_cartesian_2d_func set_boundary_condition_cartesian_2d_x_min;
    set_boundary_condition_cartesian_2d_func set_boundary_condition_cartesian_2d_x_max;
    set_boundary_condition_cartesian_2d_func set_boundary_condition_cartesian_2d_y_min;
    set_boundary_condition_cartesian_2d_func set_boundary_condition_cartesian_2d_y_max;

    int boundary_condition_flag_x_min_;
    int boundary_condition_flag_x_max_;
    int boundary_condition_flag_y_min_;
    int boundary_condition_flag_y_max_;
    int boundary_condition_flag_z_min_;
    int boundary_condition_flag_z_max_;
} BoundaryConditionParam;

#define BOUNDARY_CONDITION_NONE 1
#define BOUNDARY_CONDITION_REFLECTIVE 2
#define BOUNDARY_CONDITION_TRANSMISSIVE 3
#define BOUNDARY_CONDITION_PERIODIC 4
#define BOUNDARY_CONDITION_CUSTOM 5

BoundaryConditionParam get_new_boundary_condition_param(void);

/* Resolve the boundary-condition names to flags (src/boundary.c:391-409). */
ErrorStatus finalize_boundary_condition_param(
    const System *__restrict system,
    BoundaryConditionParam *__restrict boundary_condition_param
);

/* Fill the host ghost cells of the primitive arrays (src/boundary.c:792-824). */
ErrorStatus set_boundary_condition(
    const BoundaryConditionParam *__restrict boundary_condition_param,
    System *__restrict system
);

ErrorStatus set_boundary_condition_1d(
    const BoundaryConditionParam *__restrict boundary_condition_param,
    double *__restrict density,
    double *__restrict velocity_x,
    double *__restrict pressure,
    const int num_ghost_cells_side,
    const int num_cells_x
);

ErrorStatus set_boundary_condition_cartesian_2d(
    const BoundaryConditionParam *__restrict boundary_condition_param,
    double *__restrict density,
    double *__restrict velocity_x,
    double *__restrict velocity_y,
    double *__restrict pressure,
    const int num_ghost_cells_side,
    const int num_cells_x,
    const int num_cells_y
);

#ifdef __cplusplus
}
#endif

#endif
