/*
 * source_term.c -- source terms (src/source_term.c).
 *
 * The gravity source of the 2D integrators is a no-op when gravity == 0
 * (src/source_term.c:195-198), which is every configuration this library
 * runs; a non-zero gravity and the cylindrical/spherical geometry source are
 * not available on the GPU path and report NOT_IMPLEMENTED_ERROR.
 */
#include "hydro.h"
#include "source_term.h"

ErrorStatus add_geometry_source_term(
    const BoundaryConditionParam *__restrict boundary_condition_param,
    System *__restrict system,
    const double dt
)
{
    (void) boundary_condition_param;
    (void) dt;
    if (system->coord_sys_flag_ == COORD_SYS_CARTESIAN_1D)
    {
        return make_success_error_status();
    }
    return WRAP_RAISE_ERROR(NOT_IMPLEMENTED_ERROR,
                            "The geometric source term (cylindrical / spherical grids) is not available on the GPU path.");
}

ErrorStatus add_gravity_source_term_2d(
    const BoundaryConditionParam *__restrict boundary_condition_param,
    System *__restrict system,
    const double dt
)
{
    (void) boundary_condition_param;
    (void) dt;
    if (system->gravity == 0.0)
    {
        return make_success_error_status();
    }
    return WRAP_RAISE_ERROR(NOT_IMPLEMENTED_ERROR, "A non-zero gravity source is not available on the GPU path.");
}
