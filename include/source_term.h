/*
 * source_term.h -- source terms (reference: src/source_term.h).
 */
#ifndef SOURCE_TERM_H
#define SOURCE_TERM_H

#include "hydro.h"

#ifdef __cplusplus
extern "C" {
#endif

ErrorStatus add_geometry_source_term(
    const BoundaryConditionParam *__restrict boundary_condition_param,
    System *__restrict system,
    const double dt
);

ErrorStatus add_gravity_source_term_2d(
    const BoundaryConditionParam *__restrict boundary_condition_param,
    System *__restrict system,
    const double dt
);

#ifdef __cplusplus
}
#endif

#endif
