/*
 * hydro.h -- umbrella header of the hydroFV-compatible API (reference:
 * src/hydro.h).  Programs written for hydroFV include this header and link
 * against libhydro_gb300 (or the static `hydro` target) unchanged; the time
 * loop behind launch_simulation runs on a GB300 GPU.
 */
#ifndef HYDRO_H
#define HYDRO_H

#include "boundary.h"
#include "common.h"
#include "error.h"
#include "integrator.h"
#include "riemann_solver.h"
#include "slope_limiter.h"
#include "storing.h"
#include "system.h"
#include "utils.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Finalize parameters, validate, and run the simulation to tf
 * (src/hydro.h:53-61, src/hydro.c:29-91). */
ErrorStatus launch_simulation(
    BoundaryConditionParam *__restrict boundary_condition_param,
    System *__restrict system,
    IntegratorParam *__restrict integrator_param,
    StoringParam *__restrict storing_param,
    Settings *__restrict settings,
    SimulationParam *__restrict simulation_param,
    SimulationStatus *__restrict simulation_status
);

#ifdef __cplusplus
}
#endif

#endif
