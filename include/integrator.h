/*
 * integrator.h -- integrator parameters and entry points (reference:
 * src/integrator.h).  In this library every integrator runs on the GPU.
 */
#ifndef INTEGRATOR_H
#define INTEGRATOR_H

#include "boundary.h"
#include "common.h"
#include "system.h"

#ifdef __cplusplus
extern "C" {
#endif

#define INTEGRATOR_RANDOM_CHOICE_1D 1
#define INTEGRATOR_GODUNOV_FIRST_ORDER_1D 2
#define INTEGRATOR_GODUNOV_FIRST_ORDER_2D 3
#define INTEGRATOR_GODUNOV_FIRST_ORDER_3D 4
#define INTEGRATOR_MUSCL_HANCOCK_1D 5
#define INTEGRATOR_MUSCL_HANCOCK_2D 6

/* Defaults: cfl 0.5, initial shrink 0.2 for 10 steps, tol 1e-6
 * (src/integrator.c:16-30). */
IntegratorParam get_new_integrator_param(void);

/* Resolve integrator / Riemann solver / limiter names and check the
 * numeric parameters (src/integrator.c:68-106). */
ErrorStatus finalize_integrator_param(IntegratorParam *__restrict integrator_param);

/* Dispatch on integrator_flag_ (src/integrator.c:108-143). */
ErrorStatus integrator_launch_simulation(
    BoundaryConditionParam *__restrict boundary_condition_param,
    System *__restrict system,
    IntegratorParam *__restrict integrator_param,
    StoringParam *__restrict storing_param,
    Settings *__restrict settings,
    SimulationParam *__restrict simulation_param,
    SimulationStatus *__restrict simulation_status
);

ErrorStatus random_choice_1d(
    BoundaryConditionParam *__restrict boundary_condition_param,
    System *__restrict system,
    IntegratorParam *__restrict integrator_param,
    StoringParam *__restrict storing_param,
    Settings *__restrict settings,
    SimulationParam *__restrict simulation_param,
    SimulationStatus *__restrict simulation_status
);

ErrorStatus godunov_first_order_1d(
    BoundaryConditionParam *__restrict boundary_condition_param,
    System *__restrict system,
    IntegratorParam *__restrict integrator_param,
    StoringParam *__restrict storing_param,
    Settings *__restrict settings,
    SimulationParam *__restrict simulation_param,
    SimulationStatus *__restrict simulation_status
);

ErrorStatus godunov_first_order_2d(
    BoundaryConditionParam *__restrict boundary_condition_param,
    System *__restrict system,
    IntegratorParam *__restrict integrator_param,
    StoringParam *__restrict storing_param,
    Settings *__restrict settings,
    SimulationParam *__restrict simulation_param,
    SimulationStatus *__restrict simulation_status
);

ErrorStatus muscl_hancock_1d(
    BoundaryConditionParam *__restrict boundary_condition_param,
    System *__restrict system,
    IntegratorParam *__restrict integrator_param,
    StoringParam *__restrict storing_param,
    Settings *__restrict settings,
    SimulationParam *__restrict simulation_param,
    SimulationStatus *__restrict simulation_status
);

ErrorStatus muscl_hancock_2d(
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
