/*
 * storing.h -- snapshot storing (reference: src/storing.h).
 */
#ifndef STORING_H
#define STORING_H

#include "common.h"
#include "system.h"

#ifdef __cplusplus
extern "C" {
#endif

StoringParam get_new_storing_param(void);
ErrorStatus finalize_storing_param(StoringParam *__restrict storing_param);

ErrorStatus store_snapshot(
    const BoundaryConditionParam *__restrict boundary_condition_param,
    const System *__restrict system,
    const IntegratorParam *__restrict integrator_param,
    const SimulationStatus *__restrict simulation_status,
    StoringParam *__restrict storing_param
);

#ifdef __cplusplus
}
#endif

#endif
