/*
 * host_internal.h -- helpers shared by the host C files (not installed).
 */
#ifndef HYDRO_HOST_INTERNAL_H
#define HYDRO_HOST_INTERNAL_H

#include "hydro.h"

/* Ghost-cell count / coordinate-system / solver checks run by
 * launch_simulation before dispatch (src/hydro.c:93-265). */
ErrorStatus hydro_final_check(const System *system, const IntegratorParam *integrator_param);

/* ErrorStatus for a device error code (hydro::DEV_ERR_*), with the message
 * the reference raises for the same condition. */
ErrorStatus hydro_device_error_status(int code);

#endif
