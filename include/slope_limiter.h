/*
 * slope_limiter.h -- slope-limiter selection (reference: src/slope_limiter.h).
 */
#ifndef LIMITER_H
#define LIMITER_H

#include "common.h"

#ifdef __cplusplus
extern "C" {
#endif

#define SLOPE_LIMITER_MINMOD 1
#define SLOPE_LIMITER_VAN_LEER 2
#define SLOPE_LIMITER_MONOTONIZED_CENTRAL 3

ErrorStatus get_slope_limiter_flag(IntegratorParam *__restrict integrator_param);

ErrorStatus limit_slope(
    double *__restrict limited_slope,
    const IntegratorParam *__restrict integrator_param,
    const double slope_L,
    const double slope_R
);

#ifdef __cplusplus
}
#endif

#endif
