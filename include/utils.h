/*
 * utils.h -- timing, sound speed and host CFL helpers (reference: src/utils.h).
 */
#ifndef UTILS_H
#define UTILS_H

#include "hydro.h"

#ifdef __cplusplus
extern "C" {
#endif

double hydro_get_current_time(void);
double get_sound_speed(double gamma, double rho, double p);
double get_time_step_1d(const System *__restrict system, const double cfl);
double get_time_step_2d(const System *__restrict system, const double cfl);

#ifdef __cplusplus
}
#endif

#endif
