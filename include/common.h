/*
 * common.h -- shared C99 types of the hydroFV-compatible API.
 *
 * Layouts are identical to the reference (src/common.h:18-69) so programs
 * written against hydroFV compile and link unchanged.
 */
#ifndef COMMON_H
#define COMMON_H

#include <stdbool.h>
#include <stdint.h>

/* Marks functions private to one translation unit (src/common.h:16). */
#define IN_FILE static

typedef int64_t int64;

/* Returned by value from every API function; `traceback` is heap-owned by
 * the caller and released with free_traceback / print_and_free_traceback. */
typedef struct ErrorStatus
{
    int return_code;
    char *traceback;
    int traceback_code_;
} ErrorStatus;

typedef struct IntegratorParam
{
    char *integrator;                 /* "muscl_hancock_2d", "godunov_first_order_1d", ... */
    char *riemann_solver;             /* "riemann_solver_hllc" / "riemann_solver_exact" */
    char *slope_limiter;              /* "minmod" / "van_leer" / "monotonized_central" */
    double cfl;
    double cfl_initial_shrink_factor;
    int cfl_initial_shrink_num_steps;
    double tol;
    int integrator_flag_;
    int riemann_solver_flag_;
    int slope_limiter_flag_;
} IntegratorParam;

typedef struct StoringParam
{
    char *output_dir;
    bool is_storing;
    bool store_initial;
    double storing_interval;
    int storing_method_flag_;
    int store_count_;
} StoringParam;

typedef struct Settings
{
    int verbose;
    bool no_progress_bar;
} Settings;

typedef struct SimulationParam
{
    double tf;
} SimulationParam;

typedef struct SimulationStatus
{
    int64 num_steps;
    double t;
    double dt;
} SimulationStatus;

#endif
