/*
 * gpu_bridge.h -- C interface between the host C layer (parameter handling,
 * validation, error tracebacks, storing) and the CUDA runtime.  Internal to
 * the library; programs use hydro.h / hydro_gpu.h.
 */
#ifndef HYDRO_GPU_BRIDGE_H
#define HYDRO_GPU_BRIDGE_H

#include "hydro_gpu.h"
#include "step_control.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Outcome kinds of a bridge call. */
#define HYDRO_RUN_OK 0
#define HYDRO_RUN_DEVICE_ERROR 1    /* numerical error raised by a kernel (code = DEV_ERR_*) */
#define HYDRO_RUN_CUDA_ERROR 2      /* CUDA runtime error (code = cudaError_t) */
#define HYDRO_RUN_CALLBACK_ERROR 3  /* snapshot callback failed (code = its return value) */
#define HYDRO_RUN_UNSUPPORTED 4     /* combination not available on the GPU path */

typedef struct HydroRunOutcome
{
    int64 num_steps;
    double t;
    double dt;
    int store_count;
    int kind;
    int code;
    int where;
    char message[256];
    /* exact Riemann solves whose bisection passed 500 (k+1) iterations
     * (HydroStepControl.bisect_marks of a 1D run) */
    unsigned int bisect_marks[10];
} HydroRunOutcome;

/* A 2D Cartesian problem as the kernels see it. */
typedef struct HydroGrid2D
{
    int nx, ny, g;
    double gamma, tol;
    double dx, dy;                /* System.dx_, dy_ */
    double area_x, area_y, vol;   /* uniform face areas and cell volume */
    int bc[4];                    /* BOUNDARY_CONDITION_* of x_min, x_max, y_min, y_max */
    int limiter;                  /* SLOPE_LIMITER_* */
    int integrator;               /* INTEGRATOR_MUSCL_HANCOCK_2D or INTEGRATOR_GODUNOV_FIRST_ORDER_2D */
    double gravity;               /* System.gravity (0: no source term) */
} HydroGrid2D;

/* Host boundary routine for custom sides: receives the padded W arrays
 * (host memory) holding U->W of every cell after a step, applies the
 * boundary conditions in place; returns 0 on success. */
typedef int (*HydroHostBcFn)(void *ctx, double *const W[4]);

/* Called when a snapshot is due; W holds the padded primitive arrays
 * (host memory, valid for the duration of the call).  Returns 0 on success. */
typedef int (*HydroSnapshotFn)(void *ctx, double *const W[4], int64 num_steps, double t, double dt);

typedef struct HydroRun2D HydroRun2D;

int hydro_run2d_create(const HydroGrid2D *grid, const HydroGpuOptions *opt,
                       HydroRun2D **out, HydroRunOutcome *oc);
/* Upload W and U (padded host arrays); keep_initial keeps a device copy for
 * hydro_run2d_restore. */
int hydro_run2d_upload(HydroRun2D *run, double *const W[4], double *const U[4],
                       int keep_initial, HydroRunOutcome *oc);
int hydro_run2d_restore(HydroRun2D *run, HydroRunOutcome *oc);
/* Custom (callback) sides: after every step the state is converted and
 * handed to `fn`; the ghost bands of the sides whose BC is custom are then
 * copied back (FP64 only). */
int hydro_run2d_set_host_bc(HydroRun2D *run, HydroHostBcFn fn, void *ctx, HydroRunOutcome *oc);
/* Start a run at t = 0 from the uploaded state. */
int hydro_run2d_begin(HydroRun2D *run, const HydroStepParams *sp, double tf, int64 max_steps,
                      int store_count, HydroRunOutcome *oc);
/* Current step count / time of a begun run. */
int hydro_run2d_status(HydroRun2D *run, HydroRunOutcome *oc);
/* Move the stopping criteria of a begun run (t and the step count keep going). */
int hydro_run2d_set_limits(HydroRun2D *run, double tf, int64 max_steps, HydroRunOutcome *oc);
/* Step until the run stops (tf, step limit or error), storing snapshots
 * through `snap` when due.  step_ms (may be NULL) receives the CUDA-event
 * time of the stepping. */
int hydro_run2d_advance(HydroRun2D *run, HydroSnapshotFn snap, void *ctx,
                        HydroRunOutcome *oc, double *step_ms);
/* Full padded W (ghosts filled) and U of the current state into host arrays. */
int hydro_run2d_download(HydroRun2D *run, double *const W[4], double *const U[4],
                         HydroRunOutcome *oc);
/* Conserved totals (mass, mom_x, mom_y, energy) over the interior of the
 * current state, summed in FP64 with Neumaier compensation. */
int hydro_run2d_totals(HydroRun2D *run, double totals[4], HydroRunOutcome *oc);
void hydro_run2d_stats(const HydroRun2D *run, HydroGpuStats *stats);
void hydro_run2d_destroy(HydroRun2D *run);

/* Ensembles of independent 2D grids stepped by one launch per step. */
typedef struct HydroBatch2D HydroBatch2D;
int hydro_batch2d_create(const HydroGrid2D *grids, int n, const HydroGpuOptions *opt,
                         HydroBatch2D **out, HydroRunOutcome *oc);
int hydro_batch2d_upload(HydroBatch2D *b, int i, double *const W[4], double *const U[4],
                         HydroRunOutcome *oc);
int hydro_batch2d_restore(HydroBatch2D *b, HydroRunOutcome *oc);
int hydro_batch2d_begin(HydroBatch2D *b, const HydroStepParams *sp, double tf, int64 max_steps,
                        HydroRunOutcome *oc);
/* Every instance: stop at tf or after max_steps_more further steps. */
int hydro_batch2d_set_limits(HydroBatch2D *b, double tf, int64 max_steps_more, HydroRunOutcome *oc);
int hydro_batch2d_advance(HydroBatch2D *b, HydroRunOutcome *oc, double *step_ms);
int hydro_batch2d_status(HydroBatch2D *b, int i, HydroRunOutcome *oc);
int hydro_batch2d_download(HydroBatch2D *b, int i, double *const W[4], double *const U[4],
                           HydroRunOutcome *oc);
void hydro_batch2d_stats(const HydroBatch2D *b, HydroGpuStats *stats);
void hydro_batch2d_destroy(HydroBatch2D *b);

/* Discrete adjoint / tangent-linear session of the 2D MUSCL-Hancock step. */
typedef struct HydroAdj2D HydroAdj2D;
int hydro_adj2d_create(const HydroGrid2D *grid, const HydroGpuOptions *opt, const HydroStepParams *sp,
                       int64 num_steps, int checkpoint_every, double *const W0[4],
                       HydroAdj2D **out, HydroRunOutcome *oc);
int hydro_adj2d_forward(HydroAdj2D *a, double *const W[4], double *const U[4], HydroRunOutcome *oc);
int hydro_adj2d_backward(HydroAdj2D *a, double *const seed[4], double *const grad[4], HydroRunOutcome *oc);
int hydro_adj2d_tangent(HydroAdj2D *a, double *const w0[4], double *const dw0[4],
                        double *const wN[4], double *const dwN[4], HydroRunOutcome *oc);
int hydro_adj2d_replay(HydroAdj2D *a, double *const w0[4], double *const wN[4],
                       unsigned long long *signatures, int frozen, HydroRunOutcome *oc);
int hydro_adj2d_dt(const HydroAdj2D *a, double *dt);
void hydro_adj2d_set_tape(HydroAdj2D *a, int enabled);
void hydro_adj2d_stats(const HydroAdj2D *a, HydroGpuAdjointStats *st);
void hydro_adj2d_destroy(HydroAdj2D *a);

/* 1D Cartesian problem (Godunov first order or MUSCL-Hancock). */
typedef struct HydroGrid1D
{
    int nx, g;
    double gamma, tol, dx;
    const double *area;           /* System.surface_area_x_ (nx + 2G + 1 entries) */
    const double *vol;            /* System.volume_ (nx + 2G) */
    const double *mid;            /* System.mid_points_x_ (nx + 2G) */
    double alpha;                 /* geometry source: 0 Cartesian, 1 cylindrical, 2 spherical */
    int bc[2];
    int limiter;
    int riemann_solver;           /* RIEMANN_SOLVER_* */
    int integrator;               /* INTEGRATOR_{RANDOM_CHOICE,GODUNOV_FIRST_ORDER,MUSCL_HANCOCK}_1D */
} HydroGrid1D;

/* Whole 1D run in one launch (W, U: padded host arrays, in/out). */
int hydro_run1d(const HydroGrid1D *grid, double *const W[3], double *const U[3],
                const HydroStepParams *sp, double tf, int64 max_steps, int store_count,
                HydroSnapshotFn snap, void *ctx, const HydroGpuOptions *opt,
                HydroRunOutcome *oc, HydroGpuStats *stats);

#ifdef __cplusplus
}
#endif

#endif
