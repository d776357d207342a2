/*
 * step_control.h -- device-resident stepping state shared by the step kernels
 * and the host runtime.
 *
 * The reference's time loop (src/integrator_muscl_hancock.c:530-1160) needs t,
 * dt and the step count on the host every step.  Here they live in device
 * memory: every CTA of a step kernel derives the same dt from the previous
 * step's wave-speed maxima, and the last CTA to finish advances t and the
 * step count, decides whether stepping continues, and re-arms the maxima for
 * the step after next.  The host launches steps in chunks (optionally as a
 * CUDA graph) and only reads this block between chunks.
 */
#ifndef HYDRO_GPU_STEP_CONTROL_H
#define HYDRO_GPU_STEP_CONTROL_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct HydroStepControl {
    double t;                      /* simulation time after num_steps steps */
    double dt;                     /* dt of the last step attempted */
    long long num_steps;           /* completed steps */
    int active;                    /* 1 while steps should run */
    int snapshot_due;              /* 1: paused so the host can store a snapshot */
    int error_code;                /* first device error (hydro::DEV_ERR_*) */
    int error_cell;                /* padded index (or face) where it happened */
    unsigned int blocks_done;      /* last-CTA-done counter, reset every step */
    int work_next;                 /* next (strip, row chunk) item of the step, reset every step */
    int store_count;               /* snapshots stored so far (StoringParam.store_count_) */
    double tf;                     /* stop once t >= tf (the dt is clipped to it) */
    long long max_steps;           /* stop once num_steps reaches it; < 0: no limit */
    /* smax[k % 3] = ordered-bit maxima of (a+|u|, a+|v|) over the interior of
     * the state that step k starts from. */
    unsigned long long smax[3][2];
    /* bisect_marks[k]: exact Riemann solves whose bisection passed 500 (k+1)
     * iterations (the reference's verbose warnings; 1D runs only) */
    unsigned int bisect_marks[10];
} HydroStepControl;

/* Per-run stepping parameters (kernel arguments, constant for a run; the
 * stopping criteria live in HydroStepControl so the host can move them
 * between chunks without re-recording a graph). */
typedef struct HydroStepParams {
    double cfl;                    /* IntegratorParam.cfl */
    double cfl_shrunk;             /* cfl * cfl_initial_shrink_factor */
    long long shrink_steps;        /* cfl_initial_shrink_num_steps */
    int is_storing;
    int store_initial_offset;      /* 1 if the initial snapshot was stored */
    double storing_interval;
} HydroStepParams;

#ifdef __cplusplus
}
#endif

#endif
