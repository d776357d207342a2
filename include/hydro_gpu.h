/*
 * hydro_gpu.h -- GB300 extensions to the hydroFV-compatible C API.
 *
 * Everything in hydro.h keeps the reference's semantics; launch_simulation
 * itself runs on the GPU.  This header adds what the reference has no way to
 * express:
 *
 *   - HydroGpuOptions: device, fixed step count, precision, chunking;
 *   - hydro_gpu_launch_simulation: launch_simulation with options and
 *     device-timed statistics (H2D / stepping / D2H, bytes moved, launches);
 *   - HydroGpuSolver: a device-resident session (upload once, step many
 *     times, download when asked) for benchmarks and drivers that keep the
 *     state in HBM between calls.
 *
 * No struct declared in hydro.h changes layout.  All functions are C ABI,
 * take plain pointers and sizes, and return ErrorStatus like the rest of
 * the API.
 */
#ifndef HYDRO_GPU_H
#define HYDRO_GPU_H

#include "hydro.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Arithmetic of the 2D step. */
#define HYDRO_GPU_PRECISION_FP64 0   /* the drop-in: matches the reference */
#define HYDRO_GPU_PRECISION_FP32 1   /* FP32 state/flux, FP64 where needed */

typedef struct HydroGpuOptions
{
    int device;             /* CUDA device ordinal (default 0) */
    int64 max_steps;        /* stop after this many steps; < 0: run to tf only */
    int precision;          /* HYDRO_GPU_PRECISION_* (default FP64) */
    int chunk_steps;        /* steps enqueued between host polls (0: auto) */
    int use_graph;          /* replay step chunks as CUDA graphs (default 1) */
    int block_threads;      /* threads per step CTA (0: tuned default) */
    int chunk_rows;         /* grid rows per step work item (0: chosen from the grid shape and the resident CTAs) */
    int autotune;           /* 1: before the first step, time candidate work-item
                               shapes and persistent grid sizes on the actual
                               state (then rewind) and keep the fastest; cached
                               per shape for the process */
    int sync_snapshots;     /* 0 (default, 2D): a snapshot is copied to the host on a
                               side stream and written by a host thread while the
                               steps go on; a write error is reported at the next
                               snapshot or at the end of the run.  1: stepping
                               waits for each write (the reference's behaviour:
                               a failed write stops the run at that step). */
} HydroGpuOptions;

typedef struct HydroGpuStats
{
    double total_ms;        /* host wall clock of the whole call */
    double h2d_ms;          /* CUDA-event time of host -> device staging */
    double step_ms;         /* CUDA-event time of the stepping phase */
    double d2h_ms;          /* CUDA-event time of the final device -> host copies */
    int64 steps;            /* completed time steps */
    int64 step_launches;    /* step kernels launched (no-op tail launches included) */
    int64 kernel_launches;  /* every kernel of this library launched by the call */
    int64 h2d_bytes;
    int64 d2h_bytes;
    int64 interior_cells;   /* cells updated per step */
} HydroGpuStats;

/* Defaults: device 0, no step limit, FP64, auto chunking, graphs on, no autotuning. */
HydroGpuOptions hydro_gpu_default_options(void);

/* Options used by plain launch_simulation() in this process.  Lets programs
 * written for hydroFV pick a device or a step limit without code changes
 * (the environment variables HYDRO_GPU_DEVICE and HYDRO_GPU_MAX_STEPS are
 * read when this has not been called).  Not thread-safe against concurrent
 * calls of itself. */
void hydro_gpu_set_process_options(const HydroGpuOptions *options);

/* launch_simulation with explicit options; `stats` may be NULL. */
ErrorStatus hydro_gpu_launch_simulation(
    BoundaryConditionParam *__restrict boundary_condition_param,
    System *__restrict system,
    IntegratorParam *__restrict integrator_param,
    StoringParam *__restrict storing_param,
    Settings *__restrict settings,
    SimulationParam *__restrict simulation_param,
    SimulationStatus *__restrict simulation_status,
    const HydroGpuOptions *options,
    HydroGpuStats *stats
);

/* ------------------------------------------------------------------ */
/* Device-resident session (2D Cartesian MUSCL-Hancock / Godunov).     */
/* ------------------------------------------------------------------ */

typedef struct HydroGpuSolver HydroGpuSolver;

/* Finalize the parameters, allocate device memory and upload the System's
 * W and U arrays.  The initial state is also kept on the device so
 * hydro_gpu_solver_restart can rewind without host traffic. */
ErrorStatus hydro_gpu_solver_create(
    HydroGpuSolver **solver,
    BoundaryConditionParam *__restrict boundary_condition_param,
    System *__restrict system,
    IntegratorParam *__restrict integrator_param,
    const HydroGpuOptions *options
);

/* Rewind to the uploaded initial state (t = 0, no steps taken). */
ErrorStatus hydro_gpu_solver_restart(HydroGpuSolver *solver);

/* Advance by up to `num_steps` steps, stopping early at tf.  `status`
 * receives num_steps / t / dt since the last restart; `step_ms` (may be
 * NULL) the CUDA-event time of this call's stepping. */
ErrorStatus hydro_gpu_solver_advance(
    HydroGpuSolver *solver,
    int64 num_steps,
    double tf,
    SimulationStatus *__restrict status,
    double *step_ms
);

/* Copy the current state (W with ghost cells filled, and U) into the
 * System's host arrays. */
ErrorStatus hydro_gpu_solver_download(HydroGpuSolver *solver, System *__restrict system);

/* Conserved totals (mass, momentum_x, momentum_y, energy) over the interior
 * of the current state, summed on the device in FP64 with Neumaier
 * compensation (drift diagnostics for either precision). */
ErrorStatus hydro_gpu_solver_conserved_totals(HydroGpuSolver *solver, double totals[4]);

/* Kernels launched by this solver so far. */
int64 hydro_gpu_solver_kernel_launches(const HydroGpuSolver *solver);

void hydro_gpu_solver_destroy(HydroGpuSolver *solver);

/* ------------------------------------------------------------------ */
/* Batched ensembles of independent 2D grids.                          */
/* ------------------------------------------------------------------ */

typedef struct HydroGpuBatch HydroGpuBatch;

/* n independent 2D problems (systems[i] with boundary conditions bcps[i];
 * one integrator / Riemann solver / limiter / CFL for all) uploaded into one
 * device slab.  Each instance keeps its own time and CFL dt; every step is
 * one launch over all instances, replayed from a CUDA graph.  The initial
 * states are kept on the device for hydro_gpu_batch_restart. */
ErrorStatus hydro_gpu_batch_create(
    HydroGpuBatch **batch,
    int n_instances,
    BoundaryConditionParam *boundary_condition_params,
    System *systems,
    IntegratorParam *__restrict integrator_param,
    const HydroGpuOptions *options
);

ErrorStatus hydro_gpu_batch_restart(HydroGpuBatch *batch);

/* Advance every instance by up to num_steps steps (each stops at tf on its
 * own clock); statuses[i] (may be NULL) receives each instance's status. */
ErrorStatus hydro_gpu_batch_advance(
    HydroGpuBatch *batch,
    int64 num_steps,
    double tf,
    SimulationStatus *statuses,
    double *step_ms
);

/* Copy every instance's state back into systems[i]'s host arrays. */
ErrorStatus hydro_gpu_batch_download(HydroGpuBatch *batch, System *systems);

int64 hydro_gpu_batch_kernel_launches(const HydroGpuBatch *batch);

void hydro_gpu_batch_destroy(HydroGpuBatch *batch);

/* Measure the device's FMA throughput (TFLOP/s, 1 FMA = 2 FLOP) in FP64 and
 * FP32 with a short calibration kernel; either pointer may be NULL.  Used
 * for roofline reporting.  Returns 0 on success. */
int hydro_gpu_calibrate(int device, double *fp64_tflops, double *fp32_tflops);

/* Streaming multiprocessors of `device` (0 when it cannot be queried); with
 * the SM clock it gives the instruction-issue roof (4 warp instructions per
 * SM per clock) that roofline reporting uses for issue-bound kernels. */
int hydro_gpu_sm_count(int device);

/* The FP64 step's work items for an nx x ny grid (g ghost layers) on `slots`
 * resident CTAs: the guided row-chunk plan (h1-row items, then the last
 * `tail` rows in h2-row items) and, if rows is not NULL, each item's strip
 * and padded row range [r0, r1) as the kernel decodes it (3 ints per item,
 * at most max_items).  Returns the number of items.  Host only. */
int hydro_gpu_chunk_plan(int nx, int ny, int g, int slots, int *h1, int *h2, int *tail, int *rows,
                         int max_items);

/* ------------------------------------------------------------------ */
/* Allocation-free run.  No counterpart in the reference.              */
/* ------------------------------------------------------------------ */

/* Largest padded grid ((nx + 2G) * (ny + 2G) cells) the allocation-free
 * entry point accepts; its device state lives in a static array of about
 * 5.5 MiB that every GPU loading this library keeps until process exit. */
#define HYDRO_GPU_NOALLOC_MAX_CELLS 32768

/* MUSCL-Hancock 2D run (HLLC, built-in boundaries) that allocates nothing:
 * no cudaMalloc / cudaFree / cudaMallocHost, no stream or event creation, no
 * heap traceback.  For callers that must not allocate while they step: a
 * program whose device memory belongs to another allocator (a framework's
 * caching pool or a budget fixed at start-up, where a private cudaMalloc can
 * fail or fragment it), or a latency-sensitive loop that cannot take
 * cudaFree's device-wide synchronisation.  Same inputs and outputs as
 * launch_simulation for that integrator: the System's host arrays are read
 * and receive the final W and U; names in `boundary_condition_param` and
 * `integrator_param` are resolved here (finalize_* need not be called).
 * Runs on the calling thread's current device, until tf or `max_steps`
 * (< 0: no limit), synchronously.  No snapshots.
 *
 * Limits: grids above HYDRO_GPU_NOALLOC_MAX_CELLS padded cells are rejected
 * with VALUE_ERROR.  The first call on a device looks up the static array's
 * device address (cudaGetSymbolAddress) with that device current; make that
 * first call before any stream capture.  All calls share the array: calls
 * that overlap on the GPU (from several threads or streams) race.
 *
 * Returns SUCCESS or an error code of error.h; the message goes into
 * error_message (may be NULL). */
int hydro_gpu_muscl_hancock_2d_noalloc(
    const BoundaryConditionParam *boundary_condition_param,
    System *system,
    const IntegratorParam *integrator_param,
    double tf,
    int64 max_steps,
    SimulationStatus *simulation_status,
    char *error_message,
    int error_message_size
);

/* ------------------------------------------------------------------ */
/* Discrete adjoint and tangent-linear model of the 2D MUSCL-Hancock + */
/* HLLC step.  No counterpart in the reference.                        */
/* ------------------------------------------------------------------ */

/* The differentiated map: interior primitives W0 = (rho, vx, vy, p) of the
 * System handed to hydro_gpu_adjoint_create -> W^N after num_steps steps.
 * Ghost cells are images of the interior under the built-in boundary rules
 * (reflective, transmissive or periodic on every side), U0 is W0 converted
 * to conserved form, and every step uses the dt the forward pass chose (dt
 * is frozen: the CFL reduction is not differentiated; tf is ignored and the
 * run is exactly num_steps steps).  Limiter, Riemann-regime and region
 * decisions are those of the evaluation being differentiated.
 *
 * All field arguments are the padded host layout of the System arrays
 * ((nx + 2G) * (ny + 2G) doubles, row-major), in the order rho, vx, vy, p;
 * interior entries are read, ghost entries of outputs are written as 0. */
typedef struct HydroGpuAdjoint HydroGpuAdjoint;

typedef struct HydroGpuAdjointStats
{
    double forward_ms;            /* CUDA-event time of the forward pass */
    double recompute_ms;          /* last backward pass: segment recomputation */
    double vjp_ms;                /* last backward pass: reverse sweep */
    double tangent_ms;            /* last tangent-linear run */
    double replay_ms;             /* last replay */
    int64 steps;
    int64 checkpoint_every;
    int64 checkpoints;
    int64 recompute_mismatches;   /* recomputed dt or state differing from the forward pass (0 expected) */
    int64 kernel_launches;        /* kernels of this library launched by the session */
    int64 device_bytes;           /* device memory held by the session */
    int64 interior_cells;
} HydroGpuAdjointStats;

/* Finalize the parameters (muscl_hancock_2d with the HLLC solver, FP64),
 * allocate checkpoint and segment storage (state copies at steps 0, K, 2K,
 * ... with K = checkpoint_every, plus K resident states for recomputation)
 * and upload the System's W arrays as W0. */
ErrorStatus hydro_gpu_adjoint_create(
    HydroGpuAdjoint **adjoint,
    BoundaryConditionParam *__restrict boundary_condition_param,
    System *__restrict system,
    IntegratorParam *__restrict integrator_param,
    int64 num_steps,
    int checkpoint_every,
    const HydroGpuOptions *options
);

/* Run the forward pass (the production step kernel) from W0, logging dt and
 * storing checkpoints.  W_final (may be NULL) receives W^N. */
ErrorStatus hydro_gpu_adjoint_forward(HydroGpuAdjoint *adjoint, double *const W_final[4]);

/* Reverse pass: given seed = dJ/dW^N, write grad = dJ/dW0.  Segments are
 * recomputed from their checkpoints and swept in reverse. */
ErrorStatus hydro_gpu_adjoint_backward(HydroGpuAdjoint *adjoint, double *const seed[4],
                                       double *const grad[4]);

/* Tangent-linear model from W0 (or from w0 when not NULL) in direction dw0:
 * dw_final = (dW^N/dW0) dw0; w_final (may be NULL) receives the primal W^N,
 * which equals the forward pass's bit for bit when w0 is NULL. */
ErrorStatus hydro_gpu_adjoint_tangent(HydroGpuAdjoint *adjoint, double *const w0[4],
                                      double *const dw0[4], double *const w_final[4],
                                      double *const dw_final[4]);

/* Replay the num_steps steps from w0 with the forward pass's dt sequence
 * (finite-difference checks of the frozen-dt map).  signatures (may be
 * NULL, else num_steps entries) receives per step a hash sum of every
 * limiter / regime / region decision: equal signatures mean (up to hash
 * collisions) that the replay took the same branches. */
ErrorStatus hydro_gpu_adjoint_replay(HydroGpuAdjoint *adjoint, double *const w0[4],
                                     double *const w_final[4], unsigned long long *signatures);

/* Replay from w0 with the forward pass's dt sequence AND its branch
 * decisions (every limiter case, Riemann regime, guess floor, wave-speed
 * branch and flux region, recorded once from W0): the exact map the adjoint
 * differentiates, smooth around W0, for finite-difference checks that must
 * not cross kinks.  With w0 = W0 it returns W^N bit for bit. */
ErrorStatus hydro_gpu_adjoint_replay_frozen(HydroGpuAdjoint *adjoint, double *const w0[4],
                                            double *const w_final[4]);

/* Tape (default on): the segment recomputation writes, per face and step,
 * the face states and the HLLC guess with its factors (2 x 14 fields per
 * cell per step, K steps: about 224 bytes per cell per checkpointed step),
 * and the reverse sweep reads them instead of re-evaluating the
 * reconstruction and the guesses.  Off: nothing is stored and the reverse
 * sweep recomputes them; the gradient is the same bit for bit. */
void hydro_gpu_adjoint_set_tape(HydroGpuAdjoint *adjoint, int enabled);

/* dt of each forward step (num_steps entries). */
ErrorStatus hydro_gpu_adjoint_dt(const HydroGpuAdjoint *adjoint, double *dt);

void hydro_gpu_adjoint_stats(const HydroGpuAdjoint *adjoint, HydroGpuAdjointStats *stats);

void hydro_gpu_adjoint_destroy(HydroGpuAdjoint *adjoint);

/* Pointwise derivative kernels, host builds of the device code (for tests):
 * HLLC 2D flux (states rho, u_normal, u_tangential, p) in tangent and
 * reverse mode, and the cell reconstruction of one sweep direction
 * (dir 0: x, 1: y; cells wm, w0, wp in storage order rho, vx, vy, p;
 * limiter = SLOPE_LIMITER_*; lo / hi in sweep order). */
int hydro_ad_hllc_jvp(double gamma, double tol, const double L[4], const double R[4],
                      const double dL[4], const double dR[4], double F[4], double dF[4]);
int hydro_ad_hllc_vjp(double gamma, double tol, const double L[4], const double R[4],
                      const double Fb[4], double Lb[4], double Rb[4], int *branch_code);
void hydro_ad_recon_jvp(int limiter, int dir, double gamma, double dtA, const double wm[4],
                        const double w0[4], const double wp[4], const double dwm[4],
                        const double dw0[4], const double dwp[4], double lo[4], double hi[4],
                        double dlo[4], double dhi[4]);
void hydro_ad_recon_vjp(int limiter, int dir, double gamma, double dtA, const double wm[4],
                        const double w0[4], const double wp[4], const double lob[4],
                        const double hib[4], double wmb[4], double w0b[4], double wpb[4]);
/* The same two pieces with their branch decisions given (branch_code of
 * hydro_ad_hllc_vjp; natural_code receives the reconstruction's own code). */
void hydro_ad_hllc_forced(double gamma, double tol, const double L[4], const double R[4], int code,
                          double F[4]);
void hydro_ad_recon_forced(int limiter, int dir, double gamma, double dtA, const double wm[4],
                           const double w0[4], const double wp[4], int code, double lo[4],
                           double hi[4], int *natural_code);

/* The integer-pipe FP64 division (op 0: a[i] / b[i]), square root
 * (op 1: sqrt(a[i])) and power (op 2: pow(a[i], b[i])) the FP64 kernels use
 * in place of the FP64-pipe sequences; op 3, 4, 5: the minmod, van Leer and
 * MC limiters L(a[i], b[i]) (host: the FP64 expressions; device: as the
 * kernels evaluate them, ok[i] = 1 where the sign test was decided on the
 * bits); op 6 (host only): that sign test itself (1, 0 or -1).  Host build: out[i] = the integer form, ok[i] = 1 where its
 * fast path applied (elsewhere out[i] is meaningless).  Device build:
 * fast[i] = what the kernels compute, hw[i] = the hardware operation,
 * ok[i] as above; returns a cudaError_t. */
void hydro_fx_eval_host(int op, long long n, const double *a, const double *b, double *out,
                        unsigned char *ok);
int hydro_gpu_fx_eval(int device, int op, long long n, const double *a, const double *b,
                      double *fast, double *hw, unsigned char *ok);
/* Host build of the division with its FP32 reciprocal seed multiplied by
 * seed_scale[i] (tests of the seed check: where ok[i], out[i] = RN(a/b)). */
void hydro_fx_div_seeded_host(long long n, const double *a, const double *b, const float *seed_scale,
                              double *out, unsigned char *ok);

/* The exact solver's convergence test RN(x[i] / y[i]) < tol[i] decided without
 * the divide (host build): out[i] is the answer where decided[i] = 1. */
void hydro_fx_ratio_below_host(long long n, const double *x, const double *y, const double *tol,
                               unsigned char *out, unsigned char *decided);

/* The solvers' vacuum-generation test RN(x[i] / y[i]) <= z[i] decided without
 * the divide (host build): out[i] is the answer where decided[i] = 1. */
void hydro_fx_quot_le_host(long long n, const double *x, const double *y, const double *z,
                           unsigned char *out, unsigned char *decided);

/* Device build of the exported pointwise numerics over n state pairs:
 * L[4k..4k+3], R[4k..4k+3] = (rho, u, v, p) (the 1D forms read rho, u, p),
 * gas constants from gamma[k] and tol.
 *   op 0: solve_flux_hllc_2d (src/riemann_solver_hllc.h:46-61): out[4k..4k+3]
 *   op 1: guess_p (src/riemann_solver.h:123-134), a_L = aux[2k],
 *         a_R = aux[2k+1]: out[k]
 *   op 2: solve_flux_exact_1d at speed aux[k] (src/riemann_solver_exact.h:73-87):
 *         out[3k..3k+2]
 *   op 3: solve_flux_hllc_1d (src/riemann_solver_hllc.h:32-44): out[3k..3k+2]
 *   op 4: solve_exact_1d at speed aux[k] (src/riemann_solver_exact.h:37-51):
 *         the sampled (rho, u, p) in out[3k..3k+2]
 *   op 5, 6: ops 2 and 4 computed as the 1D kernel computes them, four lanes
 *         per state pair (quad_exact.cuh)
 * rc[k] = 0, or 1 (HLLC wave-speed error), 3 (exact solver: no bracket),
 * 4 (exact solver: bisection did not converge).  These are the functions the
 * step kernels call, compiled for the GPU, so the tests can check them
 * against the reference's known answers branch by branch.  Returns a
 * cudaError_t. */
int hydro_gpu_pointwise_eval(int device, int op, long long n, const double *gamma, double tol,
                             const double *L, const double *R, const double *aux, double *out,
                             int *rc);

/* Number of visible CUDA devices (0 when none; never fails). */
int hydro_gpu_device_count(void);

/* The 2D runs take their device memory from a per-device stream-ordered
 * pool that keeps what a finished run freed, and keep a few runs' streams,
 * events and pinned control blocks, so repeated launches neither map and
 * unmap their state nor create those objects each call.  This hands all of
 * it for `device` back to the driver (after the device is idle); 0 on
 * success.  No counterpart in the reference, which has no device memory. */
int hydro_gpu_trim_device_memory(int device);

/* Library version string. */
const char *hydro_gpu_version(void);

#ifdef __cplusplus
}
#endif

#endif
