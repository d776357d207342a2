/*
 * integrate_gpu.c -- the integrators of the hydroFV API, running on the GPU.
 *
 * Each integrator keeps the reference's contract (src/integrator_*.c):
 * validate the coordinate system, reset SimulationStatus, optionally store
 * the initial snapshot, step while t < tf with the CFL dt (shrunk for the
 * first steps) clipped to tf, store snapshots when
 * t >= interval * (count - offset + 1), and leave the final W and U in the
 * System's host arrays.  What changes is where the loop runs: the state is
 * uploaded once, stepped in HBM, and copied back at the end (and for each
 * snapshot, through pinned buffers).
 *
 * There is no CPU fallback: a CUDA failure is reported as an error.
 */
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gpu_bridge.h"
#include "hydro.h"
#include "hydro_gpu.h"
#include "host_internal.h"
#include "progress_bar.h"
#include "source_term.h"

/* ---------------------------------------------------------------- options */

static int g_have_process_options = 0;
static HydroGpuOptions g_process_options;

HydroGpuOptions hydro_gpu_default_options(void)
{
    HydroGpuOptions o;
    memset(&o, 0, sizeof o);
    o.device = 0;
    o.max_steps = -1;
    o.precision = HYDRO_GPU_PRECISION_FP64;
    o.chunk_steps = 0;
    o.use_graph = 1;
    o.block_threads = 0;
    o.chunk_rows = 0;
    return o;
}

void hydro_gpu_set_process_options(const HydroGpuOptions *options)
{
    if (options)
    {
        g_process_options = *options;
        g_have_process_options = 1;
    }
    else
    {
        g_have_process_options = 0;
    }
}

static HydroGpuOptions process_options(void)
{
    if (g_have_process_options) return g_process_options;
    HydroGpuOptions o = hydro_gpu_default_options();
    const char *dev = getenv("HYDRO_GPU_DEVICE");
    if (dev && *dev) o.device = atoi(dev);
    const char *ms = getenv("HYDRO_GPU_MAX_STEPS");
    if (ms && *ms) o.max_steps = atoll(ms);
    return o;
}

const char *hydro_gpu_version(void)
{
    return "hydrofv-gb300 0.1 (sm_103a)";
}

/* ------------------------------------------------------- error mapping */

/* Turn a bridge outcome into the reference's ErrorStatus. */
/* The reference warns every 500 bisection iterations of its exact Riemann
 * solver when Settings.verbose > 0 (src/riemann_solver_exact.c:736-744).
 * The 1D kernel counts the solves that passed each mark; the warnings are
 * printed after the run, mark by mark (for a single slow solve, the
 * reference's order). */
static void bisection_warnings(const Settings *settings, const HydroRunOutcome *oc)
{
    if (!settings || settings->verbose <= 0) return;
    for (int k = 0; k < 10; k++)
        for (unsigned int n = 0; n < oc->bisect_marks[k]; n++)
        {
            char buf[128];
            snprintf(buf, sizeof buf,
                     "Bisection method did not converge after %d iterations for exact riemann solver.",
                     500 * (k + 1));
            WRAP_RAISE_WARNING(buf);
        }
}

/* HYDRO_GPU_TRACE set (to anything but "0"): a 2D launch prints the host
 * wall time of each of its phases to stderr (set-up, upload, begin,
 * stepping, download, teardown), so a caller can see where a drop-in call's
 * time goes beyond the stepping. */
static int trace_enabled(void)
{
    /* read on every phase (six per launch): no shared cache between the
     * threads that may launch concurrently */
    const char *v = getenv("HYDRO_GPU_TRACE");
    return (v && v[0] && strcmp(v, "0") != 0) ? 1 : 0;
}

static void trace_phase(const char *what, double *t_last)
{
    if (!trace_enabled()) return;
    const double now = hydro_get_current_time();
    fprintf(stderr, "hydro_gpu: %-9s %9.3f ms\n", what, (now - *t_last) * 1e3);
    *t_last = now;
}

static ErrorStatus outcome_error(const HydroRunOutcome *oc)
{
    switch (oc->kind)
    {
        case HYDRO_RUN_DEVICE_ERROR:
            return hydro_device_error_status(oc->code);
        case HYDRO_RUN_UNSUPPORTED:
            return WRAP_RAISE_ERROR(NOT_IMPLEMENTED_ERROR, oc->message);
        case HYDRO_RUN_CALLBACK_ERROR:
            return WRAP_RAISE_ERROR(OS_ERROR, "Storing a snapshot failed.");
        case HYDRO_RUN_CUDA_ERROR:
        default:
            if (strstr(oc->message, "cudaMalloc") || strstr(oc->message, "out of memory"))
                return WRAP_RAISE_ERROR(MEMORY_ERROR, oc->message);
            return WRAP_RAISE_ERROR(FAILURE, oc->message);
    }
}

/* -------------------------------------------------------- 2D set-up */

/* 1 if a[lo, hi) all equal v: branch-free blocks the compiler vectorises,
 * with an early exit between blocks. */
static int all_equal(const double *a, long long lo, long long hi, double v)
{
    for (long long b = lo; b < hi; b += 4096)
    {
        const long long e = (b + 4096 < hi) ? b + 4096 : hi;
        int bad = 0;
        for (long long k = b; k < e; k++) bad |= (a[k] != v);
        if (bad) return 0;
    }
    return 1;
}

typedef struct UniformPart
{
    const double *a;
    long long lo, hi;
    int ok;
} UniformPart;

static void *uniform_part(void *arg)
{
    UniformPart *p = arg;
    p->ok = all_equal(p->a, p->lo, p->hi, p->a[0]);
    return NULL;
}

/* 1 if every a[k] equals a[0].  The 2D grids' volumes are one array per
 * cell (33.7 MB at 2048^2), so large arrays are split over a few host
 * threads: the scan was most of a drop-in call's set-up time. */
static int uniform(const double *a, long long n)
{
    enum { PARTS = 8 };
    if (n < (1LL << 20)) return all_equal(a, 1, n, a[0]);
    UniformPart part[PARTS];
    pthread_t tid[PARTS];
    int started[PARTS];
    for (int k = 0; k < PARTS; k++)
    {
        part[k].a = a;
        part[k].lo = n * k / PARTS;
        part[k].hi = n * (k + 1) / PARTS;
        part[k].ok = 1;
        started[k] = (k > 0) && pthread_create(&tid[k], NULL, uniform_part, &part[k]) == 0;
        if (k > 0 && !started[k]) uniform_part(&part[k]);
    }
    uniform_part(&part[0]);
    int ok = part[0].ok;
    for (int k = 1; k < PARTS; k++)
    {
        if (started[k]) pthread_join(tid[k], NULL);
        ok &= part[k].ok;
    }
    return ok;
}

/* Checks shared by the 2D integrators; fills grid. */
static ErrorStatus setup_grid2d(const BoundaryConditionParam *bcp, const System *s,
                                const IntegratorParam *ip, HydroGrid2D *grid)
{
    if (s->coord_sys_flag_ != COORD_SYS_CARTESIAN_2D)
    {
        char msg[256];
        snprintf(msg, sizeof msg,
                 "Wrong coordinate system. Supported coordinate system: \"cartesian_2d\", got: \"%s\"",
                 s->coord_sys);
        return WRAP_RAISE_ERROR(VALUE_ERROR, msg);
    }
    const int flags[4] = { bcp->boundary_condition_flag_x_min_, bcp->boundary_condition_flag_x_max_,
                           bcp->boundary_condition_flag_y_min_, bcp->boundary_condition_flag_y_max_ };
    for (int k = 0; k < 4; k++)
    {
        if (flags[k] < BOUNDARY_CONDITION_NONE || flags[k] > BOUNDARY_CONDITION_CUSTOM)
            return WRAP_RAISE_ERROR(VALUE_ERROR, "Boundary condition flag not recognized.");
        grid->bc[k] = flags[k];
    }
    grid->gravity = s->gravity;
    const int g = s->num_ghost_cells_side;
    const long long tx = s->num_cells_x + 2 * g, ty = s->num_cells_y + 2 * g;
    if (!uniform(s->surface_area_x_, tx) || !uniform(s->surface_area_y_, ty) || !uniform(s->volume_, tx * ty))
    {
        return WRAP_RAISE_ERROR(NOT_IMPLEMENTED_ERROR,
                                "The GPU path needs uniform face areas and cell volumes (as system_init sets them).");
    }
    grid->nx = s->num_cells_x;
    grid->ny = s->num_cells_y;
    grid->g = g;
    grid->gamma = s->gamma;
    grid->tol = ip->tol;
    grid->dx = s->dx_;
    grid->dy = s->dy_;
    grid->area_x = s->surface_area_x_[0];
    grid->area_y = s->surface_area_y_[0];
    grid->vol = s->volume_[0];
    grid->limiter = ip->slope_limiter_flag_;
    grid->integrator = ip->integrator_flag_;
    return make_success_error_status();
}

typedef struct SnapCtx
{
    const BoundaryConditionParam *bcp;
    const System *system;
    const IntegratorParam *ip;
    StoringParam *sp;
    ErrorStatus status;
} SnapCtx;

/* Snapshot callback: a System view whose primitive arrays are the pinned
 * buffers holding the materialized state. */
static int snapshot_cb(void *vctx, double *const W[4], int64 num_steps, double t, double dt)
{
    SnapCtx *ctx = vctx;
    System view = *ctx->system;
    view.density_ = W[0];
    view.velocity_x_ = W[1];
    if (view.coord_sys_flag_ == COORD_SYS_CARTESIAN_2D)
    {
        view.velocity_y_ = W[2];
        view.pressure_ = W[3];
    }
    else
    {
        view.pressure_ = W[2];
    }
    SimulationStatus st = { num_steps, t, dt };
    ctx->status = WRAP_TRACEBACK(store_snapshot(ctx->bcp, &view, ctx->ip, &st, ctx->sp));
    return ctx->status.return_code == SUCCESS ? 0 : 1;
}

/* Host boundary routine for custom sides: the reference's boundary routine
 * (src/boundary.c:513-777, custom sides through their callbacks) on a
 * System view of the converted state. */
typedef struct HostBcCtx
{
    BoundaryConditionParam bcp;
    System system;
    ErrorStatus status;
} HostBcCtx;

static int host_bc_cb(void *vctx, double *const W[4])
{
    HostBcCtx *ctx = vctx;
    System view = ctx->system;
    view.density_ = W[0];
    view.velocity_x_ = W[1];
    view.velocity_y_ = W[2];
    view.pressure_ = W[3];
    free_traceback(&ctx->status);
    ctx->status = WRAP_TRACEBACK(set_boundary_condition(&ctx->bcp, &view));
    return ctx->status.return_code == SUCCESS ? 0 : 1;
}

static int has_custom(const HydroGrid2D *grid)
{
    for (int k = 0; k < 4; k++)
        if (grid->bc[k] == BOUNDARY_CONDITION_CUSTOM) return 1;
    return 0;
}

static HydroStepParams step_params(const IntegratorParam *ip, const StoringParam *sp)
{
    HydroStepParams p;
    memset(&p, 0, sizeof p);
    p.cfl = ip->cfl;
    p.cfl_shrunk = ip->cfl * ip->cfl_initial_shrink_factor;
    p.shrink_steps = ip->cfl_initial_shrink_num_steps;
    p.is_storing = sp->is_storing ? 1 : 0;
    p.store_initial_offset = (sp->is_storing && sp->store_initial) ? 1 : 0;
    p.storing_interval = sp->storing_interval;
    return p;
}

static ErrorStatus run_2d(
    BoundaryConditionParam *__restrict bcp,
    System *__restrict s,
    IntegratorParam *__restrict ip,
    StoringParam *__restrict sp,
    Settings *__restrict settings,
    SimulationParam *__restrict simp,
    SimulationStatus *__restrict status,
    const HydroGpuOptions *opt,
    HydroGpuStats *stats
)
{
    const double t_start = hydro_get_current_time();
    HydroGrid2D grid;
    memset(&grid, 0, sizeof grid);
    ErrorStatus e = setup_grid2d(bcp, s, ip, &grid);
    if (e.return_code != SUCCESS) return e;
    if (opt->precision != HYDRO_GPU_PRECISION_FP64 && opt->precision != HYDRO_GPU_PRECISION_FP32)
    {
        return WRAP_RAISE_ERROR(VALUE_ERROR, "Unknown precision.");
    }

    status->num_steps = 0;
    status->dt = 0.0;
    status->t = 0.0;
    sp->store_count_ = 0;
    if (sp->is_storing && sp->store_initial)
    {
        e = WRAP_TRACEBACK(store_snapshot(bcp, s, ip, status, sp));
        if (e.return_code != SUCCESS) return e;
    }
    ProgressBarParam bar;
    if (!settings->no_progress_bar) start_progress_bar(&bar, simp->tf);

    HydroRunOutcome oc;
    HydroRun2D *run = NULL;
    double *W[4] = { s->density_, s->velocity_x_, s->velocity_y_, s->pressure_ };
    double *U[4] = { s->mass_, s->momentum_x_, s->momentum_y_, s->energy_ };
    const HydroStepParams params = step_params(ip, sp);
    SnapCtx ctx = { bcp, s, ip, sp, make_success_error_status() };
    HostBcCtx bctx;
    memset(&bctx, 0, sizeof bctx);
    bctx.bcp = *bcp;
    bctx.system = *s;
    bctx.status = make_success_error_status();

    double t_phase = t_start;
    int rc = hydro_run2d_create(&grid, opt, &run, &oc);
    if (rc == 0 && has_custom(&grid)) rc = hydro_run2d_set_host_bc(run, host_bc_cb, &bctx, &oc);
    trace_phase("set-up", &t_phase);
    if (rc == 0) rc = hydro_run2d_upload(run, W, U, 0, &oc);
    trace_phase("upload", &t_phase);
    if (rc == 0) rc = hydro_run2d_begin(run, &params, simp->tf, opt->max_steps, sp->store_count_, &oc);
    trace_phase("begin", &t_phase);
    int advanced = 0;
    HydroRunOutcome aoc;
    memset(&aoc, 0, sizeof aoc);
    if (rc == 0)
    {
        advanced = 1;
        rc = hydro_run2d_advance(run, snapshot_cb, &ctx, &aoc, NULL);
        if (rc != 0) oc = aoc;
    }
    trace_phase("stepping", &t_phase);
    /* Whatever happened, hand back the last consistent state. */
    if (advanced)
    {
        status->num_steps = aoc.num_steps;
        status->t = aoc.t;
        status->dt = aoc.dt;
        sp->store_count_ = aoc.store_count;
        if (aoc.num_steps > 0)
        {
            HydroRunOutcome doc;
            if (hydro_run2d_download(run, W, U, &doc) != 0 && rc == 0)
            {
                rc = -1;
                oc = doc;
            }
        }
    }
    trace_phase("download", &t_phase);
    if (stats && run) hydro_run2d_stats(run, stats);
    hydro_run2d_destroy(run);
    trace_phase("teardown", &t_phase);
    if (!settings->no_progress_bar) update_progress_bar(&bar, status->t, true);
    if (stats) stats->total_ms = (hydro_get_current_time() - t_start) * 1e3;

    if (rc != 0)
    {
        if (oc.kind == HYDRO_RUN_CALLBACK_ERROR && bctx.status.return_code != SUCCESS)
        {
            free_traceback(&ctx.status);
            return bctx.status;
        }
        free_traceback(&bctx.status);
        if (oc.kind == HYDRO_RUN_CALLBACK_ERROR && ctx.status.return_code != SUCCESS) return ctx.status;
        free_traceback(&ctx.status);
        return outcome_error(&oc);
    }
    free_traceback(&bctx.status);
    return make_success_error_status();
}

/* --------------------------------------------------------- integrators */

ErrorStatus muscl_hancock_2d(
    BoundaryConditionParam *__restrict bcp,
    System *__restrict system,
    IntegratorParam *__restrict ip,
    StoringParam *__restrict sp,
    Settings *__restrict settings,
    SimulationParam *__restrict simp,
    SimulationStatus *__restrict status
)
{
    const HydroGpuOptions opt = process_options();
    return run_2d(bcp, system, ip, sp, settings, simp, status, &opt, NULL);
}

ErrorStatus godunov_first_order_2d(
    BoundaryConditionParam *__restrict bcp,
    System *__restrict system,
    IntegratorParam *__restrict ip,
    StoringParam *__restrict sp,
    Settings *__restrict settings,
    SimulationParam *__restrict simp,
    SimulationStatus *__restrict status
)
{
    const HydroGpuOptions opt = process_options();
    return run_2d(bcp, system, ip, sp, settings, simp, status, &opt, NULL);
}

/* Shared body of the 1D integrators (src/integrator_godunov_first_order.c:26-261,
 * src/integrator_muscl_hancock.c:26-383), Cartesian grids. */
static ErrorStatus run_1d(
    BoundaryConditionParam *__restrict bcp,
    System *__restrict s,
    IntegratorParam *__restrict ip,
    StoringParam *__restrict sp,
    Settings *__restrict settings,
    SimulationParam *__restrict simp,
    SimulationStatus *__restrict status,
    const HydroGpuOptions *opt,
    HydroGpuStats *stats
)
{
    const int cs = s->coord_sys_flag_;
    if (cs != COORD_SYS_CARTESIAN_1D && cs != COORD_SYS_CYLINDRICAL_1D && cs != COORD_SYS_SPHERICAL_1D)
    {
        char msg[256];
        snprintf(msg, sizeof msg,
                 "Wrong coordinate system. Supported coordinate system: \"cartesian_1d\", "
                 "\"cylindrical_1d\" and \"spherical_1d\", got: \"%s\"", s->coord_sys);
        return WRAP_RAISE_ERROR(VALUE_ERROR, msg);
    }
    const int flags[2] = { bcp->boundary_condition_flag_x_min_, bcp->boundary_condition_flag_x_max_ };
    for (int k = 0; k < 2; k++)
    {
        if (flags[k] == BOUNDARY_CONDITION_CUSTOM)
            return WRAP_RAISE_ERROR(NOT_IMPLEMENTED_ERROR,
                                    "Custom boundary conditions are not available on the GPU path.");
        if (flags[k] < BOUNDARY_CONDITION_NONE || flags[k] > BOUNDARY_CONDITION_PERIODIC)
            return WRAP_RAISE_ERROR(VALUE_ERROR, "Boundary condition flag not recognized.");
    }
    if (opt->precision != HYDRO_GPU_PRECISION_FP64)
    {
        return WRAP_RAISE_ERROR(NOT_IMPLEMENTED_ERROR, "Requested precision is not available for this integrator.");
    }
    const int g = s->num_ghost_cells_side;
    if (s->num_cells_x < g)
    {
        return WRAP_RAISE_ERROR(NOT_IMPLEMENTED_ERROR,
                                "The GPU path needs at least num_ghost_cells_side interior cells.");
    }
    if (ip->integrator_flag_ == INTEGRATOR_RANDOM_CHOICE_1D && g < 2)
    {
        /* the reference's random choice reads the cell beyond the last face (src/integrator_random_choice_1d.c:190) */
        return WRAP_RAISE_ERROR(VALUE_ERROR, "random_choice_1d needs at least 2 ghost cells per side.");
    }
    HydroGrid1D grid;
    memset(&grid, 0, sizeof grid);
    grid.nx = s->num_cells_x;
    grid.g = g;
    grid.gamma = s->gamma;
    grid.tol = ip->tol;
    grid.dx = s->dx_;
    grid.area = s->surface_area_x_;
    grid.vol = s->volume_;
    grid.mid = s->mid_points_x_;
    grid.alpha = (cs == COORD_SYS_CYLINDRICAL_1D) ? 1.0 : (cs == COORD_SYS_SPHERICAL_1D) ? 2.0 : 0.0;
    grid.bc[0] = flags[0];
    grid.bc[1] = flags[1];
    grid.limiter = ip->slope_limiter_flag_;
    grid.riemann_solver = ip->riemann_solver_flag_;
    grid.integrator = ip->integrator_flag_;

    status->num_steps = 0;
    status->dt = 0.0;
    status->t = 0.0;
    sp->store_count_ = 0;
    if (sp->is_storing && sp->store_initial)
    {
        ErrorStatus e = WRAP_TRACEBACK(store_snapshot(bcp, s, ip, status, sp));
        if (e.return_code != SUCCESS) return e;
    }
    ProgressBarParam bar;
    if (!settings->no_progress_bar) start_progress_bar(&bar, simp->tf);
    double *W[3] = { s->density_, s->velocity_x_, s->pressure_ };
    double *U[3] = { s->mass_, s->momentum_x_, s->energy_ };
    const HydroStepParams params = step_params(ip, sp);
    SnapCtx ctx = { bcp, s, ip, sp, make_success_error_status() };
    HydroRunOutcome oc;
    const int rc = hydro_run1d(&grid, W, U, &params, simp->tf, opt->max_steps, sp->store_count_,
                               snapshot_cb, &ctx, opt, &oc, stats);
    bisection_warnings(settings, &oc);
    status->num_steps = oc.num_steps;
    status->t = oc.t;
    status->dt = oc.dt;
    sp->store_count_ = oc.store_count;
    if (!settings->no_progress_bar) update_progress_bar(&bar, status->t, true);
    if (rc != 0)
    {
        if (oc.kind == HYDRO_RUN_CALLBACK_ERROR && ctx.status.return_code != SUCCESS) return ctx.status;
        free_traceback(&ctx.status);
        return outcome_error(&oc);
    }
    return make_success_error_status();
}

ErrorStatus godunov_first_order_1d(
    BoundaryConditionParam *__restrict bcp,
    System *__restrict system,
    IntegratorParam *__restrict ip,
    StoringParam *__restrict sp,
    Settings *__restrict settings,
    SimulationParam *__restrict simp,
    SimulationStatus *__restrict status
)
{
    const HydroGpuOptions opt = process_options();
    return run_1d(bcp, system, ip, sp, settings, simp, status, &opt, NULL);
}

ErrorStatus muscl_hancock_1d(
    BoundaryConditionParam *__restrict bcp,
    System *__restrict system,
    IntegratorParam *__restrict ip,
    StoringParam *__restrict sp,
    Settings *__restrict settings,
    SimulationParam *__restrict simp,
    SimulationStatus *__restrict status
)
{
    const HydroGpuOptions opt = process_options();
    return run_1d(bcp, system, ip, sp, settings, simp, status, &opt, NULL);
}

ErrorStatus random_choice_1d(
    BoundaryConditionParam *__restrict bcp,
    System *__restrict system,
    IntegratorParam *__restrict ip,
    StoringParam *__restrict sp,
    Settings *__restrict settings,
    SimulationParam *__restrict simp,
    SimulationStatus *__restrict status
)
{
    const HydroGpuOptions opt = process_options();
    return run_1d(bcp, system, ip, sp, settings, simp, status, &opt, NULL);
}

/* ------------------------------------------------------- extension API */

ErrorStatus hydro_gpu_launch_simulation(
    BoundaryConditionParam *__restrict bcp,
    System *__restrict system,
    IntegratorParam *__restrict ip,
    StoringParam *__restrict sp,
    Settings *__restrict settings,
    SimulationParam *__restrict simp,
    SimulationStatus *__restrict status,
    const HydroGpuOptions *options,
    HydroGpuStats *stats
)
{
    if (stats) memset(stats, 0, sizeof *stats);
    const HydroGpuOptions opt = options ? *options : hydro_gpu_default_options();
    /* The same finalize / check sequence as launch_simulation (src/hydro.c:29-91). */
    ErrorStatus e = WRAP_TRACEBACK(finalize_boundary_condition_param(system, bcp));
    if (e.return_code != SUCCESS) return e;
    e = WRAP_TRACEBACK(finalize_integrator_param(ip));
    if (e.return_code != SUCCESS) return e;
    e = WRAP_TRACEBACK(finalize_storing_param(sp));
    if (e.return_code != SUCCESS) return e;
    e = WRAP_TRACEBACK(hydro_final_check(system, ip));
    if (e.return_code != SUCCESS) return e;
    switch (ip->integrator_flag_)
    {
        case INTEGRATOR_MUSCL_HANCOCK_2D:
        case INTEGRATOR_GODUNOV_FIRST_ORDER_2D:
            return WRAP_TRACEBACK(run_2d(bcp, system, ip, sp, settings, simp, status, &opt, stats));
        case INTEGRATOR_GODUNOV_FIRST_ORDER_1D:
        case INTEGRATOR_MUSCL_HANCOCK_1D:
        case INTEGRATOR_RANDOM_CHOICE_1D:
            return WRAP_TRACEBACK(run_1d(bcp, system, ip, sp, settings, simp, status, &opt, stats));
        default:
        {
            const int had = g_have_process_options;
            const HydroGpuOptions saved = g_process_options;
            hydro_gpu_set_process_options(&opt);
            e = WRAP_TRACEBACK(integrator_launch_simulation(bcp, system, ip, sp, settings, simp, status));
            g_process_options = saved;
            g_have_process_options = had;
            return e;
        }
    }
}

/* ------------------------------------------------------------ session */

struct HydroGpuSolver
{
    HydroRun2D *run;
    HydroGrid2D grid;
    HydroStepParams params;
    int begun;
    int64 launches_at_create;
    HostBcCtx bc;                 /* custom sides: the boundary routine's inputs */
};

ErrorStatus hydro_gpu_solver_create(
    HydroGpuSolver **out,
    BoundaryConditionParam *__restrict bcp,
    System *__restrict system,
    IntegratorParam *__restrict ip,
    const HydroGpuOptions *options
)
{
    *out = NULL;
    ErrorStatus e = WRAP_TRACEBACK(finalize_boundary_condition_param(system, bcp));
    if (e.return_code != SUCCESS) return e;
    e = WRAP_TRACEBACK(finalize_integrator_param(ip));
    if (e.return_code != SUCCESS) return e;
    if (ip->integrator_flag_ != INTEGRATOR_MUSCL_HANCOCK_2D)
        return WRAP_RAISE_ERROR(NOT_IMPLEMENTED_ERROR, "The solver session supports muscl_hancock_2d.");
    if (system->num_ghost_cells_side < 2)
        return WRAP_RAISE_ERROR(VALUE_ERROR, "Number of ghost cells must be at least 2.");
    HydroGpuSolver *sv = calloc(1, sizeof *sv);
    if (!sv) return WRAP_RAISE_ERROR(MEMORY_ERROR, "Failed to allocate the solver.");
    e = setup_grid2d(bcp, system, ip, &sv->grid);
    if (e.return_code != SUCCESS)
    {
        free(sv);
        return e;
    }
    const HydroGpuOptions opt = options ? *options : hydro_gpu_default_options();
    StoringParam none = get_new_storing_param();
    sv->params = step_params(ip, &none);
    HydroRunOutcome oc;
    double *W[4] = { system->density_, system->velocity_x_, system->velocity_y_, system->pressure_ };
    double *U[4] = { system->mass_, system->momentum_x_, system->momentum_y_, system->energy_ };
    sv->bc.bcp = *bcp;
    sv->bc.system = *system;
    sv->bc.status = make_success_error_status();
    int rc = hydro_run2d_create(&sv->grid, &opt, &sv->run, &oc);
    if (rc == 0 && has_custom(&sv->grid)) rc = hydro_run2d_set_host_bc(sv->run, host_bc_cb, &sv->bc, &oc);
    if (rc == 0) rc = hydro_run2d_upload(sv->run, W, U, 1, &oc);
    if (rc != 0)
    {
        hydro_run2d_destroy(sv->run);
        free(sv);
        return outcome_error(&oc);
    }
    *out = sv;
    return make_success_error_status();
}

ErrorStatus hydro_gpu_solver_restart(HydroGpuSolver *sv)
{
    HydroRunOutcome oc;
    if (hydro_run2d_restore(sv->run, &oc) != 0) return outcome_error(&oc);
    sv->begun = 0;
    return make_success_error_status();
}

ErrorStatus hydro_gpu_solver_advance(
    HydroGpuSolver *sv,
    int64 num_steps,
    double tf,
    SimulationStatus *__restrict status,
    double *step_ms
)
{
    HydroRunOutcome oc;
    if (!sv->begun)
    {
        if (hydro_run2d_begin(sv->run, &sv->params, tf, num_steps, 0, &oc) != 0) return outcome_error(&oc);
        sv->begun = 1;
    }
    else
    {
        if (hydro_run2d_status(sv->run, &oc) != 0) return outcome_error(&oc);
        if (hydro_run2d_set_limits(sv->run, tf, oc.num_steps + num_steps, &oc) != 0) return outcome_error(&oc);
    }
    const int rc = hydro_run2d_advance(sv->run, NULL, NULL, &oc, step_ms);
    if (status)
    {
        status->num_steps = oc.num_steps;
        status->t = oc.t;
        status->dt = oc.dt;
    }
    if (rc != 0)
    {
        if (oc.kind == HYDRO_RUN_CALLBACK_ERROR && sv->bc.status.return_code != SUCCESS)
        {
            ErrorStatus e = sv->bc.status;
            sv->bc.status = make_success_error_status();
            return e;
        }
        return outcome_error(&oc);
    }
    return make_success_error_status();
}

ErrorStatus hydro_gpu_solver_download(HydroGpuSolver *sv, System *__restrict system)
{
    HydroRunOutcome oc;
    double *W[4] = { system->density_, system->velocity_x_, system->velocity_y_, system->pressure_ };
    double *U[4] = { system->mass_, system->momentum_x_, system->momentum_y_, system->energy_ };
    if (hydro_run2d_download(sv->run, W, U, &oc) != 0) return outcome_error(&oc);
    return make_success_error_status();
}

ErrorStatus hydro_gpu_solver_conserved_totals(HydroGpuSolver *sv, double totals[4])
{
    HydroRunOutcome oc;
    if (hydro_run2d_totals(sv->run, totals, &oc) != 0) return outcome_error(&oc);
    return make_success_error_status();
}

int64 hydro_gpu_solver_kernel_launches(const HydroGpuSolver *sv)
{
    HydroGpuStats st;
    memset(&st, 0, sizeof st);
    hydro_run2d_stats(sv->run, &st);
    return st.kernel_launches;
}

void hydro_gpu_solver_destroy(HydroGpuSolver *sv)
{
    if (!sv) return;
    free_traceback(&sv->bc.status);
    hydro_run2d_destroy(sv->run);
    free(sv);
}

/* -------------------------------------------------------------- batches */

struct HydroGpuBatch
{
    HydroBatch2D *b;
    int n;
    HydroStepParams params;
    int begun;
};

ErrorStatus hydro_gpu_batch_create(
    HydroGpuBatch **out,
    int n,
    BoundaryConditionParam *bcps,
    System *systems,
    IntegratorParam *__restrict ip,
    const HydroGpuOptions *options
)
{
    *out = NULL;
    if (n < 1 || !bcps || !systems) return WRAP_RAISE_ERROR(POINTER_ERROR, "Empty batch.");
    ErrorStatus e = WRAP_TRACEBACK(finalize_integrator_param(ip));
    if (e.return_code != SUCCESS) return e;
    if (ip->integrator_flag_ != INTEGRATOR_MUSCL_HANCOCK_2D && ip->integrator_flag_ != INTEGRATOR_GODUNOV_FIRST_ORDER_2D)
        return WRAP_RAISE_ERROR(NOT_IMPLEMENTED_ERROR, "Batches run the 2D integrators.");
    HydroGrid2D *grids = calloc((size_t) n, sizeof *grids);
    HydroGpuBatch *bt = calloc(1, sizeof *bt);
    if (!grids || !bt)
    {
        free(grids);
        free(bt);
        return WRAP_RAISE_ERROR(MEMORY_ERROR, "Failed to allocate the batch.");
    }
    for (int i = 0; i < n; i++)
    {
        e = WRAP_TRACEBACK(finalize_boundary_condition_param(&systems[i], &bcps[i]));
        if (e.return_code == SUCCESS) e = WRAP_TRACEBACK(hydro_final_check(&systems[i], ip));
        if (e.return_code == SUCCESS) e = setup_grid2d(&bcps[i], &systems[i], ip, &grids[i]);
        if (e.return_code == SUCCESS && (has_custom(&grids[i]) || grids[i].gravity != 0.0))
            e = WRAP_RAISE_ERROR(NOT_IMPLEMENTED_ERROR,
                                 "Batches take built-in boundary conditions and no gravity source.");
        if (e.return_code != SUCCESS)
        {
            free(grids);
            free(bt);
            return e;
        }
    }
    const HydroGpuOptions opt = options ? *options : hydro_gpu_default_options();
    StoringParam none = get_new_storing_param();
    bt->params = step_params(ip, &none);
    bt->n = n;
    HydroRunOutcome oc;
    int rc = hydro_batch2d_create(grids, n, &opt, &bt->b, &oc);
    free(grids);
    for (int i = 0; rc == 0 && i < n; i++)
    {
        System *s = &systems[i];
        double *W[4] = { s->density_, s->velocity_x_, s->velocity_y_, s->pressure_ };
        double *U[4] = { s->mass_, s->momentum_x_, s->momentum_y_, s->energy_ };
        rc = hydro_batch2d_upload(bt->b, i, W, U, &oc);
    }
    if (rc != 0)
    {
        hydro_batch2d_destroy(bt->b);
        free(bt);
        return outcome_error(&oc);
    }
    *out = bt;
    return make_success_error_status();
}

ErrorStatus hydro_gpu_batch_restart(HydroGpuBatch *bt)
{
    HydroRunOutcome oc;
    if (hydro_batch2d_restore(bt->b, &oc) != 0) return outcome_error(&oc);
    bt->begun = 0;
    return make_success_error_status();
}

ErrorStatus hydro_gpu_batch_advance(
    HydroGpuBatch *bt,
    int64 num_steps,
    double tf,
    SimulationStatus *statuses,
    double *step_ms
)
{
    HydroRunOutcome oc;
    if (!bt->begun)
    {
        if (hydro_batch2d_begin(bt->b, &bt->params, tf, num_steps, &oc) != 0) return outcome_error(&oc);
        bt->begun = 1;
    }
    else if (hydro_batch2d_set_limits(bt->b, tf, num_steps, &oc) != 0)
    {
        return outcome_error(&oc);
    }
    const int rc = hydro_batch2d_advance(bt->b, &oc, step_ms);
    if (statuses)
    {
        for (int i = 0; i < bt->n; i++)
        {
            HydroRunOutcome so;
            hydro_batch2d_status(bt->b, i, &so);
            statuses[i].num_steps = so.num_steps;
            statuses[i].t = so.t;
            statuses[i].dt = so.dt;
        }
    }
    if (rc != 0) return outcome_error(&oc);
    return make_success_error_status();
}

ErrorStatus hydro_gpu_batch_download(HydroGpuBatch *bt, System *systems)
{
    for (int i = 0; i < bt->n; i++)
    {
        HydroRunOutcome oc;
        System *s = &systems[i];
        double *W[4] = { s->density_, s->velocity_x_, s->velocity_y_, s->pressure_ };
        double *U[4] = { s->mass_, s->momentum_x_, s->momentum_y_, s->energy_ };
        if (hydro_batch2d_download(bt->b, i, W, U, &oc) != 0) return outcome_error(&oc);
    }
    return make_success_error_status();
}

int64 hydro_gpu_batch_kernel_launches(const HydroGpuBatch *bt)
{
    HydroGpuStats st;
    hydro_batch2d_stats(bt->b, &st);
    return st.kernel_launches;
}

void hydro_gpu_batch_destroy(HydroGpuBatch *bt)
{
    if (!bt) return;
    hydro_batch2d_destroy(bt->b);
    free(bt);
}

/* ------------------------------------------------------------- adjoint */

struct HydroGpuAdjoint
{
    HydroAdj2D *adj;
};

ErrorStatus hydro_gpu_adjoint_create(
    HydroGpuAdjoint **out,
    BoundaryConditionParam *__restrict bcp,
    System *__restrict system,
    IntegratorParam *__restrict ip,
    int64 num_steps,
    int checkpoint_every,
    const HydroGpuOptions *options
)
{
    *out = NULL;
    ErrorStatus e = WRAP_TRACEBACK(finalize_boundary_condition_param(system, bcp));
    if (e.return_code != SUCCESS) return e;
    e = WRAP_TRACEBACK(finalize_integrator_param(ip));
    if (e.return_code != SUCCESS) return e;
    if (ip->integrator_flag_ != INTEGRATOR_MUSCL_HANCOCK_2D)
        return WRAP_RAISE_ERROR(NOT_IMPLEMENTED_ERROR, "The adjoint differentiates muscl_hancock_2d.");
    if (system->num_ghost_cells_side < 2)
        return WRAP_RAISE_ERROR(VALUE_ERROR, "Number of ghost cells must be at least 2.");
    if (num_steps < 1 || checkpoint_every < 1)
        return WRAP_RAISE_ERROR(VALUE_ERROR, "num_steps and checkpoint_every must be at least 1.");
    HydroGrid2D grid;
    memset(&grid, 0, sizeof grid);
    e = setup_grid2d(bcp, system, ip, &grid);
    if (e.return_code != SUCCESS) return e;
    if (grid.gravity != 0.0)
        return WRAP_RAISE_ERROR(NOT_IMPLEMENTED_ERROR, "The adjoint does not differentiate the gravity source.");
    HydroGpuAdjoint *ad = calloc(1, sizeof *ad);
    if (!ad) return WRAP_RAISE_ERROR(MEMORY_ERROR, "Failed to allocate the adjoint session.");
    const HydroGpuOptions opt = options ? *options : hydro_gpu_default_options();
    StoringParam none = get_new_storing_param();
    const HydroStepParams params = step_params(ip, &none);
    double *W[4] = { system->density_, system->velocity_x_, system->velocity_y_, system->pressure_ };
    HydroRunOutcome oc;
    if (hydro_adj2d_create(&grid, &opt, &params, num_steps, checkpoint_every, W, &ad->adj, &oc) != 0)
    {
        hydro_adj2d_destroy(ad->adj);
        free(ad);
        return outcome_error(&oc);
    }
    *out = ad;
    return make_success_error_status();
}

ErrorStatus hydro_gpu_adjoint_forward(HydroGpuAdjoint *ad, double *const W_final[4])
{
    HydroRunOutcome oc;
    if (hydro_adj2d_forward(ad->adj, W_final, NULL, &oc) != 0) return outcome_error(&oc);
    return make_success_error_status();
}

ErrorStatus hydro_gpu_adjoint_backward(HydroGpuAdjoint *ad, double *const seed[4], double *const grad[4])
{
    HydroRunOutcome oc;
    if (hydro_adj2d_backward(ad->adj, seed, grad, &oc) != 0) return outcome_error(&oc);
    return make_success_error_status();
}

ErrorStatus hydro_gpu_adjoint_tangent(HydroGpuAdjoint *ad, double *const w0[4], double *const dw0[4],
                                      double *const w_final[4], double *const dw_final[4])
{
    HydroRunOutcome oc;
    if (hydro_adj2d_tangent(ad->adj, w0, dw0, w_final, dw_final, &oc) != 0) return outcome_error(&oc);
    return make_success_error_status();
}

ErrorStatus hydro_gpu_adjoint_replay(HydroGpuAdjoint *ad, double *const w0[4], double *const w_final[4],
                                     unsigned long long *signatures)
{
    HydroRunOutcome oc;
    if (hydro_adj2d_replay(ad->adj, w0, w_final, signatures, 0, &oc) != 0) return outcome_error(&oc);
    return make_success_error_status();
}

ErrorStatus hydro_gpu_adjoint_replay_frozen(HydroGpuAdjoint *ad, double *const w0[4], double *const w_final[4])
{
    HydroRunOutcome oc;
    if (hydro_adj2d_replay(ad->adj, w0, w_final, NULL, 1, &oc) != 0) return outcome_error(&oc);
    return make_success_error_status();
}

ErrorStatus hydro_gpu_adjoint_dt(const HydroGpuAdjoint *ad, double *dt)
{
    if (hydro_adj2d_dt(ad->adj, dt) != 0)
        return WRAP_RAISE_ERROR(VALUE_ERROR, "Run the forward pass first.");
    return make_success_error_status();
}

void hydro_gpu_adjoint_set_tape(HydroGpuAdjoint *ad, int enabled)
{
    hydro_adj2d_set_tape(ad->adj, enabled);
}

void hydro_gpu_adjoint_stats(const HydroGpuAdjoint *ad, HydroGpuAdjointStats *stats)
{
    hydro_adj2d_stats(ad->adj, stats);
}

void hydro_gpu_adjoint_destroy(HydroGpuAdjoint *ad)
{
    if (!ad) return;
    hydro_adj2d_destroy(ad->adj);
    free(ad);
}
