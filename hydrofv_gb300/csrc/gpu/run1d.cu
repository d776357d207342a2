/*
 * run1d.cu -- 1D integrators (Cartesian, cylindrical, spherical) in one
 * persistent CTA.
 *
 * Replaces the time loops of godunov_first_order_1d
 * (src/integrator_godunov_first_order.c:26-261), muscl_hancock_1d
 * (src/integrator_muscl_hancock.c:26-383) and random_choice_1d
 * (src/integrator_random_choice_1d.c:28-290) with their exact / HLLC flux
 * (src/riemann_solver.c:47-97), get_time_step_1d (src/utils.c:28-53),
 * convert_conserved_to_primitive_1d (src/system.c:735-761),
 * set_boundary_condition_1d (src/boundary.c:411-511) and the cylindrical /
 * spherical geometry source (src/source_term.c:14-183).
 *
 * Geometry: face areas and cell volumes are per cell, as system_init sets
 * them (src/system.c:365-529).  As in the reference, the flux through face i
 * updates cell i-1 with surface_area_x[i-1] and cell i with surface_area_x[i]
 * (src/integrator_godunov_first_order.c:182-192).
 *
 * 1D problems are small (the Sod tube of the benchmark configurations has
 * 1000 cells), so the whole run is one launch of one CTA of 1024 threads:
 * per step a block-wide max gives dt, every face flux is computed into a
 * global scratch array, and after a barrier each cell gathers its two faces
 * in the reference's order (+F_left, then -F_right, each (F*dt)*A), then
 * the all-cell U->W conversion and the ghost fill run.  The arrays are
 * L2-resident at these sizes.  The exact solver's Newton (<= 100) and
 * bisection (<= 5000) loops are bounded.  The kernel leaves the loop when
 * the run stops or a snapshot is due (the host stores it and relaunches).
 *
 * Serial-order semantics: the reference's 1D OpenMP loops race on shared
 * cells, so the serial build is the oracle; the gather update here is the
 * serial order.  A flux error in the Godunov integrator stops the run with
 * the state from before the failing step (the reference leaves the partial
 * update); MUSCL-Hancock 1D ignores flux errors as the reference does
 * (src/integrator_muscl_hancock.c:309 overwrites the status).
 *
 * Compiled with --fmad=false (same IEEE operation sequence as the reference).
 */
#include <cuda_runtime.h>
#include <math_constants.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>

#include "gpu_bridge.h"
#include "numerics.cuh"
#include "step_control.h"

using namespace hydro;

namespace {

constexpr int kThreads = 1024;

struct Run1dArgs {
    double *W[3];          /* rho, u, p (padded, nx + 2G) */
    double *U[3];          /* mass, mom, energy */
    double *F[3];          /* face fluxes, index = face (= right cell) */
    double *Lf[3];         /* MUSCL interface states (left of face i at [i]) */
    double *Rf[3];         /* (right of face i at [i]) */
    const double *area;    /* surface_area_x (per cell index) */
    const double *vol;     /* volume */
    const double *mid;     /* mid_points_x */
    HydroStepControl *ctrl;
    HydroStepParams sp;
    GasConst<double> gas;
    int nx, g;
    int bc[2];
    int limiter;
    int solver;            /* RIEMANN_SOLVER_EXACT (1) or _HLLC (2) */
    int scheme;            /* 0: Godunov first order, 1: MUSCL-Hancock, 2: random choice */
    double dx;
    double alpha;          /* 0: Cartesian; 1 cylindrical, 2 spherical (geometry source) */
};

/* src/integrator_random_choice_1d.c:28-43: base-5 van der Corput sequence
 * with digit scrambling a -> 3a mod 5. */
__device__ double van_der_corput(long long n)
{
    double result = 0;
    const int base = 5;
    double bk = 1.0 / (double) base;
    while (n > 0) {
        const int a_i = (int) (n % base);
        const int A_i = (3 * a_i) % 5;
        result += A_i * bk;
        n /= base;
        bk /= (double) base;
    }
    return result;
}

/* src/source_term.c:25-39 */
__device__ __forceinline__ void geometry_rates(double pf, double gm1, double rho, double sm, double se,
                                               double &dm, double &dmom, double &de)
{
    const double p = gm1 * (se - 0.5 * sm * sm / rho);
    dm = pf * sm;
    dmom = pf * sm * sm / rho;
    de = pf * sm * (se + p) / rho;
}

__device__ int face_flux(const Run1dArgs &a, double rl, double ul, double pl, double rr,
                         double ur, double pr, double F[3])
{
    if (a.solver == 1) return exact_flux_1d(a.gas, rl, ul, pl, rr, ur, pr, 0.0, F);
    return hllc_flux_1d(a.gas, rl, ul, pl, rr, ur, pr, F);
}

__device__ double block_max(double v, double *red)
{
    for (int o = 16; o > 0; o >>= 1) {
        const double w = __shfl_xor_sync(0xffffffffu, v, o);
        if (w > v) v = w;
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = (threadIdx.x < kThreads / 32) ? red[threadIdx.x] : -CUDART_INF;
        for (int o = 16; o > 0; o >>= 1) {
            const double w = __shfl_xor_sync(0xffffffffu, v, o);
            if (w > v) v = w;
        }
        if (threadIdx.x == 0) red[0] = v;
    }
    __syncthreads();
    const double r = red[0];
    __syncthreads();
    return r;
}

/* All-cell U -> W (src/system.c:735-761). */
__device__ void convert_all(const Run1dArgs &a, double *const *U, double *const *W, int ntot)
{
    for (int i = threadIdx.x; i < ntot; i += kThreads) {
        const double m = U[0][i];
        const double vol = a.vol[i];
        const double rho = m / vol;
        const double u = U[1][i] / m;
        W[0][i] = rho;
        W[1][i] = u;
        W[2][i] = a.gas.gm1 * (U[2][i] - 0.5 * m * u * u) / vol;
    }
}

/* Ghost fill (src/boundary.c:411-511). */
__device__ void ghost_fill(const Run1dArgs &a, double *const *W, int g, int n)
{
    for (int k = threadIdx.x; k < g; k += kThreads) {
        for (int side = 0; side < 2; side++) {
            const int f = a.bc[side];
            if (f == BC_NONE || (f == BC_PERIODIC && side == 0)) continue;
            if (f == BC_PERIODIC) {
                for (int q = 0; q < 3; q++) W[q][g + n + k] = W[q][g + k];
                for (int q = 0; q < 3; q++) W[q][g - 1 - k] = W[q][g + n - 1 - k];
                continue;
            }
            const int dst = side == 0 ? g - 1 - k : g + n + k;
            const int src = side == 0 ? g + k : g + n - 1 - k;
            W[0][dst] = W[0][src];
            W[1][dst] = (f == BC_REFLECTIVE) ? -W[1][src] : W[1][src];
            W[2][dst] = W[2][src];
        }
    }
}

__global__ void __launch_bounds__(kThreads) run1d_kernel(const Run1dArgs a)
{
    __shared__ double red[kThreads / 32];
    __shared__ int s_err;
    HydroStepControl *ctrl = a.ctrl;
    const int g = a.g, n = a.nx, ntot = n + 2 * g;
    const int tid = threadIdx.x;
    double *const *W = a.W;
    double *const *U = a.U;

    /* at most 65536 steps per launch; the host relaunches while active */
    for (int guard = 0; guard < 65536; guard++) {
        if (!*(volatile int *) &ctrl->active) return;
        const long long ns = ctrl->num_steps;
        const double t = ctrl->t;
        const double tf = ctrl->tf;

        /* ---- dt (src/utils.c:28-53) ---- */
        double smax = -CUDART_INF;
        for (int i = g + tid; i < g + n; i += kThreads) {
            const double s = sound_speed(a.gas, W[0][i], W[2][i]) + fabs(W[1][i]);
            if (s > smax) smax = s;
        }
        smax = block_max(smax, red);
        const double cfl = (ns < a.sp.shrink_steps) ? a.sp.cfl_shrunk : a.sp.cfl;
        double dt = cfl * a.dx / smax;
        if (t + dt > tf) dt = tf - t;
        if (dt == 0.0) {
            if (tid == 0) {
                ctrl->dt = dt;
                ctrl->error_code = DEV_ERR_DT_ZERO;
                ctrl->active = 0;
            }
            return;
        }
        if (tid == 0) s_err = 0;
        __syncthreads();

        /* ---- interface states (MUSCL-Hancock, :159-246) ---- */
        if (a.scheme == 1) {
            for (int i = tid; i < n + 2; i += kThreads) {
                const int k = g + i - 1;
                const double dtA = dt * a.area[k] / a.vol[k];
                const double rho = W[0][k], u = W[1][k], p = W[2][k];
                const double as = sound_speed(a.gas, rho, p);
                double d[3];
                for (int q = 0; q < 3; q++)
                    d[q] = limit_slope_rt(a.limiter, W[q][k] - W[q][k - 1], W[q][k + 1] - W[q][k]);
                double lo[3], hi[3];
                hancock_1d(dtA, rho, u, p, as, d, lo, hi);
                /* cell k's low face is face g+i-1 (its right state); high face is g+i (left state) */
                if (i > 0)
                    for (int q = 0; q < 3; q++) a.Rf[q][g + i - 1] = lo[q];
                if (i < n + 1)
                    for (int q = 0; q < 3; q++) a.Lf[q][g + i] = hi[q];
            }
            __syncthreads();
        }

        if (a.scheme == 2) {
            /* ---- random choice (src/integrator_random_choice_1d.c:157-237): the
             * exact solution of the left or right Riemann problem of each cell,
             * sampled at theta dx / dt or (theta - 1) dx / dt, from a copy of W ---- */
            const double theta = van_der_corput(ns + 1);
            for (int i = tid; i < ntot; i += kThreads)
                for (int q = 0; q < 3; q++) a.Lf[q][i] = W[q][i];
            __syncthreads();
            double *const *T = a.Lf;
            for (int i = g + tid; i <= g + n; i += kThreads) {
                const bool left = theta <= 0.5;
                const int l = left ? i - 1 : i, r = left ? i : i + 1;
                const double speed = left ? theta * a.dx / dt : (theta - 1.0) * a.dx / dt;
                double o[3];
                const int rc = exact_solve_1d(a.gas, T[0][l], T[1][l], T[2][l], T[0][r], T[1][r], T[2][r],
                                              speed, o);
                if (rc != DEV_OK) atomicCAS(&s_err, 0, rc);
                W[0][i] = o[0];
                W[1][i] = o[1];
                W[2][i] = o[2];
            }
            __syncthreads();
            if (s_err) {
                /* the state from before the failing step */
                for (int i = tid; i < ntot; i += kThreads)
                    for (int q = 0; q < 3; q++) W[q][i] = T[q][i];
                __syncthreads();
                if (tid == 0) {
                    ctrl->dt = dt;
                    ctrl->error_code = s_err;
                    ctrl->active = 0;
                }
                return;
            }
            ghost_fill(a, W, g, n);
            __syncthreads();
            /* all-cell W -> U (src/system.c:866-883) */
            for (int i = tid; i < ntot; i += kThreads) {
                const double rho = W[0][i], u = W[1][i], p = W[2][i], vol = a.vol[i];
                const double m = rho * vol;
                U[0][i] = m;
                U[1][i] = m * u;
                U[2][i] = vol * (0.5 * rho * u * u + p / a.gas.gm1);
            }
            __syncthreads();
        } else {
            /* ---- face fluxes: face i between cells i-1 and i, i in [g, g+n] ---- */
            for (int i = g + tid; i <= g + n; i += kThreads) {
                double F[3] = { 0.0, 0.0, 0.0 };
                int rc;
                if (a.scheme == 1)
                    rc = face_flux(a, a.Lf[0][i], a.Lf[1][i], a.Lf[2][i], a.Rf[0][i], a.Rf[1][i],
                                   a.Rf[2][i], F);
                else
                    rc = face_flux(a, W[0][i - 1], W[1][i - 1], W[2][i - 1], W[0][i], W[1][i], W[2][i], F);
                if (rc != DEV_OK && a.scheme == 0) atomicCAS(&s_err, 0, rc);
                for (int q = 0; q < 3; q++) a.F[q][i] = F[q];
            }
            __syncthreads();
            if (s_err) {
                if (tid == 0) {
                    ctrl->dt = dt;
                    ctrl->error_code = s_err;
                    ctrl->active = 0;
                }
                return;
            }

            /* ---- gather update in the serial order ---- */
            for (int c = g - 1 + tid; c <= g + n; c += kThreads) {
                const double A = a.area[c];
                for (int q = 0; q < 3; q++) {
                    double v = U[q][c];
                    if (c >= g) v = v + (a.F[q][c] * dt) * A;          /* face c: c is its right cell */
                    if (c + 1 <= g + n) v = v - (a.F[q][c + 1] * dt) * A; /* face c+1: c is its left cell */
                    U[q][c] = v;
                }
            }
            __syncthreads();
            convert_all(a, U, W, ntot);
            __syncthreads();
            ghost_fill(a, W, g, n);
            __syncthreads();
        }

        /* ---- cylindrical / spherical source, RK4 (src/source_term.c:45-183) ---- */
        if (a.alpha != 0.0) {
            const double gm1 = a.gas.gm1;
            for (int i = g + tid; i < g + n; i += kThreads) {
                const double vol = a.vol[i];
                const double m = U[0][i], mom = U[1][i], E = U[2][i], rho = W[0][i];
                const double pf = -a.alpha * vol / a.mid[i];
                double k1m, k1p, k1e, k2m, k2p, k2e, k3m, k3p, k3e, k4m, k4p, k4e;
                geometry_rates(pf, gm1, rho, mom / vol, E / vol, k1m, k1p, k1e);
                double tm = m + 0.5 * dt * k1m, tp = mom + 0.5 * dt * k1p, te = E + 0.5 * dt * k1e;
                geometry_rates(pf, gm1, tm / vol, tp / vol, te / vol, k2m, k2p, k2e);
                tm = m + 0.5 * dt * k2m;
                tp = mom + 0.5 * dt * k2p;
                te = E + 0.5 * dt * k2e;
                geometry_rates(pf, gm1, tm / vol, tp / vol, te / vol, k3m, k3p, k3e);
                tm = m + dt * k3m;
                tp = mom + dt * k3p;
                te = E + dt * k3e;
                geometry_rates(pf, gm1, tm / vol, tp / vol, te / vol, k4m, k4p, k4e);
                U[0][i] = m + dt * (k1m + 2.0 * k2m + 2.0 * k3m + k4m) / 6.0;
                U[1][i] = mom + dt * (k1p + 2.0 * k2p + 2.0 * k3p + k4p) / 6.0;
                U[2][i] = E + dt * (k1e + 2.0 * k2e + 2.0 * k3e + k4e) / 6.0;
            }
            __syncthreads();
            convert_all(a, U, W, ntot);
            __syncthreads();
            ghost_fill(a, W, g, n);
            __syncthreads();
        }

        /* ---- clock (thread 0 only; everyone re-reads after the barrier) ---- */
        if (tid == 0) {
            const double tn = t + dt;
            const long long nn = ns + 1;
            ctrl->t = tn;
            ctrl->dt = dt;
            ctrl->num_steps = nn;
            int act = (tn < tf) && (ctrl->max_steps < 0 || nn < ctrl->max_steps);
            if (a.sp.is_storing &&
                tn >= a.sp.storing_interval * (double) (ctrl->store_count - a.sp.store_initial_offset + 1)) {
                ctrl->snapshot_due = 1;
                act = 0;
            }
            ctrl->active = act;
            __threadfence_block();
        }
        __syncthreads();
    }
}

}  // namespace

#define CK1(call, what)                                                                      \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            oc->kind = HYDRO_RUN_CUDA_ERROR;                                                 \
            oc->code = (int) e_;                                                             \
            snprintf(oc->message, sizeof oc->message, "CUDA error in %s: %s", what,          \
                     cudaGetErrorString(e_));                                                \
            goto done;                                                                       \
        }                                                                                    \
    } while (0)

extern "C" int hydro_run1d(const HydroGrid1D *grid, double *const Wh[3], double *const Uh[3],
                           const HydroStepParams *sp, double tf, int64 max_steps, int store_count,
                           HydroSnapshotFn snap, void *ctx, const HydroGpuOptions *opt,
                           HydroRunOutcome *oc, HydroGpuStats *stats)
{
    memset(oc, 0, sizeof *oc);
    const auto t0 = std::chrono::steady_clock::now();
    const int ntot = grid->nx + 2 * grid->g;
    const size_t bytes = (size_t) ntot * sizeof(double);
    double *slab = nullptr;
    HydroStepControl *ctrl_d = nullptr;
    HydroStepControl c;
    double *snap_h = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t ev[4] = {};
    float ms_h2d = 0, ms_steps = 0, ms_d2h = 0;
    long long launches = 0;
    int rc = -1;
    Run1dArgs a;
    memset(&a, 0, sizeof a);

    CK1(cudaSetDevice(opt->device), "cudaSetDevice");
    CK1(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate");
    for (auto &e : ev) CK1(cudaEventCreate(&e), "cudaEventCreate");
    CK1(cudaMalloc(&slab, 18 * bytes + sizeof(double)), "cudaMalloc(state)");
    CK1(cudaMalloc(&ctrl_d, sizeof(HydroStepControl)), "cudaMalloc(control)");
    for (int q = 0; q < 3; q++) {
        a.W[q] = slab + q * ntot;
        a.U[q] = slab + (3 + q) * ntot;
        a.F[q] = slab + (6 + q) * ntot;
        a.Lf[q] = slab + (9 + q) * ntot;
        a.Rf[q] = slab + (12 + q) * ntot;
    }
    {
        double *geo = slab + 15 * ntot;   /* area (ntot + 1), volume, mid points */
        CK1(cudaMemcpyAsync(geo, grid->area, bytes + sizeof(double), cudaMemcpyHostToDevice, s), "H2D area");
        CK1(cudaMemcpyAsync(geo + ntot + 1, grid->vol, bytes, cudaMemcpyHostToDevice, s), "H2D volume");
        CK1(cudaMemcpyAsync(geo + 2 * ntot + 1, grid->mid, bytes, cudaMemcpyHostToDevice, s), "H2D mid points");
        a.area = geo;
        a.vol = geo + ntot + 1;
        a.mid = geo + 2 * ntot + 1;
    }
    a.ctrl = ctrl_d;
    a.sp = *sp;
    a.gas = make_gas_const<double>(grid->gamma, grid->tol);
    a.nx = grid->nx;
    a.g = grid->g;
    a.bc[0] = grid->bc[0];
    a.bc[1] = grid->bc[1];
    a.limiter = grid->limiter;
    a.solver = grid->riemann_solver;
    a.scheme = grid->integrator == INTEGRATOR_MUSCL_HANCOCK_1D ? 1
             : grid->integrator == INTEGRATOR_RANDOM_CHOICE_1D ? 2 : 0;
    a.dx = grid->dx;
    a.alpha = grid->alpha;

    CK1(cudaEventRecord(ev[0], s), "cudaEventRecord");
    for (int q = 0; q < 3; q++) {
        CK1(cudaMemcpyAsync(a.W[q], Wh[q], bytes, cudaMemcpyHostToDevice, s), "H2D W");
        CK1(cudaMemcpyAsync(a.U[q], Uh[q], bytes, cudaMemcpyHostToDevice, s), "H2D U");
    }
    CK1(cudaEventRecord(ev[1], s), "cudaEventRecord");
    memset(&c, 0, sizeof c);
    c.tf = tf;
    c.max_steps = max_steps;
    c.store_count = store_count;
    c.active = (0.0 < tf) && (max_steps != 0);
    CK1(cudaMemcpyAsync(ctrl_d, &c, sizeof c, cudaMemcpyHostToDevice, s), "H2D control");
    CK1(cudaStreamSynchronize(s), "upload");
    CK1(cudaEventElapsedTime(&ms_h2d, ev[0], ev[1]), "cudaEventElapsedTime");

    for (;;) {
        if (!c.active) break;
        CK1(cudaEventRecord(ev[2], s), "cudaEventRecord");
        run1d_kernel<<<1, kThreads, 0, s>>>(a);
        launches++;
        CK1(cudaGetLastError(), "run1d kernel");
        CK1(cudaEventRecord(ev[3], s), "cudaEventRecord");
        CK1(cudaMemcpyAsync(&c, ctrl_d, sizeof c, cudaMemcpyDeviceToHost, s), "D2H control");
        CK1(cudaStreamSynchronize(s), "run1d");
        float ms = 0;
        CK1(cudaEventElapsedTime(&ms, ev[2], ev[3]), "cudaEventElapsedTime");
        ms_steps += ms;
        if (c.error_code) break;
        if (c.snapshot_due) {
            if (snap) {
                if (!snap_h) CK1(cudaMallocHost(&snap_h, 3 * bytes), "cudaMallocHost(snapshot)");
                double *Ws[4] = { snap_h, snap_h + ntot, snap_h + 2 * ntot, nullptr };
                for (int q = 0; q < 3; q++)
                    CK1(cudaMemcpyAsync(Ws[q], a.W[q], bytes, cudaMemcpyDeviceToHost, s), "D2H snapshot");
                CK1(cudaStreamSynchronize(s), "snapshot");
                const int src = snap(ctx, Ws, c.num_steps, c.t, c.dt);
                if (src != 0) {
                    oc->kind = HYDRO_RUN_CALLBACK_ERROR;
                    oc->code = src;
                    break;
                }
            }
            c.store_count += 1;
            c.snapshot_due = 0;
            c.active = (c.t < c.tf) && (c.max_steps < 0 || c.num_steps < c.max_steps);
            CK1(cudaMemcpyAsync(ctrl_d, &c, sizeof c, cudaMemcpyHostToDevice, s), "H2D control");
        }
    }
    if (c.num_steps > 0) {
        CK1(cudaEventRecord(ev[0], s), "cudaEventRecord");
        for (int q = 0; q < 3; q++) {
            CK1(cudaMemcpyAsync(Wh[q], a.W[q], bytes, cudaMemcpyDeviceToHost, s), "D2H W");
            CK1(cudaMemcpyAsync(Uh[q], a.U[q], bytes, cudaMemcpyDeviceToHost, s), "D2H U");
        }
        CK1(cudaEventRecord(ev[1], s), "cudaEventRecord");
        CK1(cudaStreamSynchronize(s), "download");
        CK1(cudaEventElapsedTime(&ms_d2h, ev[0], ev[1]), "cudaEventElapsedTime");
    }
    if (c.error_code && oc->kind == 0) {
        oc->kind = HYDRO_RUN_DEVICE_ERROR;
        oc->code = c.error_code;
    }
    rc = (oc->kind == 0) ? 0 : -1;
done:
    oc->num_steps = c.num_steps;
    oc->t = c.t;
    oc->dt = c.dt;
    oc->store_count = c.store_count;
    if (stats) {
        stats->h2d_ms = ms_h2d;
        stats->step_ms = ms_steps;
        stats->d2h_ms = ms_d2h;
        stats->steps = c.num_steps;
        stats->step_launches = launches;
        stats->kernel_launches = launches;
        stats->h2d_bytes = (long long) (6 * bytes);
        stats->d2h_bytes = c.num_steps > 0 ? (long long) (6 * bytes) : 0;
        stats->interior_cells = grid->nx;
        stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    if (s) cudaStreamSynchronize(s);
    for (auto &e : ev)
        if (e) cudaEventDestroy(e);
    cudaFree(slab);
    cudaFree(ctrl_d);
    if (snap_h) cudaFreeHost(snap_h);
    if (s) cudaStreamDestroy(s);
    return rc;
}
