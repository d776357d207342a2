/*
 * run1d.cu -- 1D integrators (Cartesian, cylindrical, spherical) in one
 * persistent thread-block cluster.
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
 * 1000 cells), so the whole run is one launch of one thread-block cluster:
 * 16 CTAs of 256 threads (8 where the device cannot place 16), one per SM,
 * with hardware cluster barriers between the phases of a step.  A single
 * CTA would put every face's exact Riemann solve (Newton iterations, pow)
 * on one SM's FP64 pipe, about as fast as one host core; the cluster spreads
 * the faces over 16 SMs, and four lanes share each exact Riemann solve
 * (quad_exact_solve, quad_exact.cuh).  Per step a cluster-wide max (partials exchanged
 * through distributed shared memory) gives dt, every face flux is computed
 * into a global scratch array, and after a barrier each cell gathers its two
 * faces in the reference's order (+F_left, then -F_right, each (F*dt)*A)
 * and converts U->W, then the ghost fill runs.  The arrays are L2-resident
 * at these sizes.  The exact solver's Newton (<= 100) and
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
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <math_constants.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>

#include "gpu_bridge.h"
#include "numerics.cuh"
#include "quad_exact.cuh"
#include "step_control.h"

using namespace hydro;
namespace cg = cooperative_groups;

namespace {

/* threads per CTA (a multiple of 4: the exact solver's quads); a run is
 * one cluster of up to 16 CTAs, one per SM */
constexpr int kThreads = 256;
/* four lanes per exact Riemann solve (quad_exact_solve) instead of one */
constexpr bool kQuadExact = true;
constexpr int kClusterMax = 16;

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

/* The cluster's threads: a global index and count for the cell and face loops. */
struct Lanes {
    int gt, GT;
};

/* The CTA's maximum of v, written to *part (this CTA's shared memory). */
__device__ void block_partial_max(double v, double *red, double *part)
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
        if (threadIdx.x == 0) *part = v;
    }
}

/* The maximum of every CTA's *part: after a cluster barrier, warp 0 reads
 * the partials through distributed shared memory.  Callers alternate two
 * `part` slots between steps, so no CTA overwrites a slot another may still
 * be reading; a cluster barrier separates the reads from any exit. */
__device__ double cluster_gather_max(double *part, double *red, cg::cluster_group &cl)
{
    cl.sync();
    if (threadIdx.x < 32) {
        double v = (threadIdx.x < (int) cl.num_blocks()) ? *cl.map_shared_rank(part, threadIdx.x) : -CUDART_INF;
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

/* The first nonzero error code of the cluster's CTAs (lowest rank first),
 * from each CTA's `err` slot, after a cluster barrier. */
__device__ int cluster_error(int *err, int *bcast, cg::cluster_group &cl)
{
    cl.sync();
    if (threadIdx.x < 32) {
        const int e = (threadIdx.x < (int) cl.num_blocks()) ? *cl.map_shared_rank(err, threadIdx.x) : 0;
        const unsigned m = __ballot_sync(0xffffffffu, e != 0);
        const int first = __shfl_sync(0xffffffffu, e, m ? __ffs(m) - 1 : 0);
        if (threadIdx.x == 0) *bcast = first;
    }
    __syncthreads();
    const int r = *bcast;
    __syncthreads();
    return r;
}

/* All-cell U -> W (src/system.c:735-761). */
__device__ void convert_all(const Run1dArgs &a, double *const *U, double *const *W, int ntot, Lanes L)
{
    for (int i = L.gt; i < ntot; i += L.GT) {
        const double m = U[0][i];
        const double vol = a.vol[i];
        const double rho = dv(m, vol);
        const double u = dv(U[1][i], m);
        W[0][i] = rho;
        W[1][i] = u;
        W[2][i] = dv(a.gas.gm1 * (U[2][i] - 0.5 * m * u * u), vol);
    }
}

/* Ghost fill (src/boundary.c:411-511). */
__device__ void ghost_fill(const Run1dArgs &a, double *const *W, int g, int n, Lanes L)
{
    for (int k = L.gt; k < g; k += L.GT) {
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

/* Every phase boundary is a cluster barrier: it orders the phase's global
 * writes (release) before the next phase's reads on any SM of the cluster
 * (acquire).  Every exit is taken by all CTAs at the same point, after a
 * cluster barrier that follows the last distributed-shared-memory read. */
__global__ void __launch_bounds__(kThreads) run1d_kernel(const Run1dArgs a)
{
    __shared__ double red[kThreads / 32];
    __shared__ double part[2];
    __shared__ int errs[2];
    __shared__ int s_err;
    cg::cluster_group cl = cg::this_cluster();
    const Lanes L{ (int) cl.block_rank() * kThreads + (int) threadIdx.x, (int) cl.num_blocks() * kThreads };
    const bool leader = cl.block_rank() == 0 && threadIdx.x == 0;
    const Quad Q = make_quad();
    volatile HydroStepControl *ctrl = a.ctrl;
    const int g = a.g, n = a.nx, ntot = n + 2 * g;
    const int tid = threadIdx.x;
    double *const *W = a.W;
    double *const *U = a.U;

    /* The control state is constant during a launch or advanced identically
     * by every CTA (dt is cluster-uniform), so it lives in registers; the
     * leader writes t, dt, the step count and the stop flags back each step
     * for the host. */
    if (!ctrl->active) return;
    const double tf = ctrl->tf;
    const long long max_steps = ctrl->max_steps;
    const int store_count = ctrl->store_count;
    long long ns = ctrl->num_steps;
    double t = ctrl->t;
    /* Godunov or MUSCL-Hancock on a Cartesian grid: the final per-cell loop
     * also writes the ghost cells (each from its source cell, by the thread
     * that converts that cell) and the next step's partial maximum of
     * a + |u|, so a step needs two cluster barriers */
    const bool fused = a.scheme != 2 && a.alpha == 0.0;
    const bool periodic = a.bc[1] == BC_PERIODIC;
    const bool ghost_l = periodic || (a.bc[0] != BC_NONE && a.bc[0] != BC_PERIODIC);
    const bool ghost_r = a.bc[1] != BC_NONE;
    bool have_part = false;

    /* at most 65536 steps per launch; the host relaunches while active */
    for (int guard = 0; guard < 65536; guard++) {
        const int buf = guard & 1;
        if (tid == 0) errs[buf] = 0;

        /* ---- dt (src/utils.c:28-53) ---- */
        if (!have_part) {
            double smax = -CUDART_INF;
            for (int i = g + L.gt; i < g + n; i += L.GT) {
                const double s = sound_speed(a.gas, W[0][i], W[2][i]) + fabs(W[1][i]);
                if (s > smax) smax = s;
            }
            block_partial_max(smax, red, &part[buf]);
        }
        const double smax = cluster_gather_max(&part[buf], red, cl);
        const double cfl = (ns < a.sp.shrink_steps) ? a.sp.cfl_shrunk : a.sp.cfl;
        double dt = dv(cfl * a.dx, smax);
        if (t + dt > tf) dt = tf - t;
        if (dt == 0.0) {
            if (leader) {
                ctrl->dt = dt;
                ctrl->error_code = DEV_ERR_DT_ZERO;
                ctrl->active = 0;
            }
            cl.sync();
            return;
        }

        /* ---- interface states (MUSCL-Hancock, :159-246) ---- */
        if (a.scheme == 1) {
            for (int i = L.gt; i < n + 2; i += L.GT) {
                const int k = g + i - 1;
                const double dtA = dv(dt * a.area[k], a.vol[k]);
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
            cl.sync();
        }

        if (a.scheme == 2) {
            /* ---- random choice (src/integrator_random_choice_1d.c:157-237): the
             * exact solution of the left or right Riemann problem of each cell,
             * sampled at theta dx / dt or (theta - 1) dx / dt, from a copy of W ---- */
            const double theta = van_der_corput(ns + 1);
            for (int i = L.gt; i < ntot; i += L.GT)
                for (int q = 0; q < 3; q++) a.Lf[q][i] = W[q][i];
            cl.sync();
            double *const *T = a.Lf;
            const int c0 = kQuadExact ? (L.gt >> 2) : L.gt, cs = kQuadExact ? (L.GT >> 2) : L.GT;
            for (int i = g + c0; i <= g + n; i += cs) {
                const bool left = theta <= 0.5;
                const int l = left ? i - 1 : i, r = left ? i : i + 1;
                const double speed = left ? dv(theta * a.dx, dt) : dv((theta - 1.0) * a.dx, dt);
                double o[3];
                const int rc = kQuadExact
                    ? quad_exact_solve(Q, a.gas, T[0][l], T[1][l], T[2][l], T[0][r], T[1][r], T[2][r], speed, o,
                                       a.ctrl->bisect_marks)
                    : exact_solve_1d(a.gas, T[0][l], T[1][l], T[2][l], T[0][r], T[1][r], T[2][r], speed, o,
                                     a.ctrl->bisect_marks);
                if (!kQuadExact || Q.q == 0) {
                    if (rc != DEV_OK) atomicCAS(&errs[buf], 0, rc);
                    W[0][i] = o[0];
                    W[1][i] = o[1];
                    W[2][i] = o[2];
                }
            }
            const int err = cluster_error(&errs[buf], &s_err, cl);
            if (err) {
                /* the state from before the failing step */
                for (int i = L.gt; i < ntot; i += L.GT)
                    for (int q = 0; q < 3; q++) W[q][i] = T[q][i];
                if (leader) {
                    ctrl->dt = dt;
                    ctrl->error_code = err;
                    ctrl->active = 0;
                }
                cl.sync();
                return;
            }
            ghost_fill(a, W, g, n, L);
            cl.sync();
            /* all-cell W -> U (src/system.c:866-883) */
            for (int i = L.gt; i < ntot; i += L.GT) {
                const double rho = W[0][i], u = W[1][i], p = W[2][i], vol = a.vol[i];
                const double m = rho * vol;
                U[0][i] = m;
                U[1][i] = m * u;
                U[2][i] = vol * (0.5 * rho * u * u + dv(p, a.gas.gm1));
            }
            cl.sync();
        } else {
            /* ---- face fluxes: face i between cells i-1 and i, i in [g, g+n];
             * the exact solver takes a quad of lanes per face, HLLC one ---- */
            const bool quad = kQuadExact && a.solver == 1;
            const int f0 = quad ? (L.gt >> 2) : L.gt, fs = quad ? (L.GT >> 2) : L.GT;
            for (int i = g + f0; i <= g + n; i += fs) {
                double F[3] = { 0.0, 0.0, 0.0 };
                double *const *sl = a.scheme == 1 ? a.Lf : W;
                double *const *sr = a.scheme == 1 ? a.Rf : W;
                const int il = a.scheme == 1 ? i : i - 1;
                const double rl = sl[0][il], ul = sl[1][il], pl = sl[2][il];
                const double rr = sr[0][i], ur = sr[1][i], pr = sr[2][i];
                const int rc = quad ? quad_exact_flux(Q, a.gas, rl, ul, pl, rr, ur, pr, F, a.ctrl->bisect_marks)
                             : a.solver == 1 ? exact_flux_1d(a.gas, rl, ul, pl, rr, ur, pr, 0.0, F, a.ctrl->bisect_marks)
                                             : hllc_flux_1d(a.gas, rl, ul, pl, rr, ur, pr, F);
                if (!quad || Q.q == 0) {
                    if (rc != DEV_OK && a.scheme == 0) atomicCAS(&errs[buf], 0, rc);
                    for (int q = 0; q < 3; q++) a.F[q][i] = F[q];
                }
            }
            const int err = cluster_error(&errs[buf], &s_err, cl);
            if (err) {
                if (leader) {
                    ctrl->dt = dt;
                    ctrl->error_code = err;
                    ctrl->active = 0;
                }
                cl.sync();
                return;
            }

            /* ---- gather update in the serial order, then U -> W of the same
             * cell (the conversion reads only the cell's own U, which this
             * thread just wrote; cells outside the update range keep U) ---- */
            double snext = -CUDART_INF;
            for (int c = L.gt; c < ntot; c += L.GT) {
                if (c >= g - 1 && c <= g + n) {
                    const double A = a.area[c];
                    for (int q = 0; q < 3; q++) {
                        double v = U[q][c];
                        if (c >= g) v = v + (a.F[q][c] * dt) * A;          /* face c: c is its right cell */
                        if (c + 1 <= g + n) v = v - (a.F[q][c + 1] * dt) * A; /* face c+1: c is its left cell */
                        U[q][c] = v;
                    }
                }
                /* a ghost cell that the boundary routine fills keeps only its U */
                if (fused && ((c < g && ghost_l) || (c >= g + n && ghost_r))) continue;
                const double m = U[0][c];
                const double vol = a.vol[c];
                const double rho = dv(m, vol);
                const double u = dv(U[1][c], m);
                const double p = dv(a.gas.gm1 * (U[2][c] - 0.5 * m * u * u), vol);
                W[0][c] = rho;
                W[1][c] = u;
                W[2][c] = p;
                if (fused && c >= g && c < g + n) {
                    /* the ghost cells filled from this cell (src/boundary.c:411-511:
                     * the left side mirrors cell g + k into g - 1 - k, the right
                     * side cell g + n - 1 - k into g + n + k; a periodic right
                     * side copies both ways instead) */
                    const int kl = c - g, kr = g + n - 1 - c;
                    if (kl < g) {
                        if (periodic) {
                            W[0][g + n + kl] = rho; W[1][g + n + kl] = u; W[2][g + n + kl] = p;
                        } else if (ghost_l) {
                            W[0][g - 1 - kl] = rho;
                            W[1][g - 1 - kl] = (a.bc[0] == BC_REFLECTIVE) ? -u : u;
                            W[2][g - 1 - kl] = p;
                        }
                    }
                    if (kr < g) {
                        if (periodic) {
                            W[0][g - 1 - kr] = rho; W[1][g - 1 - kr] = u; W[2][g - 1 - kr] = p;
                        } else if (ghost_r) {
                            W[0][g + n + kr] = rho;
                            W[1][g + n + kr] = (a.bc[1] == BC_REFLECTIVE) ? -u : u;
                            W[2][g + n + kr] = p;
                        }
                    }
                    const double s = sound_speed(a.gas, rho, p) + fabs(u);
                    if (s > snext) snext = s;
                }
            }
            if (fused) {
                block_partial_max(snext, red, &part[buf ^ 1]);
            } else {
                cl.sync();
                ghost_fill(a, W, g, n, L);
                cl.sync();
            }
        }

        /* ---- cylindrical / spherical source, RK4 (src/source_term.c:45-183) ---- */
        if (a.alpha != 0.0) {
            const double gm1 = a.gas.gm1;
            for (int i = g + L.gt; i < g + n; i += L.GT) {
                const double vol = a.vol[i];
                const double m = U[0][i], mom = U[1][i], E = U[2][i], rho = W[0][i];
                double mm = m, mp = mom, me = E;
                geometry_source_rk4(dv(-a.alpha * vol, a.mid[i]), gm1, vol, dt, rho, mm, mp, me);
                U[0][i] = mm;
                U[1][i] = mp;
                U[2][i] = me;
            }
            cl.sync();
            convert_all(a, U, W, ntot, L);
            cl.sync();
            ghost_fill(a, W, g, n, L);
            cl.sync();
        }

        /* ---- clock: every thread advances its copy; the leader publishes it ---- */
        t = t + dt;
        ns = ns + 1;
        int act = (t < tf) && (max_steps < 0 || ns < max_steps);
        bool snap = false;
        if (a.sp.is_storing &&
            t >= a.sp.storing_interval * (double) (store_count - a.sp.store_initial_offset + 1)) {
            snap = true;
            act = 0;
        }
        if (leader) {
            ctrl->t = t;
            ctrl->dt = dt;
            ctrl->num_steps = ns;
            if (snap) ctrl->snapshot_due = 1;
            ctrl->active = act;
        }
        have_part = fused;
        /* the fused path's next barrier is the dt gather at the top */
        if (!act || !fused) cl.sync();
        if (!act) return;
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

/* The largest cluster (16, 8, ... CTAs of kThreads) that this device can
 * place: 16 needs the non-portable cluster size. */
int run1d_cluster_size()
{
    cudaFuncSetAttribute(run1d_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    for (int c = kClusterMax; c > 1; c /= 2) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(c);
        cfg.blockDim = dim3(kThreads);
        cudaLaunchAttribute at;
        at.id = cudaLaunchAttributeClusterDimension;
        at.val.clusterDim.x = c;
        at.val.clusterDim.y = 1;
        at.val.clusterDim.z = 1;
        cfg.attrs = &at;
        cfg.numAttrs = 1;
        int num = 0;
        if (cudaOccupancyMaxActiveClusters(&num, run1d_kernel, &cfg) == cudaSuccess && num > 0) return c;
        cudaGetLastError();
    }
    return 1;
}

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
    memset(&c, 0, sizeof c);
    cudaLaunchConfig_t lcfg = {};
    cudaLaunchAttribute lattr;
    memset(&lattr, 0, sizeof lattr);

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

    {
        const int cs = run1d_cluster_size();
        lcfg.gridDim = dim3(cs);
        lcfg.blockDim = dim3(kThreads);
        lcfg.stream = s;
        lattr.id = cudaLaunchAttributeClusterDimension;
        lattr.val.clusterDim.x = cs;
        lattr.val.clusterDim.y = 1;
        lattr.val.clusterDim.z = 1;
        lcfg.attrs = &lattr;
        lcfg.numAttrs = 1;
    }
    for (;;) {
        if (!c.active) break;
        CK1(cudaEventRecord(ev[2], s), "cudaEventRecord");
        CK1(cudaLaunchKernelEx(&lcfg, run1d_kernel, a), "run1d launch");
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
    for (int k = 0; k < 10; k++) oc->bisect_marks[k] = c.bisect_marks[k];
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
