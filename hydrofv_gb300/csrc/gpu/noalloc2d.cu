/*
 * noalloc2d.cu -- a MUSCL-Hancock 2D run that allocates nothing.
 *
 * Who needs it: callers that must not allocate while they run the solver.
 * Examples are programs whose device memory belongs to another allocator (a
 * framework's caching pool, or a budget carved out at start-up, where an
 * extra cudaMalloc can fail or fragment the pool), and latency-sensitive loops
 * that cannot afford cudaFree's implicit device-wide synchronisation.  The
 * regular path (runtime2d.cu) allocates a device slab, a pinned control block,
 * a stream and events per call; this one uses none of them.
 *
 * How: all device state of a run lives in g_noalloc_scratch, a file-scope
 * __device__ array sized for HYDRO_GPU_NOALLOC_MAX_CELLS padded cells (22
 * fields: U and W double-buffered, W with the sound speed, a materialization
 * target; then the control block), about 5.5 MiB that every GPU which loads
 * this library keeps until the process exits.  Host code cannot use the
 * symbol itself (on the host it names a stand-in, not device memory), so the
 * first call on each device, with that device current, asks
 * cudaGetSymbolAddress for the device address and caches it; that first call
 * should therefore come before any stream capture.  Transfers are synchronous
 * cudaMemcpy on the legacy default stream, errors are written into the
 * caller's buffer instead of a heap-allocated traceback, and snapshots are not
 * supported (they would need pinned host buffers).
 *
 * Every call shares the array and it keeps the previous call's contents: the
 * control block is rewritten in full and every field a step reads is
 * uploaded or produced before it is read.  Calls that overlap on the GPU (two
 * host threads, or two streams) race on the array.
 */
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "gpu_internal.h"
#include "hydro_gpu.h"

using namespace hydro;

namespace {

constexpr long long kMaxCells = HYDRO_GPU_NOALLOC_MAX_CELLS;
constexpr int kFields = 22;
constexpr long long kControlDoubles =
    ((long long) sizeof(HydroStepControl) + 255) / 256 * 256 / (long long) sizeof(double);
constexpr long long kScratchDoubles = kFields * kMaxCells + kControlDoubles;

__device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
double *g_scratch_addr[kMaxDevices];   /* device address of the array, per device */

int fail(char *buf, int len, int code, const char *fmt, ...)
{
    if (buf && len > 0) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, (size_t) len, fmt, ap);
        va_end(ap);
    }
    return code;
}

int parse_bc(const char *s)
{
    if (!s) return -1;
    if (!strcmp(s, "none")) return BC_NONE;
    if (!strcmp(s, "reflective")) return BC_REFLECTIVE;
    if (!strcmp(s, "transmissive")) return BC_TRANSMISSIVE;
    if (!strcmp(s, "periodic")) return BC_PERIODIC;
    return -1;
}

int parse_limiter(const char *s)
{
    if (!s) return -1;
    if (!strcmp(s, "minmod")) return LIM_MINMOD;
    if (!strcmp(s, "van_leer")) return LIM_VAN_LEER;
    if (!strcmp(s, "monotonized_central")) return LIM_MC;
    return -1;
}

bool uniform(const double *a, long long n)
{
    for (long long k = 1; k < n; k++)
        if (a[k] != a[0]) return false;
    return true;
}

}  // namespace

#define NA_CK(call, what)                                                                   \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            return fail(errbuf, errlen, FAILURE, "CUDA error in %s: %s", what,              \
                        cudaGetErrorString(e_));                                            \
    } while (0)

extern "C" int hydro_gpu_muscl_hancock_2d_noalloc(
    const BoundaryConditionParam *bcp,
    System *s,
    const IntegratorParam *ip,
    double tf,
    int64 max_steps,
    SimulationStatus *status,
    char *errbuf,
    int errlen)
{
    if (errbuf && errlen > 0) errbuf[0] = '\0';
    if (!bcp || !s || !ip || !status)
        return fail(errbuf, errlen, POINTER_ERROR, "NULL argument.");

    /* ---- validation, without allocating (no tracebacks) ---- */
    if (s->coord_sys_flag_ != COORD_SYS_CARTESIAN_2D)
        return fail(errbuf, errlen, VALUE_ERROR,
                    "Wrong coordinate system. Supported coordinate system: \"cartesian_2d\".");
    if (!ip->integrator || strcmp(ip->integrator, "muscl_hancock_2d"))
        return fail(errbuf, errlen, VALUE_ERROR, "Only \"muscl_hancock_2d\" is supported here.");
    if (!ip->riemann_solver || strcmp(ip->riemann_solver, "riemann_solver_hllc"))
        return fail(errbuf, errlen, VALUE_ERROR, "Only HLLC Riemann solver is available for cartesian 2D.");
    const int limiter = parse_limiter(ip->slope_limiter);
    if (limiter < 0) return fail(errbuf, errlen, VALUE_ERROR, "Slope limiter not recognized.");
    if (!(ip->cfl > 0.0)) return fail(errbuf, errlen, VALUE_ERROR, "CFL number must be positive.");
    if (!(ip->cfl_initial_shrink_factor > 0.0))
        return fail(errbuf, errlen, VALUE_ERROR, "CFL initial shrink factor must be positive.");
    if (ip->cfl_initial_shrink_num_steps <= 0)
        return fail(errbuf, errlen, VALUE_ERROR, "CFL initial shrink number of steps must be positive.");
    if (!(ip->tol > 0.0)) return fail(errbuf, errlen, VALUE_ERROR, "Tolerance must be positive.");
    const char *names[4] = { bcp->boundary_condition_x_min, bcp->boundary_condition_x_max,
                             bcp->boundary_condition_y_min, bcp->boundary_condition_y_max };
    int bc[4];
    for (int k = 0; k < 4; k++) {
        bc[k] = parse_bc(names[k]);
        if (bc[k] < 0)
            return fail(errbuf, errlen, VALUE_ERROR,
                        "Boundary condition not recognized (built-in conditions only).");
    }
    if ((bc[0] == BC_PERIODIC) != (bc[1] == BC_PERIODIC))
        return fail(errbuf, errlen, VALUE_ERROR, "Periodic boundary condition mismatch for x_min and x_max.");
    if ((bc[2] == BC_PERIODIC) != (bc[3] == BC_PERIODIC))
        return fail(errbuf, errlen, VALUE_ERROR, "Periodic boundary condition mismatch for y_min and y_max.");
    if (s->gravity != 0.0)
        return fail(errbuf, errlen, NOT_IMPLEMENTED_ERROR, "A non-zero gravity source is not supported.");
    const int g = s->num_ghost_cells_side, nx = s->num_cells_x, ny = s->num_cells_y;
    if (g < 2) return fail(errbuf, errlen, VALUE_ERROR, "Number of ghost cells must be at least 2.");
    if (nx < g || ny < g)
        return fail(errbuf, errlen, NOT_IMPLEMENTED_ERROR,
                    "Needs at least num_ghost_cells_side interior cells per direction.");
    const long long tx = nx + 2LL * g, ty = ny + 2LL * g;
    const long long ncell = tx * ty;
    if (ncell > kMaxCells)
        return fail(errbuf, errlen, VALUE_ERROR,
                    "Grid of %lld padded cells ((%d+2*%d) x (%d+2*%d)) exceeds the no-allocation "
                    "limit of %lld padded cells (HYDRO_GPU_NOALLOC_MAX_CELLS).",
                    ncell, nx, g, ny, g, kMaxCells);
    if (!uniform(s->surface_area_x_, tx) || !uniform(s->surface_area_y_, ty) ||
        !uniform(s->volume_, ncell))
        return fail(errbuf, errlen, NOT_IMPLEMENTED_ERROR, "Needs uniform face areas and cell volumes.");

    /* ---- the scratch array's device address, set up once per device ---- */
    int dev = 0;
    NA_CK(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return fail(errbuf, errlen, FAILURE, "Device ordinal out of range.");
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        NA_CK(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress");
        g_scratch_addr[dev] = static_cast<double *>(p);
    }
    double *base = g_scratch_addr[dev];

    /* ---- carve the run's buffers out of the array ---- */
    Mh2dArgs<double> a;
    memset(&a, 0, sizeof a);
    double *p = base;
    for (int b = 0; b < 2; b++)
        for (int q = 0; q < 4; q++) { a.U[b][q] = p; p += ncell; }
    for (int b = 0; b < 2; b++)
        for (int q = 0; q < 5; q++) { a.W[b][q] = p; p += ncell; }
    double *snap[4];
    for (int q = 0; q < 4; q++) { snap[q] = p; p += ncell; }
    HydroStepControl *ctrl_d = reinterpret_cast<HydroStepControl *>(base + kFields * kMaxCells);

    a.ctrl = ctrl_d;
    a.gas = make_gas_const<double>(s->gamma, ip->tol);
    a.nx = nx;
    a.ny = ny;
    a.g = g;
    a.pitch = (int) tx;
    a.strip_w = mh2d_threads<double>() - 2;
    a.chunk_h = 64;
    for (int k = 0; k < 4; k++) a.bc[k] = bc[k];
    a.dx = s->dx_;
    a.dy = s->dy_;
    a.area_x = s->surface_area_x_[0];
    a.area_y = s->surface_area_y_[0];
    a.vol = s->volume_[0];
    a.sp.cfl = ip->cfl;
    a.sp.cfl_shrunk = ip->cfl * ip->cfl_initial_shrink_factor;
    a.sp.shrink_steps = ip->cfl_initial_shrink_num_steps;

    /* ---- upload (synchronous, pageable host memory) ---- */
    const size_t bytes = (size_t) ncell * sizeof(double);
    double *const Wh[4] = { s->density_, s->velocity_x_, s->velocity_y_, s->pressure_ };
    double *const Uh[4] = { s->mass_, s->momentum_x_, s->momentum_y_, s->energy_ };
    for (int q = 0; q < 4; q++) {
        NA_CK(cudaMemcpy(a.U[0][q], Uh[q], bytes, cudaMemcpyHostToDevice), "upload U");
        NA_CK(cudaMemcpy(a.U[1][q], Uh[q], bytes, cudaMemcpyHostToDevice), "upload U");
        NA_CK(cudaMemcpy(a.W[0][q], Wh[q], bytes, cudaMemcpyHostToDevice), "upload W");
    }

    /* ---- control block: rewritten in full on every call ---- */
    HydroStepControl c;
    memset(&c, 0, sizeof c);
    c.tf = tf;
    c.max_steps = max_steps;
    const unsigned long long ninf = ordered_bits(-INFINITY);
    for (int k = 0; k < 3; k++) c.smax[k][0] = c.smax[k][1] = ninf;
    c.active = (c.t < c.tf) && (max_steps < 0 || max_steps > 0);
    NA_CK(cudaMemcpy(ctrl_d, &c, sizeof c, cudaMemcpyHostToDevice), "upload control");
    NA_CK(mh2d_launch_prepare<double>(a, 0), "prepare kernel");

    /* ---- step until the device reports a stop ---- */
    while (c.active) {
        const long long remaining = (c.max_steps >= 0) ? c.max_steps - c.num_steps : LLONG_MAX;
        long long k;
        if (!(c.tf < 1e290) && remaining != LLONG_MAX) k = remaining;
        else if (c.num_steps == 0 || !(c.dt > 0.0)) k = 16;
        else {
            double est = (c.tf - c.t) / c.dt + 2.0;
            if (!(est < 4096.0)) est = 4096.0;
            k = (long long) est;
        }
        if (k > remaining) k = remaining;
        if (k < 1) k = 1;
        for (long long i = 0; i < k; i++) NA_CK(mh2d_launch_step<double>(a, limiter, 0), "step kernel");
        NA_CK(cudaMemcpy(&c, ctrl_d, sizeof c, cudaMemcpyDeviceToHost), "read control");
    }
    status->num_steps = c.num_steps;
    status->t = c.t;
    status->dt = c.dt;

    /* ---- hand back the last consistent state ---- */
    if (c.num_steps > 0) {
        const int buf = (int) (c.num_steps & 1);
        NA_CK(mh2d_launch_materialize<double>(a, buf, snap, 0), "materialize kernel");
        for (int q = 0; q < 4; q++) {
            NA_CK(cudaMemcpy(Wh[q], snap[q], bytes, cudaMemcpyDeviceToHost), "download W");
            NA_CK(cudaMemcpy(Uh[q], a.U[buf][q], bytes, cudaMemcpyDeviceToHost), "download U");
        }
    }
    if (c.error_code == DEV_ERR_HLLC_WAVE_SPEED)
        return fail(errbuf, errlen, VALUE_ERROR,
                    "Invalid wave speed for the HLLC riemann solver. Possible fix: use a smaller CFL.");
    if (c.error_code == DEV_ERR_DT_ZERO) return fail(errbuf, errlen, VALUE_ERROR, "dt is zero.");
    if (c.error_code) return fail(errbuf, errlen, FAILURE, "Device error %d.", c.error_code);
    return SUCCESS;
}
