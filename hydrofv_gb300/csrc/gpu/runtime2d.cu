/*
 * runtime2d.cu -- device memory, streams, graphs and the host-side stepping
 * loop for 2D grids (the part of src/integrator_muscl_hancock.c:385-1225
 * that is not arithmetic).
 *
 * Memory: one device slab holds, per field, the padded grid with the same
 * row-major layout as the host arrays (pitch = nx + 2G): U double-buffered
 * (2 x 4 fields), W double-buffered (2 x 5 fields incl. sound speed), a
 * 4-field materialization target for snapshots / download, and optionally
 * a copy of the initial U and W for rewinding.  A 2048^2 FP64 run needs
 * ~0.7 GB; an 8192^2 run ~12 GB.
 *
 * Stepping: all stepping state lives in a device HydroStepControl, so the
 * host only enqueues step kernels.  With a fixed step count every step is
 * enqueued up front (as CUDA-graph replays of a 32-step chunk) and the host
 * waits once; when running to tf the host enqueues chunks sized from the
 * last dt and polls the control block between them.  Steps enqueued past
 * the stop are no-ops (the kernel returns after reading `active`).
 */
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <tuple>
#include <vector>

#include "gpu_bridge.h"
#include "gpu_internal.h"

using namespace hydro;

namespace {

constexpr int kGraphSteps = 32;

void set_cuda_error(HydroRunOutcome *oc, cudaError_t e, const char *what)
{
    if (!oc) return;
    oc->kind = HYDRO_RUN_CUDA_ERROR;
    oc->code = (int) e;
    snprintf(oc->message, sizeof oc->message, "CUDA error in %s: %s", what, cudaGetErrorString(e));
}

#define CK(call, what)                                  \
    do {                                                \
        cudaError_t e_ = (call);                        \
        if (e_ != cudaSuccess) {                        \
            set_cuda_error(oc, e_, what);               \
            return -1;                                  \
        }                                               \
    } while (0)

}  // namespace

struct HydroRun2D {
    HydroGrid2D grid{};
    HydroGpuOptions opt{};
    int device = 0;
    int fp32 = 0;                   /* state precision: 0 FP64 (drop-in), 1 FP32 */
    size_t elem = sizeof(double);   /* bytes per state value */
    cudaStream_t stream = nullptr;
    int tx = 0, ty = 0;
    size_t ncell = 0;
    void *slab = nullptr;
    void *init_slab = nullptr;      /* initial U and W, kept for rewinding */
    void *init_U[4] = {};
    void *init_W[4] = {};
    void *snap_d[4] = {};           /* materialized W (state precision) */
    double *stage_d = nullptr;      /* FP32 form: FP64 staging for transfers (4 fields) */
    double *totals_d = nullptr;     /* conserved totals (4 doubles) */
    double *snap_h = nullptr;       /* pinned, 4 * ncell */
    HydroStepControl *ctrl_d = nullptr;
    HydroStepControl *ctrl_h = nullptr;   /* pinned */
    Mh2dArgs<double> args{};
    Mh2dArgs<float> args32{};
    cudaGraphExec_t graph = nullptr;
    cudaEvent_t ev[6] = {};
    /* asynchronous snapshots: D2H on a side stream, the writer on a host thread */
    cudaStream_t side = nullptr;
    cudaEvent_t snap_ready = nullptr;    /* materialized state complete (main stream) */
    cudaEvent_t snap_copied = nullptr;   /* host copy complete (side stream) */
    std::thread writer;
    int writer_rc = 0;
    long long snapshots_async = 0;
    HydroHostBcFn host_bc = nullptr;  /* custom sides: host boundary routine after every step */
    void *host_bc_ctx = nullptr;
    int custom_mask = 0;              /* bit s: side s (x_min, x_max, y_min, y_max) is custom */
    bool begun = false;
    bool have_initial = false;
    bool pooled = true;               /* state memory from the device's pool (else cudaMalloc) */
    /* statistics */
    double h2d_ms = 0, step_ms = 0, d2h_ms = 0;
    long long step_launches = 0, kernel_launches = 0;
    long long h2d_bytes = 0, d2h_bytes = 0;
};

static void fill_outcome(const HydroRun2D *run, HydroRunOutcome *oc)
{
    oc->num_steps = run->ctrl_h->num_steps;
    oc->t = run->ctrl_h->t;
    oc->dt = run->ctrl_h->dt;
    oc->store_count = run->ctrl_h->store_count;
}

/* Point the per-field arrays of `a` into the slab. */
template <class R>
static void carve(HydroRun2D *run, Mh2dArgs<R> &a)
{
    R *p = static_cast<R *>(run->slab);
    for (int b = 0; b < 2; b++)
        for (int q = 0; q < 4; q++) { a.U[b][q] = p; p += run->ncell; }
    for (int b = 0; b < 2; b++)
        for (int q = 0; q < 5; q++) { a.W[b][q] = p; p += run->ncell; }
    for (int q = 0; q < 4; q++) { run->snap_d[q] = p; p += run->ncell; }
}

template <class R>
static void setup_args(HydroRun2D *run, Mh2dArgs<R> &a, const HydroGrid2D *grid, const HydroGpuOptions *opt)
{
    a.ctrl = run->ctrl_d;
    a.gas = make_gas_const<R>(grid->gamma, grid->tol);
    a.nx = grid->nx;
    a.ny = grid->ny;
    a.g = grid->g;
    a.pitch = run->tx;
    a.strip_w = mh2d_threads<R>() - 2;
    for (int s = 0; s < 4; s++) a.bc[s] = grid->bc[s];
    a.dx = grid->dx;
    a.dy = grid->dy;
    a.area_x = grid->area_x;
    a.area_y = grid->area_y;
    a.vol = grid->vol;
    a.first_order = (grid->integrator == INTEGRATOR_GODUNOV_FIRST_ORDER_2D) ? 1 : 0;
    a.grid_ctas = mh2d_resident_ctas<R>(grid->limiter, a.first_order, run->device);
    /* FP64: guided row chunks (measured on the 2048^2 shear layer: 1287 M
     * against 1257 M with one height).  FP32, at 8 CTAs per SM sharing an SM,
     * does not fit the model's equal workers (10.8 G against 11.1 G): one
     * height from the fill model. */
    if (opt->chunk_rows > 0) {
        a.chunk_h = opt->chunk_rows;
    } else if (sizeof(R) == 8) {
        mh2d_guided_chunks(a.nx, a.ny, a.strip_w, a.grid_ctas, a.chunk_h, a.tail_h, a.tail_rows);
    } else {
        a.chunk_h = mh2d_default_chunk(a.nx, a.ny, a.strip_w, a.grid_ctas);
    }
    a.gravity = grid->gravity;
}

static cudaError_t launch_step(HydroRun2D *run)
{
    return run->fp32 ? mh2d_launch_step<float>(run->args32, run->grid.limiter, run->stream)
                     : mh2d_launch_step<double>(run->args, run->grid.limiter, run->stream);
}

/* The FP64 step's work-item plan for an nx x ny grid on `slots` resident CTAs
 * (guided row chunks), and each item's strip and padded rows as the kernel
 * decodes them (rows: 3 ints per item, or NULL).  Host only; for tests. */
extern "C" int hydro_gpu_chunk_plan(int nx, int ny, int g, int slots, int *h1, int *h2, int *tail,
                                    int *rows, int max_items)
{
    Mh2dArgs<double> a{};
    a.nx = nx;
    a.ny = ny;
    a.g = g;
    a.strip_w = mh2d_threads<double>() - 2;
    mh2d_guided_chunks(nx, ny, a.strip_w, slots, a.chunk_h, a.tail_h, a.tail_rows);
    *h1 = a.chunk_h;
    *h2 = a.tail_h;
    *tail = a.tail_rows;
    const int n = mh2d_n_items(a);
    if (rows) {
        for (int i = 0; i < n && i < max_items; i++)
            mh2d_item_rows(a, i, rows[3 * i], rows[3 * i + 1], rows[3 * i + 2]);
    }
    return n;
}

/*
 * Device memory of the 2D runs comes from one stream-ordered pool per device
 * that keeps what a finished run freed (release threshold: no limit).  A
 * program that calls launch_simulation repeatedly therefore does not map and
 * unmap its 0.7 GB (2048^2, FP64) of state on every call; the memory stays
 * with the process until hydro_gpu_trim_device_memory() or exit.
 */
static std::mutex g_pool_mutex;
static std::map<int, cudaMemPool_t> g_pools;

static cudaError_t device_pool(int dev, cudaMemPool_t *out)
{
    std::lock_guard<std::mutex> lock(g_pool_mutex);
    auto it = g_pools.find(dev);
    if (it != g_pools.end()) {
        *out = it->second;
        return cudaSuccess;
    }
    cudaMemPoolProps props;
    memset(&props, 0, sizeof props);
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool;
    cudaError_t e = cudaMemPoolCreate(&pool, &props);
    if (e != cudaSuccess) return e;
    unsigned long long keep = ~0ull;
    e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    if (e != cudaSuccess) {
        cudaMemPoolDestroy(pool);
        return e;
    }
    g_pools[dev] = pool;
    *out = pool;
    return cudaSuccess;
}

/* Stream-ordered allocation from the device's pool on the run's stream; on a
 * device without memory pools, plain cudaMalloc (run->pooled = false, and
 * the run's teardown frees with cudaFree). */
static cudaError_t pool_alloc(HydroRun2D *run, void **p, size_t bytes)
{
    int supported = 0;
    if (cudaDeviceGetAttribute(&supported, cudaDevAttrMemoryPoolsSupported, run->device) != cudaSuccess ||
        !supported) {
        cudaGetLastError();
        run->pooled = false;
        return cudaMalloc(p, bytes);
    }
    cudaMemPool_t pool;
    const cudaError_t e = device_pool(run->device, &pool);
    if (e != cudaSuccess) return e;
    return cudaMallocFromPoolAsync(p, bytes, pool, run->stream);
}

/*
 * The per-run CUDA objects that do not depend on the grid -- the stream, the
 * timing events, the device and pinned host control blocks and the totals
 * buffer -- are kept per device when a run ends and handed to the next one
 * (creating them, pinned host memory above all, took most of a drop-in
 * call's ~2 ms of set-up).  At most kKeptRuns sets per device.
 */
struct RunResources {
    cudaStream_t stream;
    cudaEvent_t ev[6];
    HydroStepControl *ctrl_d;
    HydroStepControl *ctrl_h;
    double *totals_d;
};
static constexpr size_t kKeptRuns = 4;
static std::mutex g_res_mutex;
static std::map<int, std::vector<RunResources>> g_res;

static bool take_resources(HydroRun2D *run)
{
    std::lock_guard<std::mutex> lock(g_res_mutex);
    auto &v = g_res[run->device];
    if (v.empty()) return false;
    const RunResources r = v.back();
    v.pop_back();
    run->stream = r.stream;
    for (int k = 0; k < 6; k++) run->ev[k] = r.ev[k];
    run->ctrl_d = r.ctrl_d;
    run->ctrl_h = r.ctrl_h;
    run->totals_d = r.totals_d;
    return true;
}

/* Keep the run's resources for the next run (its stream is idle); false if
 * they are incomplete or the device already keeps enough. */
static bool keep_resources(HydroRun2D *run)
{
    if (!run->stream || !run->ctrl_d || !run->ctrl_h || !run->totals_d) return false;
    for (auto e : run->ev)
        if (!e) return false;
    std::lock_guard<std::mutex> lock(g_res_mutex);
    auto &v = g_res[run->device];
    if (v.size() >= kKeptRuns) return false;
    RunResources r;
    r.stream = run->stream;
    for (int k = 0; k < 6; k++) r.ev[k] = run->ev[k];
    r.ctrl_d = run->ctrl_d;
    r.ctrl_h = run->ctrl_h;
    r.totals_d = run->totals_d;
    v.push_back(r);
    return true;
}

extern "C" int hydro_gpu_trim_device_memory(int device)
{
    /* the device first: on failure the kept sets stay where they are */
    if (cudaSetDevice(device) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    std::vector<RunResources> kept;
    {
        std::lock_guard<std::mutex> lock(g_res_mutex);
        kept.swap(g_res[device]);
    }
    cudaMemPool_t pool = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_pool_mutex);
        auto it = g_pools.find(device);
        if (it != g_pools.end()) pool = it->second;
    }
    for (auto &r : kept) {
        for (auto e : r.ev) cudaEventDestroy(e);
        cudaFree(r.totals_d);
        cudaFree(r.ctrl_d);
        cudaFreeHost(r.ctrl_h);
        cudaStreamDestroy(r.stream);
    }
    if (pool && cudaMemPoolTrimTo(pool, 0) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    return 0;
}

extern "C" int hydro_run2d_create(const HydroGrid2D *grid, const HydroGpuOptions *opt,
                                  HydroRun2D **out, HydroRunOutcome *oc)
{
    memset(oc, 0, sizeof *oc);
    *out = nullptr;
    if (grid->integrator != INTEGRATOR_MUSCL_HANCOCK_2D &&
        grid->integrator != INTEGRATOR_GODUNOV_FIRST_ORDER_2D) {
        oc->kind = HYDRO_RUN_UNSUPPORTED;
        snprintf(oc->message, sizeof oc->message,
                 "The GPU 2D path implements muscl_hancock_2d and godunov_first_order_2d.");
        return -1;
    }
    if (grid->nx < grid->g || grid->ny < grid->g) {
        oc->kind = HYDRO_RUN_UNSUPPORTED;
        snprintf(oc->message, sizeof oc->message,
                 "The GPU 2D path needs at least num_ghost_cells_side interior cells per "
                 "direction (got %d x %d, G = %d).", grid->nx, grid->ny, grid->g);
        return -1;
    }
    if (opt->precision != HYDRO_GPU_PRECISION_FP64 && opt->precision != HYDRO_GPU_PRECISION_FP32) {
        oc->kind = HYDRO_RUN_UNSUPPORTED;
        snprintf(oc->message, sizeof oc->message, "Unknown precision %d.", opt->precision);
        return -1;
    }
    HydroRun2D *run = new (std::nothrow) HydroRun2D();
    if (!run) {
        oc->kind = HYDRO_RUN_CUDA_ERROR;
        snprintf(oc->message, sizeof oc->message, "Host allocation failed.");
        return -1;
    }
    run->grid = *grid;
    run->opt = *opt;
    run->device = opt->device;
    run->fp32 = (opt->precision == HYDRO_GPU_PRECISION_FP32);
    run->elem = run->fp32 ? sizeof(float) : sizeof(double);
    run->tx = grid->nx + 2 * grid->g;
    run->ty = grid->ny + 2 * grid->g;
    run->ncell = (size_t) run->tx * (size_t) run->ty;
    *out = run;

    CK(cudaSetDevice(run->device), "cudaSetDevice");
    if (!take_resources(run)) {
        CK(cudaStreamCreateWithFlags(&run->stream, cudaStreamNonBlocking), "cudaStreamCreate");
        for (auto &e : run->ev) CK(cudaEventCreate(&e), "cudaEventCreate");
        CK(cudaMalloc(&run->totals_d, 4 * sizeof(double)), "cudaMalloc(totals)");
        CK(cudaMalloc(&run->ctrl_d, sizeof(HydroStepControl)), "cudaMalloc(control)");
        CK(cudaMallocHost(&run->ctrl_h, sizeof(HydroStepControl)), "cudaMallocHost(control)");
    }
    memset(run->ctrl_h, 0, sizeof(HydroStepControl));

    /* 8 (U) + 10 (W) + 4 (snapshot) fields; the initial copy is separate */
    const size_t nfield = 22;
    CK(pool_alloc(run, &run->slab, nfield * run->ncell * run->elem), "cudaMallocFromPoolAsync(state)");
    if (run->fp32)
        CK(pool_alloc(run, reinterpret_cast<void **>(&run->stage_d), 4 * run->ncell * sizeof(double)),
           "cudaMallocFromPoolAsync(staging)");
    if (run->fp32) {
        carve<float>(run, run->args32);
        setup_args<float>(run, run->args32, grid, opt);
    } else {
        carve<double>(run, run->args);
        setup_args<double>(run, run->args, grid, opt);
    }
    return 0;
}

/* Device field pointers of the active precision, as untyped pointers. */
static void *fieldU(HydroRun2D *run, int b, int q)
{
    return run->fp32 ? (void *) run->args32.U[b][q] : (void *) run->args.U[b][q];
}

static void *fieldW(HydroRun2D *run, int b, int q)
{
    return run->fp32 ? (void *) run->args32.W[b][q] : (void *) run->args.W[b][q];
}

/* Host FP64 arrays -> device fields (converted to FP32 for the FP32 form). */
static int upload_fields(HydroRun2D *run, double *const host[4], void *const dev[4], HydroRunOutcome *oc)
{
    const size_t bytes = run->ncell * sizeof(double);
    for (int q = 0; q < 4; q++) {
        if (!run->fp32) {
            CK(cudaMemcpyAsync(dev[q], host[q], bytes, cudaMemcpyHostToDevice, run->stream), "H2D");
        } else {
            double *st = run->stage_d + q * run->ncell;
            CK(cudaMemcpyAsync(st, host[q], bytes, cudaMemcpyHostToDevice, run->stream), "H2D");
            CK(convert_f64_to_f32(st, static_cast<float *>(dev[q]), (long long) run->ncell, run->stream),
               "convert");
            run->kernel_launches++;
        }
    }
    return 0;
}

/* Device fields -> host FP64 arrays. */
static int download_fields(HydroRun2D *run, void *const dev[4], double *const host[4], HydroRunOutcome *oc)
{
    const size_t bytes = run->ncell * sizeof(double);
    for (int q = 0; q < 4; q++) {
        if (!run->fp32) {
            CK(cudaMemcpyAsync(host[q], dev[q], bytes, cudaMemcpyDeviceToHost, run->stream), "D2H");
        } else {
            double *st = run->stage_d + q * run->ncell;
            CK(convert_f32_to_f64(static_cast<const float *>(dev[q]), st, (long long) run->ncell, run->stream),
               "convert");
            run->kernel_launches++;
            CK(cudaMemcpyAsync(host[q], st, bytes, cudaMemcpyDeviceToHost, run->stream), "D2H");
        }
    }
    return 0;
}

extern "C" int hydro_run2d_upload(HydroRun2D *run, double *const W[4], double *const U[4],
                                  int keep_initial, HydroRunOutcome *oc)
{
    memset(oc, 0, sizeof *oc);
    CK(cudaSetDevice(run->device), "cudaSetDevice");
    const size_t fbytes = run->ncell * run->elem;
    CK(cudaEventRecord(run->ev[0], run->stream), "cudaEventRecord");
    void *u0[4], *w0[4];
    for (int q = 0; q < 4; q++) { u0[q] = fieldU(run, 0, q); w0[q] = fieldW(run, 0, q); }
    if (upload_fields(run, U, u0, oc)) return -1;
    if (upload_fields(run, W, w0, oc)) return -1;
    for (int q = 0; q < 4; q++)
        CK(cudaMemcpyAsync(fieldU(run, 1, q), u0[q], fbytes, cudaMemcpyDeviceToDevice, run->stream), "D2D U");
    if (keep_initial) {
        if (!run->init_slab) {
            CK(pool_alloc(run, &run->init_slab, 8 * fbytes), "cudaMallocFromPoolAsync(initial state)");
            for (int q = 0; q < 4; q++) {
                run->init_U[q] = static_cast<char *>(run->init_slab) + q * fbytes;
                run->init_W[q] = static_cast<char *>(run->init_slab) + (4 + q) * fbytes;
            }
        }
        for (int q = 0; q < 4; q++) {
            CK(cudaMemcpyAsync(run->init_U[q], u0[q], fbytes, cudaMemcpyDeviceToDevice, run->stream), "D2D");
            CK(cudaMemcpyAsync(run->init_W[q], w0[q], fbytes, cudaMemcpyDeviceToDevice, run->stream), "D2D");
        }
        run->have_initial = true;
    }
    CK(cudaEventRecord(run->ev[1], run->stream), "cudaEventRecord");
    CK(cudaEventSynchronize(run->ev[1]), "upload");
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, run->ev[0], run->ev[1]), "cudaEventElapsedTime");
    run->h2d_ms += ms;
    run->h2d_bytes += (long long) (8 * run->ncell * sizeof(double));
    run->begun = false;
    return 0;
}

extern "C" int hydro_run2d_restore(HydroRun2D *run, HydroRunOutcome *oc)
{
    memset(oc, 0, sizeof *oc);
    if (!run->have_initial) {
        oc->kind = HYDRO_RUN_UNSUPPORTED;
        snprintf(oc->message, sizeof oc->message, "No initial state was kept on the device.");
        return -1;
    }
    CK(cudaSetDevice(run->device), "cudaSetDevice");
    const size_t fbytes = run->ncell * run->elem;
    for (int q = 0; q < 4; q++) {
        CK(cudaMemcpyAsync(fieldU(run, 0, q), run->init_U[q], fbytes, cudaMemcpyDeviceToDevice, run->stream), "D2D");
        CK(cudaMemcpyAsync(fieldU(run, 1, q), run->init_U[q], fbytes, cudaMemcpyDeviceToDevice, run->stream), "D2D");
        CK(cudaMemcpyAsync(fieldW(run, 0, q), run->init_W[q], fbytes, cudaMemcpyDeviceToDevice, run->stream), "D2D");
    }
    CK(cudaStreamSynchronize(run->stream), "restore");
    run->begun = false;
    return 0;
}

static int push_control(HydroRun2D *run, HydroRunOutcome *oc)
{
    CK(cudaMemcpyAsync(run->ctrl_d, run->ctrl_h, sizeof(HydroStepControl), cudaMemcpyHostToDevice,
                       run->stream), "H2D control");
    return 0;
}

static int pull_control(HydroRun2D *run, HydroRunOutcome *oc)
{
    CK(cudaMemcpyAsync(run->ctrl_h, run->ctrl_d, sizeof(HydroStepControl), cudaMemcpyDeviceToHost,
                       run->stream), "D2H control");
    CK(cudaStreamSynchronize(run->stream), "step chunk");
    return 0;
}

static int recompute_active(HydroStepControl *c)
{
    return (c->t < c->tf) && (c->max_steps < 0 || c->num_steps < c->max_steps) && !c->snapshot_due &&
           c->error_code == 0;
}

/* ------------------------------------------------------------ autotuner */

/* Work-item shape (rows per item) and persistent grid size are tuned on the
 * run's own state: each candidate runs one warm-up and two timed steps from
 * the initial state (CUDA events), the fastest is kept, the state is rewound
 * and the choice is cached for the process per (precision, limiter, order,
 * grid shape). */
namespace {
std::mutex g_tune_mutex;
std::map<std::tuple<int, int, int, int, int>, std::pair<int, int>> g_tune_cache;
}

static void set_shape(HydroRun2D *run, int chunk, int ctas)
{
    run->args.chunk_h = run->args32.chunk_h = chunk;
    run->args.tail_rows = run->args32.tail_rows = 0;
    run->args.grid_ctas = run->args32.grid_ctas = ctas;
    if (run->graph) {
        cudaGraphExecDestroy(run->graph);
        run->graph = nullptr;
    }
}

static int ensure_initial_copy(HydroRun2D *run, HydroRunOutcome *oc)
{
    const size_t fbytes = run->ncell * run->elem;
    if (!run->init_slab) {
        CK(pool_alloc(run, &run->init_slab, 8 * fbytes), "cudaMallocFromPoolAsync(initial state)");
        for (int q = 0; q < 4; q++) {
            run->init_U[q] = static_cast<char *>(run->init_slab) + q * fbytes;
            run->init_W[q] = static_cast<char *>(run->init_slab) + (4 + q) * fbytes;
        }
    }
    if (!run->have_initial) {
        for (int q = 0; q < 4; q++) {
            CK(cudaMemcpyAsync(run->init_U[q], fieldU(run, 0, q), fbytes, cudaMemcpyDeviceToDevice, run->stream), "D2D");
            CK(cudaMemcpyAsync(run->init_W[q], fieldW(run, 0, q), fbytes, cudaMemcpyDeviceToDevice, run->stream), "D2D");
        }
        run->have_initial = true;
    }
    return 0;
}

static int autotune(HydroRun2D *run, const HydroStepParams *sp, HydroRunOutcome *oc)
{
    const auto key = std::make_tuple(run->fp32, run->grid.limiter, run->args.first_order + 2 * run->args32.first_order,
                                     run->grid.nx, run->grid.ny);
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            set_shape(run, it->second.first, it->second.second);
            return 0;
        }
    }
    if (ensure_initial_copy(run, oc)) return -1;
    const int resident = run->fp32 ? run->args32.grid_ctas : run->args.grid_ctas;
    const int storing = run->args.sp.is_storing;
    run->args.sp.is_storing = run->args32.sp.is_storing = 0;
    const int chunks[] = { 8, 16, 32, 64 };
    int best_chunk = 32, best_ctas = resident;
    float best_ms = 1e30f;
    HydroStepControl *c = run->ctrl_h;
    const unsigned long long ninf = ordered_bits(-INFINITY);
    for (int ci = 0; ci < 4; ci++) {
        for (int half = 0; half < 2; half++) {
            const int ctas = half ? (resident / 2 > 0 ? resident / 2 : 1) : resident;
            set_shape(run, chunks[ci], ctas);
            memset(c, 0, sizeof *c);
            c->tf = 1e300;
            c->max_steps = 3;
            for (int k = 0; k < 3; k++) c->smax[k][0] = c->smax[k][1] = ninf;
            c->active = 1;
            CK(cudaMemcpyAsync(run->ctrl_d, c, sizeof *c, cudaMemcpyHostToDevice, run->stream), "H2D control");
            CK(run->fp32 ? mh2d_launch_prepare<float>(run->args32, run->stream)
                         : mh2d_launch_prepare<double>(run->args, run->stream), "prepare kernel");
            CK(launch_step(run), "step kernel");
            CK(cudaEventRecord(run->ev[2], run->stream), "cudaEventRecord");
            CK(launch_step(run), "step kernel");
            CK(launch_step(run), "step kernel");
            CK(cudaEventRecord(run->ev[3], run->stream), "cudaEventRecord");
            CK(cudaEventSynchronize(run->ev[3]), "autotune");
            run->kernel_launches += 4;
            float ms = 0;
            CK(cudaEventElapsedTime(&ms, run->ev[2], run->ev[3]), "cudaEventElapsedTime");
            if (ms < best_ms) {
                best_ms = ms;
                best_chunk = chunks[ci];
                best_ctas = ctas;
            }
            /* rewind: the buffers the candidate wrote */
            const size_t fbytes = run->ncell * run->elem;
            for (int q = 0; q < 4; q++) {
                CK(cudaMemcpyAsync(fieldU(run, 0, q), run->init_U[q], fbytes, cudaMemcpyDeviceToDevice, run->stream), "D2D");
                CK(cudaMemcpyAsync(fieldU(run, 1, q), run->init_U[q], fbytes, cudaMemcpyDeviceToDevice, run->stream), "D2D");
                CK(cudaMemcpyAsync(fieldW(run, 0, q), run->init_W[q], fbytes, cudaMemcpyDeviceToDevice, run->stream), "D2D");
            }
        }
    }
    set_shape(run, best_chunk, best_ctas);
    run->args.sp.is_storing = run->args32.sp.is_storing = storing;
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tune_cache[key] = std::make_pair(best_chunk, best_ctas);
    return 0;
}

extern "C" int hydro_run2d_begin(HydroRun2D *run, const HydroStepParams *sp, double tf,
                                 int64 max_steps, int store_count, HydroRunOutcome *oc)
{
    memset(oc, 0, sizeof *oc);
    CK(cudaSetDevice(run->device), "cudaSetDevice");
    run->args.sp = *sp;
    run->args32.sp = *sp;
    if (run->opt.autotune && autotune(run, sp, oc)) return -1;
    HydroStepControl *c = run->ctrl_h;
    memset(c, 0, sizeof *c);
    c->tf = tf;
    c->max_steps = max_steps;
    c->store_count = store_count;
    const unsigned long long ninf = ordered_bits(-INFINITY);
    for (int k = 0; k < 3; k++) c->smax[k][0] = c->smax[k][1] = ninf;
    c->active = recompute_active(c);
    if (push_control(run, oc)) return -1;
    CK(run->fp32 ? mh2d_launch_prepare<float>(run->args32, run->stream)
                 : mh2d_launch_prepare<double>(run->args, run->stream), "prepare kernel");
    run->kernel_launches++;
    CK(cudaStreamSynchronize(run->stream), "prepare");
    /* The kernel arguments changed: any recorded graph is stale. */
    if (run->graph) {
        cudaGraphExecDestroy(run->graph);
        run->graph = nullptr;
    }
    run->begun = true;
    fill_outcome(run, oc);
    return 0;
}

extern "C" int hydro_run2d_set_limits(HydroRun2D *run, double tf, int64 max_steps, HydroRunOutcome *oc)
{
    memset(oc, 0, sizeof *oc);
    CK(cudaSetDevice(run->device), "cudaSetDevice");
    if (pull_control(run, oc)) return -1;
    HydroStepControl *c = run->ctrl_h;
    c->tf = tf;
    c->max_steps = max_steps;
    c->active = recompute_active(c);
    if (push_control(run, oc)) return -1;
    CK(cudaStreamSynchronize(run->stream), "set limits");
    fill_outcome(run, oc);
    return 0;
}

extern "C" int hydro_run2d_status(HydroRun2D *run, HydroRunOutcome *oc)
{
    memset(oc, 0, sizeof *oc);
    CK(cudaSetDevice(run->device), "cudaSetDevice");
    if (pull_control(run, oc)) return -1;
    fill_outcome(run, oc);
    return 0;
}

static int record_graph(HydroRun2D *run, HydroRunOutcome *oc)
{
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(run->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    cudaError_t le = cudaSuccess;
    for (int k = 0; k < kGraphSteps && le == cudaSuccess; k++)
        le = launch_step(run);
    cudaError_t ce = cudaStreamEndCapture(run->stream, &g);
    if (le != cudaSuccess) { set_cuda_error(oc, le, "step kernel (capture)"); if (g) cudaGraphDestroy(g); return -1; }
    if (ce != cudaSuccess) { set_cuda_error(oc, ce, "end capture"); return -1; }
    cudaError_t ie = cudaGraphInstantiate(&run->graph, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) { set_cuda_error(oc, ie, "graph instantiate"); return -1; }
    return 0;
}

extern "C" int hydro_run2d_set_host_bc(HydroRun2D *run, HydroHostBcFn fn, void *ctx, HydroRunOutcome *oc)
{
    memset(oc, 0, sizeof *oc);
    int mask = 0;
    for (int s = 0; s < 4; s++)
        if (run->grid.bc[s] == BC_CUSTOM) mask |= 1 << s;
    if (mask && run->fp32) {
        oc->kind = HYDRO_RUN_UNSUPPORTED;
        snprintf(oc->message, sizeof oc->message, "Custom boundary conditions need the FP64 state.");
        return -1;
    }
    run->host_bc = mask ? fn : nullptr;
    run->host_bc_ctx = ctx;
    run->custom_mask = mask;
    return 0;
}

/* After a step: U->W of every cell to the host, the host boundary routine,
 * the ghost bands of the custom sides back into the W the next step reads,
 * and their sound speed (src/integrator_muscl_hancock.c:1121-1130 with the
 * boundary routine on the host). */
static int apply_host_bc(HydroRun2D *run, HydroRunOutcome *oc)
{
    const int buf = (int) (run->ctrl_h->num_steps & 1);
    double *out[4];
    for (int q = 0; q < 4; q++) out[q] = static_cast<double *>(run->snap_d[q]);
    CK(mh2d_launch_convert_all<double>(run->args, buf, out, run->stream), "convert kernel");
    run->kernel_launches++;
    if (!run->snap_h)
        CK(cudaMallocHost(&run->snap_h, 4 * run->ncell * sizeof(double)), "cudaMallocHost(boundary)");
    double *Wh[4];
    for (int q = 0; q < 4; q++) Wh[q] = run->snap_h + q * run->ncell;
    if (download_fields(run, run->snap_d, Wh, oc)) return -1;
    CK(cudaStreamSynchronize(run->stream), "boundary download");
    const int rc = run->host_bc(run->host_bc_ctx, Wh);
    if (rc != 0) {
        oc->kind = HYDRO_RUN_CALLBACK_ERROR;
        oc->code = rc;
        snprintf(oc->message, sizeof oc->message, "The host boundary routine failed.");
        return -1;
    }
    const int g = run->grid.g, nx = run->grid.nx, ny = run->grid.ny, tx = run->tx, ty = run->ty;
    const size_t pitch = (size_t) tx * sizeof(double);
    for (int q = 0; q < 4; q++) {
        double *dst = run->args.W[buf][q];
        const double *src = Wh[q];
        if (run->custom_mask & 1)
            CK(cudaMemcpy2DAsync(dst, pitch, src, pitch, (size_t) g * sizeof(double), (size_t) ty,
                                 cudaMemcpyHostToDevice, run->stream), "H2D boundary");
        if (run->custom_mask & 2)
            CK(cudaMemcpy2DAsync(dst + g + nx, pitch, src + g + nx, pitch, (size_t) g * sizeof(double),
                                 (size_t) ty, cudaMemcpyHostToDevice, run->stream), "H2D boundary");
        if (run->custom_mask & 4)
            CK(cudaMemcpyAsync(dst, src, (size_t) g * pitch, cudaMemcpyHostToDevice, run->stream), "H2D boundary");
        if (run->custom_mask & 8)
            CK(cudaMemcpyAsync(dst + (size_t) (g + ny) * tx, src + (size_t) (g + ny) * tx, (size_t) g * pitch,
                               cudaMemcpyHostToDevice, run->stream), "H2D boundary");
    }
    CK(mh2d_launch_ghost_sound_speed<double>(run->args, buf, run->custom_mask, run->stream), "sound speed kernel");
    run->kernel_launches++;
    return 0;
}

/* Enqueue `k` step kernels. */
static int enqueue_steps(HydroRun2D *run, long long k, HydroRunOutcome *oc)
{
    const bool graphs = run->opt.use_graph && k >= kGraphSteps;
    if (graphs && !run->graph && record_graph(run, oc)) return -1;
    while (k > 0) {
        if (graphs && k >= kGraphSteps) {
            CK(cudaGraphLaunch(run->graph, run->stream), "graph launch");
            k -= kGraphSteps;
            run->step_launches += kGraphSteps;
            run->kernel_launches += kGraphSteps;
        } else {
            CK(launch_step(run), "step kernel");
            k -= 1;
            run->step_launches += 1;
            run->kernel_launches += 1;
        }
    }
    return 0;
}

/* Wait for the snapshot writer thread; its callback status becomes the outcome. */
static int join_writer(HydroRun2D *run, HydroRunOutcome *oc)
{
    if (run->writer.joinable()) run->writer.join();
    if (run->writer_rc != 0) {
        oc->kind = HYDRO_RUN_CALLBACK_ERROR;
        oc->code = run->writer_rc;
        run->writer_rc = 0;
        return -1;
    }
    return 0;
}

/*
 * Snapshot without stopping the stream: the materialized state (and, for
 * the FP32 form, its FP64 conversion) is produced on the main stream; a
 * side stream waits for it and copies it to pinned host memory; a host
 * thread waits for that copy and runs the writer while the main stream
 * steps on.  One snapshot is in flight at a time (the next one, and the
 * end of the run, join the writer first), so the snapshot buffers and the
 * writer's state are never shared.
 */
static int snapshot_async(HydroRun2D *run, HydroSnapshotFn snap, void *ctx, HydroRunOutcome *oc)
{
    if (join_writer(run, oc)) return -1;
    if (!run->side) {
        CK(cudaStreamCreateWithFlags(&run->side, cudaStreamNonBlocking), "cudaStreamCreate(snapshots)");
        CK(cudaEventCreateWithFlags(&run->snap_ready, cudaEventDisableTiming), "cudaEventCreate");
        CK(cudaEventCreateWithFlags(&run->snap_copied, cudaEventDisableTiming), "cudaEventCreate");
    }
    if (!run->snap_h)
        CK(cudaMallocHost(&run->snap_h, 4 * run->ncell * sizeof(double)), "cudaMallocHost(snapshot)");
    const int buf = (int) (run->ctrl_h->num_steps & 1);
    const void *src[4];
    if (run->fp32) {
        float *out[4];
        for (int q = 0; q < 4; q++) out[q] = static_cast<float *>(run->snap_d[q]);
        CK(mh2d_launch_materialize<float>(run->args32, buf, out, run->stream), "materialize kernel");
        for (int q = 0; q < 4; q++) {
            double *st = run->stage_d + q * run->ncell;
            CK(convert_f32_to_f64(out[q], st, (long long) run->ncell, run->stream), "convert");
            src[q] = st;
        }
        run->kernel_launches += 4;
    } else {
        double *out[4];
        for (int q = 0; q < 4; q++) out[q] = static_cast<double *>(run->snap_d[q]);
        CK(mh2d_launch_materialize<double>(run->args, buf, out, run->stream), "materialize kernel");
        for (int q = 0; q < 4; q++) src[q] = out[q];
    }
    run->kernel_launches++;
    CK(cudaEventRecord(run->snap_ready, run->stream), "cudaEventRecord");
    CK(cudaStreamWaitEvent(run->side, run->snap_ready, 0), "cudaStreamWaitEvent");
    const size_t bytes = run->ncell * sizeof(double);
    for (int q = 0; q < 4; q++)
        CK(cudaMemcpyAsync(run->snap_h + q * run->ncell, src[q], bytes, cudaMemcpyDeviceToHost, run->side),
           "D2H snapshot");
    CK(cudaEventRecord(run->snap_copied, run->side), "cudaEventRecord");
    const long long steps = run->ctrl_h->num_steps;
    const double t = run->ctrl_h->t, dt = run->ctrl_h->dt;
    const int device = run->device;
    run->snapshots_async++;
    run->writer = std::thread([run, snap, ctx, steps, t, dt, device]() {
        cudaSetDevice(device);
        if (cudaEventSynchronize(run->snap_copied) != cudaSuccess) {
            run->writer_rc = -1;
            return;
        }
        double *Wh[4];
        for (int q = 0; q < 4; q++) Wh[q] = run->snap_h + q * run->ncell;
        run->writer_rc = snap(ctx, Wh, steps, t, dt);
    });
    return 0;
}

static int materialize_to_host(HydroRun2D *run, double *const W[4], HydroRunOutcome *oc)
{
    const int buf = (int) (run->ctrl_h->num_steps & 1);
    if (run->fp32) {
        float *out[4];
        for (int q = 0; q < 4; q++) out[q] = static_cast<float *>(run->snap_d[q]);
        CK(mh2d_launch_materialize<float>(run->args32, buf, out, run->stream), "materialize kernel");
    } else {
        double *out[4];
        for (int q = 0; q < 4; q++) out[q] = static_cast<double *>(run->snap_d[q]);
        CK(mh2d_launch_materialize<double>(run->args, buf, out, run->stream), "materialize kernel");
    }
    run->kernel_launches++;
    return download_fields(run, run->snap_d, W, oc);
}

extern "C" int hydro_run2d_advance(HydroRun2D *run, HydroSnapshotFn snap, void *ctx,
                                   HydroRunOutcome *oc, double *step_ms)
{
    memset(oc, 0, sizeof *oc);
    CK(cudaSetDevice(run->device), "cudaSetDevice");
    if (!run->begun) {
        oc->kind = HYDRO_RUN_UNSUPPORTED;
        snprintf(oc->message, sizeof oc->message, "Run not begun.");
        return -1;
    }
    HydroStepControl *c = run->ctrl_h;
    double elapsed = 0.0;
    for (;;) {
        if (!c->active) break;
        /* How many steps to enqueue before looking at the control block. */
        const long long remaining = (c->max_steps >= 0) ? c->max_steps - c->num_steps : LLONG_MAX;
        const bool open_ended = !(c->tf < 1e290);   /* stopping by step count only */
        long long k;
        if (run->opt.chunk_steps > 0) {
            k = run->opt.chunk_steps;
        } else if (open_ended && !run->args.sp.is_storing && remaining != LLONG_MAX) {
            k = remaining;
        } else if (c->num_steps == 0 || !(c->dt > 0.0)) {
            k = 16;
        } else {
            double horizon = c->tf - c->t;
            if (run->args.sp.is_storing) {
                const double next = run->args.sp.storing_interval *
                                    (double) (c->store_count - run->args.sp.store_initial_offset + 1);
                if (next - c->t < horizon) horizon = next - c->t;
            }
            double est = horizon / c->dt + 2.0;
            if (!(est < 4096.0)) est = 4096.0;
            k = (long long) est;
        }
        if (k > remaining) k = remaining;
        if (k < 1) k = 1;
        if (run->host_bc) k = 1;   /* the host boundary routine runs after every step */
        const long long steps_before = c->num_steps;
        CK(cudaEventRecord(run->ev[2], run->stream), "cudaEventRecord");
        if (enqueue_steps(run, k, oc)) return -1;
        if (run->host_bc) {
            if (pull_control(run, oc)) return -1;
            if (c->num_steps > steps_before && c->error_code == 0 && apply_host_bc(run, oc)) {
                fill_outcome(run, oc);
                return -1;
            }
        }
        CK(cudaEventRecord(run->ev[3], run->stream), "cudaEventRecord");
        if (pull_control(run, oc)) return -1;
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, run->ev[2], run->ev[3]), "cudaEventElapsedTime");
        elapsed += ms;
        if (c->error_code) {
            fill_outcome(run, oc);
            oc->kind = HYDRO_RUN_DEVICE_ERROR;
            oc->code = c->error_code;
            oc->where = c->error_cell;
            run->step_ms += elapsed;
            if (step_ms) *step_ms = elapsed;
            return -1;
        }
        if (c->snapshot_due) {
            if (snap && !run->opt.sync_snapshots) {
                if (snapshot_async(run, snap, ctx, oc)) {
                    fill_outcome(run, oc);
                    run->step_ms += elapsed;
                    if (step_ms) *step_ms = elapsed;
                    return -1;
                }
            } else if (snap) {
                if (!run->snap_h) {
                    CK(cudaMallocHost(&run->snap_h, 4 * run->ncell * sizeof(double)), "cudaMallocHost(snapshot)");
                }
                double *Wh[4];
                for (int q = 0; q < 4; q++) Wh[q] = run->snap_h + q * run->ncell;
                if (materialize_to_host(run, Wh, oc)) return -1;
                CK(cudaStreamSynchronize(run->stream), "snapshot");
                const int rc = snap(ctx, Wh, c->num_steps, c->t, c->dt);
                if (rc != 0) {
                    fill_outcome(run, oc);
                    oc->kind = HYDRO_RUN_CALLBACK_ERROR;
                    oc->code = rc;
                    run->step_ms += elapsed;
                    if (step_ms) *step_ms = elapsed;
                    return -1;
                }
            }
            c->store_count += 1;
            c->snapshot_due = 0;
            c->active = recompute_active(c);
            if (push_control(run, oc)) return -1;
        }
    }
    run->step_ms += elapsed;
    if (step_ms) *step_ms = elapsed;
    fill_outcome(run, oc);
    if (join_writer(run, oc)) return -1;
    return 0;
}

extern "C" int hydro_run2d_download(HydroRun2D *run, double *const W[4], double *const U[4],
                                    HydroRunOutcome *oc)
{
    memset(oc, 0, sizeof *oc);
    CK(cudaSetDevice(run->device), "cudaSetDevice");
    if (run->writer.joinable()) run->writer.join();   /* the snapshot buffers are reused */
    const int buf = (int) (run->ctrl_h->num_steps & 1);
    const size_t bytes = run->ncell * sizeof(double);
    CK(cudaEventRecord(run->ev[4], run->stream), "cudaEventRecord");
    if (materialize_to_host(run, W, oc)) return -1;
    void *ub[4];
    for (int q = 0; q < 4; q++) ub[q] = fieldU(run, buf, q);
    if (download_fields(run, ub, U, oc)) return -1;
    CK(cudaEventRecord(run->ev[5], run->stream), "cudaEventRecord");
    CK(cudaEventSynchronize(run->ev[5]), "download");
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, run->ev[4], run->ev[5]), "cudaEventElapsedTime");
    run->d2h_ms += ms;
    run->d2h_bytes += (long long) (8 * bytes);
    fill_outcome(run, oc);
    return 0;
}

extern "C" int hydro_run2d_totals(HydroRun2D *run, double totals[4], HydroRunOutcome *oc)
{
    memset(oc, 0, sizeof *oc);
    CK(cudaSetDevice(run->device), "cudaSetDevice");
    if (pull_control(run, oc)) return -1;
    const int buf = (int) (run->ctrl_h->num_steps & 1);
    CK(run->fp32 ? mh2d_launch_totals<float>(run->args32, buf, run->totals_d, run->stream)
                 : mh2d_launch_totals<double>(run->args, buf, run->totals_d, run->stream), "totals kernel");
    run->kernel_launches++;
    CK(cudaMemcpyAsync(totals, run->totals_d, 4 * sizeof(double), cudaMemcpyDeviceToHost, run->stream), "D2H totals");
    CK(cudaStreamSynchronize(run->stream), "totals");
    fill_outcome(run, oc);
    return 0;
}

extern "C" void hydro_run2d_stats(const HydroRun2D *run, HydroGpuStats *st)
{
    st->h2d_ms = run->h2d_ms;
    st->step_ms = run->step_ms;
    st->d2h_ms = run->d2h_ms;
    st->steps = run->ctrl_h ? run->ctrl_h->num_steps : 0;
    st->step_launches = run->step_launches;
    st->kernel_launches = run->kernel_launches;
    st->h2d_bytes = run->h2d_bytes;
    st->d2h_bytes = run->d2h_bytes;
    st->interior_cells = (int64) run->grid.nx * (int64) run->grid.ny;
}

extern "C" void hydro_run2d_destroy(HydroRun2D *run)
{
    if (!run) return;
    cudaSetDevice(run->device);
    if (run->writer.joinable()) run->writer.join();
    if (run->stream) cudaStreamSynchronize(run->stream);
    if (run->side) {
        cudaStreamSynchronize(run->side);
        cudaStreamDestroy(run->side);
    }
    if (run->snap_ready) cudaEventDestroy(run->snap_ready);
    if (run->snap_copied) cudaEventDestroy(run->snap_copied);
    if (run->graph) cudaGraphExecDestroy(run->graph);
    bool idle = false;
    if (run->stream) {
        /* back to the pool, in stream order (the stream is idle here) */
        for (void *m : { run->slab, run->init_slab, static_cast<void *>(run->stage_d) }) {
            if (!m) continue;
            if (run->pooled) cudaFreeAsync(m, run->stream);
            else cudaFree(m);
        }
        idle = cudaStreamSynchronize(run->stream) == cudaSuccess;
    }
    if (run->snap_h) cudaFreeHost(run->snap_h);
    if (!(idle && cudaGetLastError() == cudaSuccess && keep_resources(run))) {
        for (auto &e : run->ev)
            if (e) cudaEventDestroy(e);
        cudaFree(run->totals_d);
        cudaFree(run->ctrl_d);
        if (run->ctrl_h) cudaFreeHost(run->ctrl_h);
        if (run->stream) cudaStreamDestroy(run->stream);
    }
    delete run;
}

extern "C" int hydro_gpu_device_count(void)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}
