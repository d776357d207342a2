/*
 * runtime_batch.cu -- ensembles of independent 2D grids stepped together.
 *
 * Many small grids are a poor fit for one-grid-per-launch stepping: a 128^2
 * grid has 8 work items for 152 SMs.  Here every instance keeps its own
 * padded arrays, its own HydroStepControl (t, dt, CFL maxima, stop criteria,
 * error word) and therefore its own dt, but one persistent launch per step
 * (mh2d_batch_step_kernel) serves the items of all instances from one queue.
 * Instances are stored largest first so the queue ends with small items.
 * The step loop is replayed from a CUDA graph of 32 launches.
 *
 * Memory: one slab holds every instance's 22 fields (U and W double-buffered,
 * the materialization target), a second one the initial U and W for
 * rewinding; FP32 instances stage transfers through an FP64 buffer sized for
 * the largest instance.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <numeric>
#include <vector>

#include "gpu_bridge.h"
#include "gpu_internal.h"

using namespace hydro;

namespace {

constexpr int kGraphSteps = 32;

void set_err(HydroRunOutcome *oc, cudaError_t e, const char *what)
{
    oc->kind = HYDRO_RUN_CUDA_ERROR;
    oc->code = (int) e;
    snprintf(oc->message, sizeof oc->message, "CUDA error in %s: %s", what, cudaGetErrorString(e));
}

#define BK(call, what)                          \
    do {                                        \
        cudaError_t e_ = (call);                \
        if (e_ != cudaSuccess) {                \
            set_err(oc, e_, what);              \
            return -1;                          \
        }                                       \
    } while (0)

}  // namespace

struct HydroBatch2D {
    int n = 0;
    int fp32 = 0;
    size_t elem = sizeof(double);
    int device = 0;
    int limiter = 0, first_order = 0;
    HydroGpuOptions opt{};
    cudaStream_t stream = nullptr;
    std::vector<HydroGrid2D> grids;         /* user order */
    std::vector<int> pos;                   /* user index -> storage position */
    std::vector<size_t> ncell;              /* storage order */
    std::vector<size_t> off;                /* storage order, in elements */
    std::vector<int> item_off;              /* storage order, n + 1 */
    void *slab = nullptr, *init_slab = nullptr;
    double *stage_d = nullptr;
    HydroStepControl *ctrl_d = nullptr;
    HydroStepControl *ctrl_h = nullptr;     /* pinned, n entries */
    HydroBatchControl *bctrl_d = nullptr;
    int *item_off_d = nullptr;
    void *args_d = nullptr;                 /* Mh2dArgs<R>[n] */
    std::vector<Mh2dArgs<double>> a64;
    std::vector<Mh2dArgs<float>> a32;
    int grid_ctas = 0;
    bool tuned = false;
    cudaGraphExec_t graph = nullptr;
    cudaEvent_t ev[2] = {};
    double step_ms = 0;
    long long launches = 0;
};

template <class R>
static void build_args(HydroBatch2D *b, std::vector<Mh2dArgs<R>> &av)
{
    av.assign(b->n, Mh2dArgs<R>());
    for (int u = 0; u < b->n; u++) {
        const int k = b->pos[u];
        const HydroGrid2D &g = b->grids[u];
        Mh2dArgs<R> &a = av[k];
        memset(&a, 0, sizeof a);
        R *p = static_cast<R *>(b->slab) + b->off[k];
        for (int bb = 0; bb < 2; bb++)
            for (int q = 0; q < 4; q++) { a.U[bb][q] = p; p += b->ncell[k]; }
        for (int bb = 0; bb < 2; bb++)
            for (int q = 0; q < 5; q++) { a.W[bb][q] = p; p += b->ncell[k]; }
        a.ctrl = b->ctrl_d + k;
        a.gas = make_gas_const<R>(g.gamma, g.tol);
        a.nx = g.nx;
        a.ny = g.ny;
        a.g = g.g;
        a.pitch = g.nx + 2 * g.g;
        a.strip_w = mh2d_threads<R>() - 2;
        a.chunk_h = b->opt.chunk_rows > 0 ? b->opt.chunk_rows : 32;
        for (int s = 0; s < 4; s++) a.bc[s] = g.bc[s];
        a.dx = g.dx;
        a.dy = g.dy;
        a.area_x = g.area_x;
        a.area_y = g.area_y;
        a.vol = g.vol;
        a.first_order = b->first_order;
    }
}

template <class R>
static R *snap_field(HydroBatch2D *b, int k, int q)
{
    return static_cast<R *>(b->slab) + b->off[k] + (18 + q) * b->ncell[k];
}

extern "C" int hydro_batch2d_create(const HydroGrid2D *grids, int n, const HydroGpuOptions *opt,
                                    HydroBatch2D **out, HydroRunOutcome *oc)
{
    memset(oc, 0, sizeof *oc);
    *out = nullptr;
    if (n < 1) {
        oc->kind = HYDRO_RUN_UNSUPPORTED;
        snprintf(oc->message, sizeof oc->message, "A batch needs at least one instance.");
        return -1;
    }
    for (int i = 0; i < n; i++) {
        if (grids[i].nx < grids[i].g || grids[i].ny < grids[i].g ||
            grids[i].limiter != grids[0].limiter || grids[i].integrator != grids[0].integrator) {
            oc->kind = HYDRO_RUN_UNSUPPORTED;
            snprintf(oc->message, sizeof oc->message,
                     "Instance %d: every instance needs >= G interior cells per direction and the "
                     "same integrator and limiter.", i);
            return -1;
        }
    }
    HydroBatch2D *b = new (std::nothrow) HydroBatch2D();
    if (!b) {
        oc->kind = HYDRO_RUN_CUDA_ERROR;
        snprintf(oc->message, sizeof oc->message, "Host allocation failed.");
        return -1;
    }
    *out = b;
    b->n = n;
    b->opt = *opt;
    b->device = opt->device;
    b->fp32 = opt->precision == HYDRO_GPU_PRECISION_FP32;
    b->elem = b->fp32 ? sizeof(float) : sizeof(double);
    b->limiter = grids[0].limiter;
    b->first_order = grids[0].integrator == INTEGRATOR_GODUNOV_FIRST_ORDER_2D;
    b->grids.assign(grids, grids + n);

    /* storage order: largest first */
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    auto cells = [&](int i) { return (size_t) (grids[i].nx + 2 * grids[i].g) * (grids[i].ny + 2 * grids[i].g); };
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cells(x) > cells(y); });
    b->pos.assign(n, 0);
    for (int k = 0; k < n; k++) b->pos[order[k]] = k;
    b->ncell.resize(n);
    b->off.resize(n);
    b->item_off.assign(n + 1, 0);
    size_t total = 0, max_cells = 0;
    const int chunk_h = opt->chunk_rows > 0 ? opt->chunk_rows : 32;
    for (int k = 0; k < n; k++) {
        const HydroGrid2D &g = grids[order[k]];
        b->ncell[k] = cells(order[k]);
        b->off[k] = total;
        total += 22 * b->ncell[k];
        max_cells = std::max(max_cells, b->ncell[k]);
        const int nt = mh2d_threads_for(b->fp32);
        const int items = ((g.nx + nt - 3) / (nt - 2)) * ((g.ny + chunk_h - 1) / chunk_h);
        b->item_off[k + 1] = b->item_off[k] + items;
    }
    if (b->item_off[n] <= 0 || (long long) b->item_off[n] > INT_MAX / 2) {
        oc->kind = HYDRO_RUN_UNSUPPORTED;
        snprintf(oc->message, sizeof oc->message, "Batch too large.");
        return -1;
    }

    BK(cudaSetDevice(b->device), "cudaSetDevice");
    BK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    for (auto &e : b->ev) BK(cudaEventCreate(&e), "cudaEventCreate");
    BK(cudaMalloc(&b->slab, total * b->elem), "cudaMalloc(batch state)");
    size_t init_total = 0;
    for (int k = 0; k < n; k++) init_total += 8 * b->ncell[k];
    BK(cudaMalloc(&b->init_slab, init_total * b->elem), "cudaMalloc(batch initial state)");
    if (b->fp32) BK(cudaMalloc(&b->stage_d, 4 * max_cells * sizeof(double)), "cudaMalloc(staging)");
    BK(cudaMalloc(&b->ctrl_d, n * sizeof(HydroStepControl)), "cudaMalloc(controls)");
    BK(cudaMallocHost(&b->ctrl_h, n * sizeof(HydroStepControl)), "cudaMallocHost(controls)");
    memset(b->ctrl_h, 0, n * sizeof(HydroStepControl));
    BK(cudaMalloc(&b->bctrl_d, sizeof(HydroBatchControl)), "cudaMalloc(queue)");
    BK(cudaMemsetAsync(b->bctrl_d, 0, sizeof(HydroBatchControl), b->stream), "memset(queue)");
    BK(cudaMalloc(&b->item_off_d, (n + 1) * sizeof(int)), "cudaMalloc(items)");
    BK(cudaMemcpyAsync(b->item_off_d, b->item_off.data(), (n + 1) * sizeof(int), cudaMemcpyHostToDevice,
                       b->stream), "H2D items");
    if (b->fp32) {
        build_args<float>(b, b->a32);
        BK(cudaMalloc(&b->args_d, n * sizeof(Mh2dArgs<float>)), "cudaMalloc(args)");
        b->grid_ctas = mh2d_resident_ctas<float>(b->limiter, b->first_order, b->device);
    } else {
        build_args<double>(b, b->a64);
        BK(cudaMalloc(&b->args_d, n * sizeof(Mh2dArgs<double>)), "cudaMalloc(args)");
        b->grid_ctas = mh2d_resident_ctas<double>(b->limiter, b->first_order, b->device);
    }
    if (b->grid_ctas <= 0 || b->grid_ctas > b->item_off[n]) b->grid_ctas = b->item_off[n];
    BK(cudaStreamSynchronize(b->stream), "batch create");
    return 0;
}

static void *field(HydroBatch2D *b, int k, int f)
{
    return static_cast<char *>(b->slab) + (b->off[k] + (size_t) f * b->ncell[k]) * b->elem;
}

static void *init_field(HydroBatch2D *b, int k, int f)
{
    size_t o = 0;
    for (int j = 0; j < k; j++) o += 8 * b->ncell[j];
    return static_cast<char *>(b->init_slab) + (o + (size_t) f * b->ncell[k]) * b->elem;
}

/* field numbering inside an instance: U[b][q] = 4b+q, W[b][q] = 8+5b+q, snap = 18+q */
extern "C" int hydro_batch2d_upload(HydroBatch2D *b, int i, double *const W[4], double *const U[4],
                                    HydroRunOutcome *oc)
{
    memset(oc, 0, sizeof *oc);
    BK(cudaSetDevice(b->device), "cudaSetDevice");
    const int k = b->pos[i];
    const size_t n = b->ncell[k];
    const size_t bytes = n * sizeof(double), fbytes = n * b->elem;
    for (int src = 0; src < 2; src++) {
        for (int q = 0; q < 4; q++) {
            void *dst = field(b, k, src == 0 ? q : 8 + q);
            const double *h = src == 0 ? U[q] : W[q];
            if (!b->fp32) {
                BK(cudaMemcpyAsync(dst, h, bytes, cudaMemcpyHostToDevice, b->stream), "H2D");
            } else {
                BK(cudaMemcpyAsync(b->stage_d, h, bytes, cudaMemcpyHostToDevice, b->stream), "H2D");
                BK(convert_f64_to_f32(b->stage_d, static_cast<float *>(dst), (long long) n, b->stream), "convert");
                b->launches++;
            }
        }
    }
    for (int q = 0; q < 4; q++) {
        BK(cudaMemcpyAsync(field(b, k, 4 + q), field(b, k, q), fbytes, cudaMemcpyDeviceToDevice, b->stream), "D2D");
        BK(cudaMemcpyAsync(init_field(b, k, q), field(b, k, q), fbytes, cudaMemcpyDeviceToDevice, b->stream), "D2D");
        BK(cudaMemcpyAsync(init_field(b, k, 4 + q), field(b, k, 8 + q), fbytes, cudaMemcpyDeviceToDevice, b->stream), "D2D");
    }
    BK(cudaStreamSynchronize(b->stream), "upload");
    return 0;
}

extern "C" int hydro_batch2d_restore(HydroBatch2D *b, HydroRunOutcome *oc)
{
    memset(oc, 0, sizeof *oc);
    BK(cudaSetDevice(b->device), "cudaSetDevice");
    for (int k = 0; k < b->n; k++) {
        const size_t fbytes = b->ncell[k] * b->elem;
        for (int q = 0; q < 4; q++) {
            BK(cudaMemcpyAsync(field(b, k, q), init_field(b, k, q), fbytes, cudaMemcpyDeviceToDevice, b->stream), "D2D");
            BK(cudaMemcpyAsync(field(b, k, 4 + q), init_field(b, k, q), fbytes, cudaMemcpyDeviceToDevice, b->stream), "D2D");
            BK(cudaMemcpyAsync(field(b, k, 8 + q), init_field(b, k, 4 + q), fbytes, cudaMemcpyDeviceToDevice, b->stream), "D2D");
        }
    }
    BK(cudaStreamSynchronize(b->stream), "restore");
    return 0;
}

static int push(HydroBatch2D *b, HydroRunOutcome *oc)
{
    BK(cudaMemcpyAsync(b->ctrl_d, b->ctrl_h, b->n * sizeof(HydroStepControl), cudaMemcpyHostToDevice,
                       b->stream), "H2D controls");
    return 0;
}

static int pull(HydroBatch2D *b, HydroRunOutcome *oc)
{
    BK(cudaMemcpyAsync(b->ctrl_h, b->ctrl_d, b->n * sizeof(HydroStepControl), cudaMemcpyDeviceToHost,
                       b->stream), "D2H controls");
    BK(cudaStreamSynchronize(b->stream), "batch chunk");
    return 0;
}

static int active(const HydroStepControl &c)
{
    return (c.t < c.tf) && (c.max_steps < 0 || c.num_steps < c.max_steps) && !c.error_code;
}

static cudaError_t launch_batch(HydroBatch2D *b)
{
    if (b->fp32) {
        Mh2dBatchArgs<float> a;
        a.inst = static_cast<const Mh2dArgs<float> *>(b->args_d);
        a.item_off = b->item_off_d;
        a.n_inst = b->n;
        a.total_items = b->item_off[b->n];
        a.bctrl = b->bctrl_d;
        return mh2d_launch_batch_step<float>(a, b->limiter, b->first_order, b->grid_ctas, b->stream);
    }
    Mh2dBatchArgs<double> a;
    a.inst = static_cast<const Mh2dArgs<double> *>(b->args_d);
    a.item_off = b->item_off_d;
    a.n_inst = b->n;
    a.total_items = b->item_off[b->n];
    a.bctrl = b->bctrl_d;
    return mh2d_launch_batch_step<double>(a, b->limiter, b->first_order, b->grid_ctas, b->stream);
}

/* Rows per work item for every instance: item table and arguments. */
static int set_chunk(HydroBatch2D *b, int chunk, int ctas, HydroRunOutcome *oc)
{
    b->item_off[0] = 0;
    for (int k = 0; k < b->n; k++) {
        const int nx = b->fp32 ? b->a32[k].nx : b->a64[k].nx;
        const int ny = b->fp32 ? b->a32[k].ny : b->a64[k].ny;
        const int nt = mh2d_threads_for(b->fp32);
        b->item_off[k + 1] = b->item_off[k] + ((nx + nt - 3) / (nt - 2)) * ((ny + chunk - 1) / chunk);
        if (b->fp32) b->a32[k].chunk_h = chunk;
        else b->a64[k].chunk_h = chunk;
    }
    BK(cudaMemcpyAsync(b->item_off_d, b->item_off.data(), (b->n + 1) * sizeof(int), cudaMemcpyHostToDevice,
                       b->stream), "H2D items");
    if (b->fp32)
        BK(cudaMemcpyAsync(b->args_d, b->a32.data(), b->n * sizeof(Mh2dArgs<float>), cudaMemcpyHostToDevice,
                           b->stream), "H2D args");
    else
        BK(cudaMemcpyAsync(b->args_d, b->a64.data(), b->n * sizeof(Mh2dArgs<double>), cudaMemcpyHostToDevice,
                           b->stream), "H2D args");
    b->grid_ctas = std::min(ctas, b->item_off[b->n]);
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    BK(cudaStreamSynchronize(b->stream), "set chunk");
    return 0;
}

static int batch_prepare_all(HydroBatch2D *b, double tf, int64 max_steps, HydroRunOutcome *oc);

/* Time candidate (rows per item, persistent CTAs) pairs on the batch's own
 * initial state, keep the fastest, rewind (see runtime2d.cu). */
static int batch_autotune(HydroBatch2D *b, HydroRunOutcome *oc)
{
    int resident = b->fp32 ? mh2d_resident_ctas<float>(b->limiter, b->first_order, b->device)
                           : mh2d_resident_ctas<double>(b->limiter, b->first_order, b->device);
    if (resident <= 0) resident = b->grid_ctas;
    const int chunks[] = { 8, 16, 32, 64 };
    int best_chunk = 32, best_ctas = resident;
    float best_ms = 1e30f;
    for (int ci = 0; ci < 4; ci++) {
        for (int half = 0; half < 2; half++) {
            const int ctas = half ? std::max(1, resident / 2) : resident;
            if (set_chunk(b, chunks[ci], ctas, oc)) return -1;
            if (batch_prepare_all(b, 1e300, 3, oc)) return -1;
            BK(launch_batch(b), "batch step kernel");
            BK(cudaEventRecord(b->ev[0], b->stream), "cudaEventRecord");
            BK(launch_batch(b), "batch step kernel");
            BK(launch_batch(b), "batch step kernel");
            BK(cudaEventRecord(b->ev[1], b->stream), "cudaEventRecord");
            BK(cudaEventSynchronize(b->ev[1]), "autotune");
            b->launches += 3;
            float ms = 0;
            BK(cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]), "cudaEventElapsedTime");
            if (ms < best_ms) {
                best_ms = ms;
                best_chunk = chunks[ci];
                best_ctas = ctas;
            }
            if (hydro_batch2d_restore(b, oc)) return -1;
        }
    }
    return set_chunk(b, best_chunk, best_ctas, oc);
}

static int batch_prepare_all(HydroBatch2D *b, double tf, int64 max_steps, HydroRunOutcome *oc)
{
    const unsigned long long ninf = ordered_bits(-INFINITY);
    for (int k = 0; k < b->n; k++) {
        HydroStepControl &c = b->ctrl_h[k];
        memset(&c, 0, sizeof c);
        c.tf = tf;
        c.max_steps = max_steps;
        for (int j = 0; j < 3; j++) c.smax[j][0] = c.smax[j][1] = ninf;
        c.active = active(c);
    }
    if (push(b, oc)) return -1;
    if (b->fp32) {
        for (auto &a : b->a32) BK(mh2d_launch_prepare<float>(a, b->stream), "prepare kernel");
    } else {
        for (auto &a : b->a64) BK(mh2d_launch_prepare<double>(a, b->stream), "prepare kernel");
    }
    b->launches += b->n;
    BK(cudaStreamSynchronize(b->stream), "prepare");
    return 0;
}

extern "C" int hydro_batch2d_begin(HydroBatch2D *b, const HydroStepParams *sp, double tf, int64 max_steps,
                                   HydroRunOutcome *oc)
{
    memset(oc, 0, sizeof *oc);
    BK(cudaSetDevice(b->device), "cudaSetDevice");
    HydroStepParams p = *sp;
    p.is_storing = 0;
    if (b->fp32) {
        for (auto &a : b->a32) a.sp = p;
        BK(cudaMemcpyAsync(b->args_d, b->a32.data(), b->n * sizeof(Mh2dArgs<float>), cudaMemcpyHostToDevice,
                           b->stream), "H2D args");
    } else {
        for (auto &a : b->a64) a.sp = p;
        BK(cudaMemcpyAsync(b->args_d, b->a64.data(), b->n * sizeof(Mh2dArgs<double>), cudaMemcpyHostToDevice,
                           b->stream), "H2D args");
    }
    if (b->opt.autotune && !b->tuned) {
        if (batch_autotune(b, oc)) return -1;
        b->tuned = true;
    }
    return batch_prepare_all(b, tf, max_steps, oc);
}

extern "C" int hydro_batch2d_set_limits(HydroBatch2D *b, double tf, int64 max_steps_more, HydroRunOutcome *oc)
{
    memset(oc, 0, sizeof *oc);
    BK(cudaSetDevice(b->device), "cudaSetDevice");
    if (pull(b, oc)) return -1;
    for (int k = 0; k < b->n; k++) {
        HydroStepControl &c = b->ctrl_h[k];
        c.tf = tf;
        c.max_steps = c.num_steps + max_steps_more;
        c.active = active(c);
    }
    if (push(b, oc)) return -1;
    BK(cudaStreamSynchronize(b->stream), "set limits");
    return 0;
}

extern "C" int hydro_batch2d_advance(HydroBatch2D *b, HydroRunOutcome *oc, double *step_ms)
{
    memset(oc, 0, sizeof *oc);
    BK(cudaSetDevice(b->device), "cudaSetDevice");
    double elapsed = 0;
    for (;;) {
        long long k = 0;
        bool any = false;
        for (int j = 0; j < b->n; j++) {
            const HydroStepControl &c = b->ctrl_h[j];
            if (!c.active) continue;
            any = true;
            long long want;
            if (c.max_steps >= 0 && !(c.tf < 1e290)) want = c.max_steps - c.num_steps;
            else if (c.num_steps == 0 || !(c.dt > 0)) want = 16;
            else {
                double est = (c.tf - c.t) / c.dt + 2.0;
                if (!(est < 4096.0)) est = 4096.0;
                want = (long long) est;
                if (c.max_steps >= 0) want = std::min(want, c.max_steps - c.num_steps);
            }
            k = std::max(k, want);
        }
        if (!any) break;
        if (k < 1) k = 1;
        if (!b->graph && k >= kGraphSteps) {
            cudaGraph_t g = nullptr;
            BK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
            cudaError_t le = cudaSuccess;
            for (int s = 0; s < kGraphSteps && le == cudaSuccess; s++) le = launch_batch(b);
            cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
            if (le != cudaSuccess) { set_err(oc, le, "batch step (capture)"); if (g) cudaGraphDestroy(g); return -1; }
            if (ce != cudaSuccess) { set_err(oc, ce, "end capture"); return -1; }
            cudaError_t ie = cudaGraphInstantiate(&b->graph, g, 0);
            cudaGraphDestroy(g);
            if (ie != cudaSuccess) { set_err(oc, ie, "graph instantiate"); return -1; }
        }
        BK(cudaEventRecord(b->ev[0], b->stream), "cudaEventRecord");
        while (k > 0) {
            if (b->graph && k >= kGraphSteps) {
                BK(cudaGraphLaunch(b->graph, b->stream), "graph launch");
                k -= kGraphSteps;
                b->launches += kGraphSteps;
            } else {
                BK(launch_batch(b), "batch step kernel");
                k -= 1;
                b->launches += 1;
            }
        }
        BK(cudaEventRecord(b->ev[1], b->stream), "cudaEventRecord");
        if (pull(b, oc)) return -1;
        float ms = 0;
        BK(cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]), "cudaEventElapsedTime");
        elapsed += ms;
        for (int j = 0; j < b->n; j++) {
            if (b->ctrl_h[j].error_code) {
                oc->kind = HYDRO_RUN_DEVICE_ERROR;
                oc->code = b->ctrl_h[j].error_code;
                oc->where = j;
            }
        }
        if (oc->kind) break;
    }
    b->step_ms += elapsed;
    if (step_ms) *step_ms = elapsed;
    return oc->kind ? -1 : 0;
}

extern "C" int hydro_batch2d_status(HydroBatch2D *b, int i, HydroRunOutcome *oc)
{
    memset(oc, 0, sizeof *oc);
    const HydroStepControl &c = b->ctrl_h[b->pos[i]];
    oc->num_steps = c.num_steps;
    oc->t = c.t;
    oc->dt = c.dt;
    if (c.error_code) {
        oc->kind = HYDRO_RUN_DEVICE_ERROR;
        oc->code = c.error_code;
    }
    return 0;
}

extern "C" int hydro_batch2d_download(HydroBatch2D *b, int i, double *const W[4], double *const U[4],
                                      HydroRunOutcome *oc)
{
    memset(oc, 0, sizeof *oc);
    BK(cudaSetDevice(b->device), "cudaSetDevice");
    const int k = b->pos[i];
    const size_t n = b->ncell[k], bytes = n * sizeof(double);
    const int buf = (int) (b->ctrl_h[k].num_steps & 1);
    if (b->fp32) {
        float *out[4];
        for (int q = 0; q < 4; q++) out[q] = snap_field<float>(b, k, q);
        BK(mh2d_launch_materialize<float>(b->a32[k], buf, out, b->stream), "materialize kernel");
    } else {
        double *out[4];
        for (int q = 0; q < 4; q++) out[q] = snap_field<double>(b, k, q);
        BK(mh2d_launch_materialize<double>(b->a64[k], buf, out, b->stream), "materialize kernel");
    }
    b->launches++;
    for (int src = 0; src < 2; src++) {
        for (int q = 0; q < 4; q++) {
            const void *dev = field(b, k, src == 0 ? 18 + q : 4 * buf + q);
            double *h = src == 0 ? W[q] : U[q];
            if (!b->fp32) {
                BK(cudaMemcpyAsync(h, dev, bytes, cudaMemcpyDeviceToHost, b->stream), "D2H");
            } else {
                BK(convert_f32_to_f64(static_cast<const float *>(dev), b->stage_d, (long long) n, b->stream), "convert");
                b->launches++;
                BK(cudaMemcpyAsync(h, b->stage_d, bytes, cudaMemcpyDeviceToHost, b->stream), "D2H");
                BK(cudaStreamSynchronize(b->stream), "D2H");
            }
        }
    }
    BK(cudaStreamSynchronize(b->stream), "download");
    return 0;
}

extern "C" void hydro_batch2d_stats(const HydroBatch2D *b, HydroGpuStats *st)
{
    memset(st, 0, sizeof *st);
    st->step_ms = b->step_ms;
    st->kernel_launches = b->launches;
    long long cells = 0;
    for (const auto &g : b->grids) cells += (long long) g.nx * g.ny;
    st->interior_cells = cells;
}

extern "C" void hydro_batch2d_destroy(HydroBatch2D *b)
{
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (auto &e : b->ev)
        if (e) cudaEventDestroy(e);
    cudaFree(b->slab);
    cudaFree(b->init_slab);
    cudaFree(b->stage_d);
    cudaFree(b->ctrl_d);
    if (b->ctrl_h) cudaFreeHost(b->ctrl_h);
    cudaFree(b->bctrl_d);
    cudaFree(b->item_off_d);
    cudaFree(b->args_d);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}
