/*
 * gpu_internal.h -- declarations shared by the CUDA translation units.
 */
#ifndef HYDRO_GPU_INTERNAL_H
#define HYDRO_GPU_INTERNAL_H

#include <cuda_runtime.h>

#include <algorithm>
#include <functional>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "mh2d_kernel.cuh"


namespace hydro {

/*
 * Rows per work item when the caller sets none.  The step's CTAs are
 * persistent (one per resident slot) and take (strip, row chunk) items from
 * a queue, so a last partial round of items leaves slots idle.  The choice
 * maximises the filled fraction of whole rounds, less the extra y
 * reconstruction an item adds below its first row (about 0.4 of a row's
 * work).  Measured on the FP64 shear layer (608 resident CTAs): 1024^2
 * takes 16 rows (1117 M cell-updates/s against 792 M at 32), 2048^2 takes
 * 12 (1249 M against 1226 M).
 */
inline int mh2d_default_chunk(int nx, int ny, int strip_w, int slots)
{
    static const int cand[] = { 8, 12, 16, 20, 24, 32, 40, 48, 64 };
    if (slots <= 0 || strip_w <= 0) return 32;
    const long long strips = (nx + strip_w - 1) / strip_w;
    int best = 32;
    double best_eff = -1.0;
    for (int c : cand) {
        const long long items = strips * ((ny + c - 1) / c);
        const long long rounds = (items + slots - 1) / slots;
        const double eff = (double) items / (double) (rounds * slots) * (1.0 - 0.4 / c);
        if (eff > best_eff + 1e-9) {
            best_eff = eff;
            best = c;
        }
    }
    return best;
}

/*
 * Guided row chunks: tall items first, short items last.  The step's work
 * items go to the persistent CTAs in queue order, each CTA taking the next
 * item when it is done.  Tall items pay their per-item prologue (about half
 * a row: the rows below the chunk and its first y faces) less often; short
 * items at the end of the queue keep the last round full.  This models the
 * queue as greedy list scheduling of items costing (rows + 0.5) x (strip
 * width + 2 halo columns) on `slots` equal workers, and picks the heights
 * and the split with the smallest makespan (ties: fewer items).  tail_rows
 * = 0 is one of the candidates: a single height.
 */
inline double mh2d_queue_makespan(int nx, int ny, int strip_w, int slots, int h1, int h2, int tail)
{
    std::vector<double> free_at((size_t) slots, 0.0);
    std::make_heap(free_at.begin(), free_at.end(), std::greater<double>());
    const int strips = (nx + strip_w - 1) / strip_w;
    double makespan = 0.0;
    auto chunk = [&](int rows) {
        for (int s = 0; s < strips; s++) {
            const int sw = (s + 1) * strip_w <= nx ? strip_w : nx - s * strip_w;
            std::pop_heap(free_at.begin(), free_at.end(), std::greater<double>());
            double &t = free_at.back();
            t += (rows + 0.5) * (sw + 2) / (double) (strip_w + 2);
            if (t > makespan) makespan = t;
            std::push_heap(free_at.begin(), free_at.end(), std::greater<double>());
        }
    };
    const int big = ny - tail;
    for (int r = 0; r < big; r += h1) chunk(big - r < h1 ? big - r : h1);
    for (int r = big; r < ny; r += h2) chunk(ny - r < h2 ? ny - r : h2);
    return makespan;
}

inline void mh2d_guided_chunks(int nx, int ny, int strip_w, int slots, int &h1, int &h2, int &tail)
{
    /* 40 candidate queues besides the single height; one search per shape
     * (about 4 ms at 2048^2 on one host core), then cached */
    static const int tall[] = { 16, 24, 32, 48, 64 };
    static const int short_h[] = { 4, 8 };
    static const double waves[] = { 0.5, 1.0, 1.5, 2.0 };
    static std::mutex cache_mutex;
    static std::map<std::tuple<int, int, int, int>, std::tuple<int, int, int>> cache;
    const auto key = std::make_tuple(nx, ny, strip_w, slots);
    {
        std::lock_guard<std::mutex> lock(cache_mutex);
        const auto it = cache.find(key);
        if (it != cache.end()) {
            std::tie(h1, h2, tail) = it->second;
            return;
        }
    }
    h1 = mh2d_default_chunk(nx, ny, strip_w, slots);
    h2 = h1;
    tail = 0;
    if (slots <= 0 || strip_w <= 0 || nx <= 0 || ny <= 0) return;
    const int strips = (nx + strip_w - 1) / strip_w;
    double best = mh2d_queue_makespan(nx, ny, strip_w, slots, h1, h1, 0);
    for (int a : tall) {
        for (int b : short_h) {
            if (b >= a) continue;
            for (double w : waves) {
                /* enough short items for about w rounds of the persistent CTAs */
                int t = (int) (w * slots / strips) * b;
                t = ny - ((ny - t) / a) * a;                      /* tall part: whole chunks */
                if (t <= 0 || t >= ny) continue;
                const double m = mh2d_queue_makespan(nx, ny, strip_w, slots, a, b, t);
                if (m < best * (1.0 - 1e-9)) {
                    best = m;
                    h1 = a;
                    h2 = b;
                    tail = t;
                }
            }
        }
    }
    std::lock_guard<std::mutex> lock(cache_mutex);
    cache[key] = std::make_tuple(h1, h2, tail);
}

template <class R>
cudaError_t mh2d_launch_step(const Mh2dArgs<R> &a, int limiter, cudaStream_t s);
template <class R>
cudaError_t mh2d_launch_step_tape(const Mh2dArgs<R> &a, int limiter, cudaStream_t s);
template <class R>
int mh2d_resident_ctas(int limiter, int first_order, int device);
template <class R>
cudaError_t mh2d_launch_batch_step(const Mh2dBatchArgs<R> &b, int limiter, int first_order, int grid,
                                   cudaStream_t s);
template <class R>
cudaError_t mh2d_launch_prepare(const Mh2dArgs<R> &a, cudaStream_t s);
template <class R>
cudaError_t mh2d_launch_materialize(const Mh2dArgs<R> &a, int buf, R *const out[4], cudaStream_t s);
template <class R>
cudaError_t mh2d_launch_totals(const Mh2dArgs<R> &a, int buf, double *out4, cudaStream_t s);
template <class R>
cudaError_t mh2d_launch_convert_all(const Mh2dArgs<R> &a, int buf, R *const out[4], cudaStream_t s);
template <class R>
cudaError_t mh2d_launch_ghost_sound_speed(const Mh2dArgs<R> &a, int buf, int mask, cudaStream_t s);
cudaError_t convert_f64_to_f32(const double *src, float *dst, long long n, cudaStream_t s);
cudaError_t convert_f32_to_f64(const float *src, double *dst, long long n, cudaStream_t s);

}  // namespace hydro

#endif
