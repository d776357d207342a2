/*
 * gpu_internal.h -- declarations shared by the CUDA translation units.
 */
#ifndef HYDRO_GPU_INTERNAL_H
#define HYDRO_GPU_INTERNAL_H

#include <cuda_runtime.h>

#include "mh2d_kernel.cuh"

/* Threads per 2D step CTA: a strip of MH2D_THREADS-2 interior columns. */
#define MH2D_THREADS 128

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
