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
