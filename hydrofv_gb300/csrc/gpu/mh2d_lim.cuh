/*
 * mh2d_lim.cuh -- definitions of the per-limiter launchers declared in
 * mh2d_launch.cuh, and the macro that instantiates them for one
 * (precision, limiter).  Included only by the translation units that
 * instantiate step kernels.
 */
#ifndef HYDRO_GPU_MH2D_LIM_CUH
#define HYDRO_GPU_MH2D_LIM_CUH

#include "mh2d_launch.cuh"

namespace hydro {

template <class R, int LIM, int FIRST_ORDER>
cudaError_t mh2d_launch_step_lim(const Mh2dArgs<R> &a, int grid, cudaStream_t s)
{
    if (a.gravity != 0.0)
        mh2d_step_kernel<R, LIM, mh2d_threads<R>(), FIRST_ORDER, false, true><<<grid, mh2d_threads<R>(), 0, s>>>(a);
    else
        mh2d_step_kernel<R, LIM, mh2d_threads<R>(), FIRST_ORDER><<<grid, mh2d_threads<R>(), 0, s>>>(a);
    return cudaGetLastError();
}

template <class R, int LIM>
cudaError_t mh2d_launch_tape_lim(const Mh2dArgs<R> &a, int grid, cudaStream_t s)
{
    mh2d_step_kernel<R, LIM, mh2d_threads<R>(), 0, true><<<grid, mh2d_threads<R>(), 0, s>>>(a);
    return cudaGetLastError();
}

template <class R, int LIM, int FIRST_ORDER>
cudaError_t mh2d_launch_batch_lim(const Mh2dBatchArgs<R> &b, int grid, cudaStream_t s)
{
    mh2d_batch_step_kernel<R, LIM, mh2d_threads<R>(), FIRST_ORDER><<<grid, mh2d_threads<R>(), 0, s>>>(b);
    return cudaGetLastError();
}

template <class R, int LIM, int FIRST_ORDER>
cudaError_t mh2d_step_occupancy(int *per_sm)
{
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, mh2d_step_kernel<R, LIM, mh2d_threads<R>(), FIRST_ORDER>,
                                                         mh2d_threads<R>(), 0);
}

}  // namespace hydro

/* Everything one (precision, limiter, first-order) combination launches. */
#define HYDRO_MH2D_INSTANTIATE(R, LIM, FO)                                                                 \
    template cudaError_t mh2d_launch_step_lim<R, LIM, FO>(const Mh2dArgs<R> &, int, cudaStream_t);        \
    template cudaError_t mh2d_launch_batch_lim<R, LIM, FO>(const Mh2dBatchArgs<R> &, int, cudaStream_t);  \
    template cudaError_t mh2d_step_occupancy<R, LIM, FO>(int *);

#endif
