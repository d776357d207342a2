/*
 * mh2d.cu -- FP64 instantiations of the 2D step and its helper kernels.
 *
 * Compiled with --fmad=false: the FP64 path must issue the same IEEE
 * operations as the reference CPU code, which never contracts a*b+c.
 */
#include "mh2d_launch.cuh"

namespace hydro {

template int mh2d_resident_ctas<double>(int, int, int);
template cudaError_t mh2d_launch_batch_step<double>(const Mh2dBatchArgs<double> &, int, int, int, cudaStream_t);
template cudaError_t mh2d_launch_step<double>(const Mh2dArgs<double> &, int, cudaStream_t);
template cudaError_t mh2d_launch_step_tape<double>(const Mh2dArgs<double> &, int, cudaStream_t);
template cudaError_t mh2d_launch_prepare<double>(const Mh2dArgs<double> &, cudaStream_t);
template cudaError_t mh2d_launch_materialize<double>(const Mh2dArgs<double> &, int,
                                                     double *const[4], cudaStream_t);
template cudaError_t mh2d_launch_totals<double>(const Mh2dArgs<double> &, int, double *, cudaStream_t);
template cudaError_t mh2d_launch_convert_all<double>(const Mh2dArgs<double> &, int, double *const[4], cudaStream_t);
template cudaError_t mh2d_launch_ghost_sound_speed<double>(const Mh2dArgs<double> &, int, int, cudaStream_t);

}  // namespace hydro
