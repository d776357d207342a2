/*
 * mh2d_lim_vanleer.cu -- FP64 step kernels with the van Leer limiter: single grid
 * (with and without gravity), adjoint tape and batched forms.
 *
 * Compiled with --fmad=false: the FP64 path must issue the same IEEE
 * operations as the reference CPU code, which never contracts a*b+c.
 */
#include "mh2d_lim.cuh"

namespace hydro {

HYDRO_MH2D_INSTANTIATE(double, LIM_VAN_LEER, 0)
template cudaError_t mh2d_launch_tape_lim<double, LIM_VAN_LEER>(const Mh2dArgs<double> &, int, cudaStream_t);

}  // namespace hydro
