/*
 * mh2d_lim_first_order.cu -- FP64 step kernels of the first-order Godunov
 * 2D integrator (face states = cell states; no limiter): single grid (with
 * and without gravity) and batched forms.
 *
 * Compiled with --fmad=false: the FP64 path must issue the same IEEE
 * operations as the reference CPU code, which never contracts a*b+c.
 */
#include "mh2d_lim.cuh"

namespace hydro {

HYDRO_MH2D_INSTANTIATE(double, LIM_MINMOD, 1)

}  // namespace hydro
