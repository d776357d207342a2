/*
 * mh2d_fp32.cu -- FP32-state instantiations of the 2D step (the precision
 * form) and its helper kernels, plus the FP64 <-> FP32 conversions used on
 * upload and download.
 *
 * State, fluxes and limiters run in FP32 (FMA contraction allowed); FP64 is
 * kept for the dt reduction (the maxima are FP64 ordered-bit words and dt is
 * computed in FP64), for pressure recovery where kinetic energy exceeds half
 * of the total energy (cons_to_prim_2d_guarded) and for the compensated
 * conserved totals.
 */
#include "mh2d_lim.cuh"

namespace hydro {

HYDRO_MH2D_INSTANTIATE(float, LIM_MINMOD, 0)
HYDRO_MH2D_INSTANTIATE(float, LIM_MINMOD, 1)
HYDRO_MH2D_INSTANTIATE(float, LIM_VAN_LEER, 0)
HYDRO_MH2D_INSTANTIATE(float, LIM_MC, 0)
template int mh2d_resident_ctas<float>(int, int, int);
template cudaError_t mh2d_launch_batch_step<float>(const Mh2dBatchArgs<float> &, int, int, int, cudaStream_t);
template cudaError_t mh2d_launch_step<float>(const Mh2dArgs<float> &, int, cudaStream_t);
template cudaError_t mh2d_launch_prepare<float>(const Mh2dArgs<float> &, cudaStream_t);
template cudaError_t mh2d_launch_materialize<float>(const Mh2dArgs<float> &, int,
                                                    float *const[4], cudaStream_t);
template cudaError_t mh2d_launch_totals<float>(const Mh2dArgs<float> &, int, double *, cudaStream_t);

cudaError_t convert_f64_to_f32(const double *src, float *dst, long long n, cudaStream_t s)
{
    convert_kernel<double, float><<<1024, 256, 0, s>>>(src, dst, n);
    return cudaGetLastError();
}

cudaError_t convert_f32_to_f64(const float *src, double *dst, long long n, cudaStream_t s)
{
    convert_kernel<float, double><<<1024, 256, 0, s>>>(src, dst, n);
    return cudaGetLastError();
}

}  // namespace hydro
