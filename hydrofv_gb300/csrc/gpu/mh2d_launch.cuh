/*
 * mh2d_launch.cuh -- launchers of the 2D step kernel and the helper kernels
 * around a run, templated on the state precision:
 *
 *   mh2d_prepare_kernel     sound speed of the caller's primitives and the
 *                           first step's CFL maxima (src/utils.c:55-95 on the
 *                           W arrays as handed to launch_simulation);
 *   mh2d_materialize_kernel full padded W (interior, ghost fill, corners) for
 *                           snapshots and for the arrays handed back to the
 *                           caller (src/system.c:763-802 then
 *                           src/boundary.c:513-777);
 *   totals_kernel           conserved totals over the interior, summed in FP64
 *                           with Neumaier compensation (drift diagnostics);
 *   convert_kernel          FP64 <-> FP32 copies for the FP32 state form.
 *
 * Included by mh2d.cu (FP64, --fmad=false), the per-limiter FP64 units
 * mh2d_lim_*.cu and mh2d_fp32.cu (FP32).
 */
#ifndef HYDRO_GPU_MH2D_LAUNCH_CUH
#define HYDRO_GPU_MH2D_LAUNCH_CUH

#include <cuda_runtime.h>

#include "gpu_internal.h"
#include "mh2d_kernel.cuh"

namespace hydro {

template <class R>
__global__ void mh2d_prepare_kernel(const Mh2dArgs<R> a)
{
    const int tx = a.nx + 2 * a.g, ty = a.ny + 2 * a.g;
    const long long total = (long long) tx * ty;
    double mx = -CUDART_INF, my = -CUDART_INF;
    R *const *W = a.W[0];
    for (long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x; k < total;
         k += (long long) gridDim.x * blockDim.x) {
        const int r = (int) (k / tx), c = (int) (k % tx);
        const long long idx = (long long) r * a.pitch + c;
        const R as = sound_speed(a.gas, W[0][idx], W[3][idx]);
        W[4][idx] = as;
        if (r >= a.g && r < a.g + a.ny && c >= a.g && c < a.g + a.nx) {
            const double sx = (double) (as + fabs(W[1][idx]));
            const double sy = (double) (as + fabs(W[2][idx]));
            if (sx > mx) mx = sx;
            if (sy > my) my = sy;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double ox = __shfl_xor_sync(0xffffffffu, mx, o);
        const double oy = __shfl_xor_sync(0xffffffffu, my, o);
        if (ox > mx) mx = ox;
        if (oy > my) my = oy;
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&a.ctrl->smax[0][0], ordered_bits(mx));
        atomicMax(&a.ctrl->smax[0][1], ordered_bits(my));
    }
}

template <class R>
__global__ void mh2d_materialize_kernel(const Mh2dArgs<R> a, int buf, R *out0, R *out1,
                                        R *out2, R *out3)
{
    const int tx = a.nx + 2 * a.g, ty = a.ny + 2 * a.g;
    const long long total = (long long) tx * ty;
    const R *const *U = a.U[buf];
    const R *const *W = a.W[buf];
    R *out[4] = { out0, out1, out2, out3 };
    for (long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x; k < total;
         k += (long long) gridDim.x * blockDim.x) {
        const int r = (int) (k / tx), c = (int) (k % tx);
        const long long idx = (long long) r * a.pitch + c;
        const bool in_x = c >= a.g && c < a.g + a.nx;
        const bool in_y = r >= a.g && r < a.g + a.ny;
        R w[5];
        const bool custom_band = (c < a.g && a.bc[0] == BC_CUSTOM) || (c >= a.g + a.nx && a.bc[1] == BC_CUSTOM) ||
                                 (r < a.g && a.bc[2] == BC_CUSTOM) || (r >= a.g + a.ny && a.bc[3] == BC_CUSTOM);
        if (!in_x && !in_y && custom_band) {
            /* a corner inside a custom side's band: what the host routine left there */
#pragma unroll
            for (int q = 0; q < 4; q++) w[q] = W[q][idx];
        } else if (!in_x && !in_y) {
            /* corners: converted, never overwritten by a built-in boundary routine */
            cons_to_prim_2d_guarded(a.gas, (R) a.vol, U[0][idx], U[1][idx], U[2][idx], U[3][idx], w);
        } else {
            fetch_w(a, W, U, false, r, c, w);
        }
#pragma unroll
        for (int q = 0; q < 4; q++) out[q][k] = w[q];
    }
}

/* W = U->W(U) over every padded cell (src/system.c:763-802, the reference's
 * all-cell conversion before its boundary routine): what a host boundary
 * callback sees. */
template <class R>
__global__ void mh2d_convert_all_kernel(const Mh2dArgs<R> a, int buf, R *out0, R *out1, R *out2, R *out3)
{
    const long long total = (long long) (a.nx + 2 * a.g) * (a.ny + 2 * a.g);
    const R *const *U = a.U[buf];
    for (long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x; k < total;
         k += (long long) gridDim.x * blockDim.x) {
        R w[4];
        cons_to_prim_2d_guarded(a.gas, (R) a.vol, U[0][k], U[1][k], U[2][k], U[3][k], w);
        out0[k] = w[0];
        out1[k] = w[1];
        out2[k] = w[2];
        out3[k] = w[3];
    }
}

/* Sound speed of the ghost cells of custom sides (mask bit s = side s:
 * x_min, x_max, y_min, y_max) after the host wrote their W. */
template <class R>
__global__ void mh2d_ghost_sound_speed_kernel(const Mh2dArgs<R> a, int buf, int mask)
{
    const int tx = a.nx + 2 * a.g, ty = a.ny + 2 * a.g;
    const long long total = (long long) tx * ty;
    R *const *W = a.W[buf];
    for (long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x; k < total;
         k += (long long) gridDim.x * blockDim.x) {
        const int r = (int) (k / tx), c = (int) (k % tx);
        const bool on = ((mask & 1) && c < a.g) || ((mask & 2) && c >= a.g + a.nx) ||
                        ((mask & 4) && r < a.g) || ((mask & 8) && r >= a.g + a.ny);
        if (on) W[4][k] = sound_speed(a.gas, W[0][k], W[3][k]);
    }
}

/* ------------------------------------------------------------- launchers */

/*
 * Per-limiter launchers.  Their definitions (mh2d_lim.cuh) are explicitly
 * instantiated in one translation unit per (precision, limiter) --
 * mh2d_lim_{minmod,vanleer,mc}.cu for FP64, mh2d_fp32.cu for FP32 -- so that
 * the step kernels of the three limiters compile in parallel.
 */
template <class R, int LIM, int FIRST_ORDER>
cudaError_t mh2d_launch_step_lim(const Mh2dArgs<R> &a, int grid, cudaStream_t s);
template <class R, int LIM>
cudaError_t mh2d_launch_tape_lim(const Mh2dArgs<R> &a, int grid, cudaStream_t s);
template <class R, int LIM, int FIRST_ORDER>
cudaError_t mh2d_launch_batch_lim(const Mh2dBatchArgs<R> &b, int grid, cudaStream_t s);
template <class R, int LIM, int FIRST_ORDER>
cudaError_t mh2d_step_occupancy(int *per_sm);

template <class R>
cudaError_t mh2d_launch_step(const Mh2dArgs<R> &a, int limiter, cudaStream_t s)
{
    const int n_items = mh2d_n_items(a);
    const int grid = (a.grid_ctas > 0 && a.grid_ctas < n_items) ? a.grid_ctas : n_items;
    if (a.first_order) return mh2d_launch_step_lim<R, LIM_MINMOD, 1>(a, grid, s);
    switch (limiter) {
    case LIM_MINMOD: return mh2d_launch_step_lim<R, LIM_MINMOD, 0>(a, grid, s);
    case LIM_VAN_LEER: return mh2d_launch_step_lim<R, LIM_VAN_LEER, 0>(a, grid, s);
    default: return mh2d_launch_step_lim<R, LIM_MC, 0>(a, grid, s);
    }
}

/* The step kernel that also writes the adjoint tape (a.tape, FP64 MUSCL-Hancock). */
template <class R>
cudaError_t mh2d_launch_step_tape(const Mh2dArgs<R> &a, int limiter, cudaStream_t s)
{
    const int n_items = mh2d_n_items(a);
    const int grid = (a.grid_ctas > 0 && a.grid_ctas < n_items) ? a.grid_ctas : n_items;
    switch (limiter) {
    case LIM_MINMOD: return mh2d_launch_tape_lim<R, LIM_MINMOD>(a, grid, s);
    case LIM_VAN_LEER: return mh2d_launch_tape_lim<R, LIM_VAN_LEER>(a, grid, s);
    default: return mh2d_launch_tape_lim<R, LIM_MC>(a, grid, s);
    }
}

template <class R>
cudaError_t mh2d_launch_prepare(const Mh2dArgs<R> &a, cudaStream_t s)
{
    mh2d_prepare_kernel<R><<<1024, 256, 0, s>>>(a);
    return cudaGetLastError();
}

template <class R>
cudaError_t mh2d_launch_convert_all(const Mh2dArgs<R> &a, int buf, R *const out[4], cudaStream_t s)
{
    mh2d_convert_all_kernel<R><<<1024, 256, 0, s>>>(a, buf, out[0], out[1], out[2], out[3]);
    return cudaGetLastError();
}

template <class R>
cudaError_t mh2d_launch_ghost_sound_speed(const Mh2dArgs<R> &a, int buf, int mask, cudaStream_t s)
{
    mh2d_ghost_sound_speed_kernel<R><<<1024, 256, 0, s>>>(a, buf, mask);
    return cudaGetLastError();
}

template <class R>
cudaError_t mh2d_launch_materialize(const Mh2dArgs<R> &a, int buf, R *const out[4], cudaStream_t s)
{
    mh2d_materialize_kernel<R><<<1024, 256, 0, s>>>(a, buf, out[0], out[1], out[2], out[3]);
    return cudaGetLastError();
}

template <class R>
cudaError_t mh2d_launch_batch_step(const Mh2dBatchArgs<R> &b, int limiter, int first_order, int grid,
                                   cudaStream_t s)
{
    if (first_order) return mh2d_launch_batch_lim<R, LIM_MINMOD, 1>(b, grid, s);
    switch (limiter) {
    case LIM_MINMOD: return mh2d_launch_batch_lim<R, LIM_MINMOD, 0>(b, grid, s);
    case LIM_VAN_LEER: return mh2d_launch_batch_lim<R, LIM_VAN_LEER, 0>(b, grid, s);
    default: return mh2d_launch_batch_lim<R, LIM_MC, 0>(b, grid, s);
    }
}

/* CTAs of the step kernel that fit on the device at once. */
template <class R>
int mh2d_resident_ctas(int limiter, int first_order, int device)
{
    int per_sm = 0, sms = 0;
    cudaError_t e;
    if (first_order) e = mh2d_step_occupancy<R, LIM_MINMOD, 1>(&per_sm);
    else if (limiter == LIM_MINMOD) e = mh2d_step_occupancy<R, LIM_MINMOD, 0>(&per_sm);
    else if (limiter == LIM_VAN_LEER) e = mh2d_step_occupancy<R, LIM_VAN_LEER, 0>(&per_sm);
    else e = mh2d_step_occupancy<R, LIM_MC, 0>(&per_sm);
    if (e != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return 0;
    return per_sm * sms;
}

/* Neumaier-compensated FP64 sums of the four conserved fields over the
 * interior; out[8] = (sum, compensation) per field, accumulated with
 * atomics per warp (the order of warps varies, the per-warp sums do not). */
__device__ __forceinline__ void neumaier_add(double &s, double &c, double x)
{
    const double t = s + x;
    if (fabs(s) >= fabs(x)) c += (s - t) + x;
    else c += (x - t) + s;
    s = t;
}

template <class R>
__global__ void totals_kernel(const Mh2dArgs<R> a, int buf, double *out)
{
    const int tx = a.nx + 2 * a.g;
    const long long n = (long long) a.nx * a.ny;
    double s[4] = { 0, 0, 0, 0 }, c[4] = { 0, 0, 0, 0 };
    for (long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x; k < n;
         k += (long long) gridDim.x * blockDim.x) {
        const int r = a.g + (int) (k / a.nx), col = a.g + (int) (k % a.nx);
        const long long idx = (long long) r * a.pitch + col;
        (void) tx;
#pragma unroll
        for (int q = 0; q < 4; q++) neumaier_add(s[q], c[q], (double) a.U[buf][q][idx]);
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
        double v = s[q] + c[q];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(&out[q], v);
    }
}

template <class R>
cudaError_t mh2d_launch_totals(const Mh2dArgs<R> &a, int buf, double *out4, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(out4, 0, 4 * sizeof(double), s);
    if (e != cudaSuccess) return e;
    totals_kernel<R><<<608, 256, 0, s>>>(a, buf, out4);
    return cudaGetLastError();
}

template <class S, class D>
__global__ void convert_kernel(const S *src, D *dst, long long n)
{
    for (long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x; k < n;
         k += (long long) gridDim.x * blockDim.x)
        dst[k] = (D) src[k];
}

}  // namespace hydro

#endif
