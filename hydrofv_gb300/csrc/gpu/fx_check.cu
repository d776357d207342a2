/*
 * fx_check.cu -- evaluation entry points used by the tests:
 *  - the integer-pipe FP64 division, square root and power (fp64_int.cuh,
 *    pow_int.cuh) over arrays: the host build (checked on the CPU against
 *    the host's IEEE operations and libm) and the device build next to the
 *    hardware operations on the GPU;
 *  - the device build of the exported pointwise numerics (HLLC fluxes,
 *    guess_p, the exact solver) over arrays of states, so that the kernels'
 *    arithmetic is checked against the reference's known answers branch by
 *    branch (vacuum generation, TRRS, TSRS, rarefaction and shock sampling),
 *    including branches that whole simulations rarely reach.
 */
#include <cuda_runtime.h>

#include "fp64_int.cuh"
#include "pow_int.cuh"
#include "numerics.cuh"
#include "quad_exact.cuh"
#include "hydro_gpu.h"

using namespace hydro;

namespace {

/* op 0: a / b, op 1: sqrt(a), op 2: pow(a, b).  fast = the integer form where it applies
 * (else the hardware result), hw = the hardware operation, ok = 1 where the
 * integer form applied.  op 3, 4, 5: the minmod, van Leer and MC slope
 * limiters L(a, b) as the kernels evaluate them (fast = hw; ok = 1 where the
 * sign test was decided on the bits). */
__global__ void fx_eval_kernel(int op, long long n, const double *a, const double *b,
                               double *fast, double *hw, unsigned char *ok)
{
    const long long stride = (long long) gridDim.x * blockDim.x;
    for (long long i = (long long) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        bool k;
        double f;
        if (op == 0) {
            f = fx::div_fast(a[i], b[i], k);
            hw[i] = fx::div_hw(a[i], b[i]);
            fast[i] = k ? f : dv(a[i], b[i]);
        } else if (op == 1) {
            f = fx::sqrt_fast(a[i], k);
            hw[i] = fx::sqrt_hw(a[i]);
            fast[i] = k ? f : sq(a[i]);
        } else if (op == 2) {
            f = fx::pow_fast(a[i], b[i], k);
            hw[i] = fx::pow_hw(a[i], b[i]);
            fast[i] = k ? f : pw(a[i], b[i]);
        } else {
            k = fx::product_nonpositive(fx::bits(a[i]), fx::bits(b[i])) >= 0;
            f = (op == 3) ? limit_slope<LIM_MINMOD>(a[i], b[i])
              : (op == 4) ? limit_slope<LIM_VAN_LEER>(a[i], b[i]) : limit_slope<LIM_MC>(a[i], b[i]);
            fast[i] = f;
            hw[i] = f;
        }
        ok[i] = k ? 1 : 0;
    }
}

/* The exported pointwise numerics, device build (one state pair per thread;
 * the gas constants are formed per element because gamma varies). */
__global__ void pointwise_kernel(int op, long long n, const double *gamma, double tol,
                                 const double *L, const double *R, const double *aux, double *out,
                                 int *rc)
{
    const long long stride = (long long) gridDim.x * blockDim.x;
    for (long long k = (long long) blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
        const GasConst<double> c = make_gas_const<double>(gamma[k], tol);
        const double *l = L + 4 * k, *r = R + 4 * k;
        int code = DEV_OK;
        if (op == 0) {
            double F[4];
            code = hllc_flux_2d(c, l[0], l[1], l[2], l[3], r[0], r[1], r[2], r[3], F);
            for (int q = 0; q < 4; q++) out[4 * k + q] = F[q];
        } else if (op == 1) {
            out[k] = guess_p(c, l[0], l[1], l[3], aux[2 * k], r[0], r[1], r[3], aux[2 * k + 1]);
        } else if (op == 2) {
            double F[3];
            code = exact_flux_1d(c, l[0], l[1], l[3], r[0], r[1], r[3], aux[k], F);
            for (int q = 0; q < 3; q++) out[3 * k + q] = F[q];
        } else if (op == 3) {
            double F[3];
            code = hllc_flux_1d(c, l[0], l[1], l[3], r[0], r[1], r[3], F);
            for (int q = 0; q < 3; q++) out[3 * k + q] = F[q];
        } else {
            double o[3];
            code = exact_solve_1d(c, l[0], l[1], l[3], r[0], r[1], r[3], aux[k], o);
            for (int q = 0; q < 3; q++) out[3 * k + q] = o[q];
        }
        rc[k] = code;
    }
}

/* The 1D kernel's four-lane exact solver: four consecutive threads per state
 * pair (op 5: the flux at x/t = aux[k], op 6: the sampled state). */
__global__ void pointwise_quad_kernel(int op, long long n, const double *gamma, double tol,
                                      const double *L, const double *R, const double *aux, double *out,
                                      int *rc)
{
    const Quad Q = make_quad();
    const long long quads = ((long long) gridDim.x * blockDim.x) >> 2;
    for (long long k = ((long long) blockIdx.x * blockDim.x + threadIdx.x) >> 2; k < n; k += quads) {
        const GasConst<double> c = make_gas_const<double>(gamma[k], tol);
        const double *l = L + 4 * k, *r = R + 4 * k;
        double o[3];
        int code;
        if (op == 5) {
            double s[3];
            code = quad_exact_solve(Q, c, l[0], l[1], l[3], r[0], r[1], r[3], aux[k], s);
            o[0] = s[0] * s[1];
            o[1] = s[0] * s[1] * s[1] + s[2];
            o[2] = (s[2] * c.g_gm1 + 0.5 * s[0] * s[1] * s[1]) * s[1];
        } else {
            code = quad_exact_solve(Q, c, l[0], l[1], l[3], r[0], r[1], r[3], aux[k], o);
        }
        if (Q.q == 0) {
            for (int q = 0; q < 3; q++) out[3 * k + q] = o[q];
            rc[k] = code;
        }
    }
}

}  // namespace

extern "C" {

void hydro_fx_eval_host(int op, long long n, const double *a, const double *b, double *out,
                        unsigned char *ok)
{
    for (long long i = 0; i < n; i++) {
        bool k = true;
        if (op <= 2) {
            out[i] = (op == 0) ? fx::div_fast(a[i], b[i], k)
                   : (op == 1) ? fx::sqrt_fast(a[i], k) : fx::pow_fast(a[i], b[i], k);
        } else if (op == 6) {
            /* the bit-level sign test itself: out = 1, 0 or -1 */
            out[i] = (double) fx::product_nonpositive(fx::bits(a[i]), fx::bits(b[i]));
        } else {
            /* host builds evaluate the limiters' FP64 expressions */
            out[i] = (op == 3) ? limit_slope<LIM_MINMOD>(a[i], b[i])
                   : (op == 4) ? limit_slope<LIM_VAN_LEER>(a[i], b[i]) : limit_slope<LIM_MC>(a[i], b[i]);
        }
        ok[i] = k ? 1 : 0;
    }
}

void hydro_fx_div_seeded_host(long long n, const double *a, const double *b, const float *seed_scale,
                              double *out, unsigned char *ok)
{
    for (long long i = 0; i < n; i++) {
        bool k;
        out[i] = fx::div_fast(a[i], b[i], k, seed_scale[i]);
        ok[i] = k ? 1 : 0;
    }
}

void hydro_fx_ratio_below_host(long long n, const double *x, const double *y, const double *tol,
                               unsigned char *out, unsigned char *decided)
{
    for (long long i = 0; i < n; i++) {
        bool d;
        out[i] = ratio_below_fast(x[i], y[i], tol[i], d) ? 1 : 0;
        decided[i] = d ? 1 : 0;
    }
}

void hydro_fx_quot_le_host(long long n, const double *x, const double *y, const double *z,
                           unsigned char *out, unsigned char *decided)
{
    for (long long i = 0; i < n; i++) {
        bool d;
        out[i] = quot_le_fast(x[i], y[i], z[i], d) ? 1 : 0;
        decided[i] = d ? 1 : 0;
    }
}

int hydro_gpu_fx_eval(int device, int op, long long n, const double *a, const double *b,
                      double *fast, double *hw, unsigned char *ok)
{
    if (n <= 0) return 0;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return (int) e;
    const size_t nb = (size_t) n * sizeof(double);
    char *slab = nullptr;
    e = cudaMalloc(&slab, 4 * nb + (size_t) n);
    if (e != cudaSuccess) return (int) e;
    double *da = (double *) slab, *db = da + n, *df = db + n, *dh = df + n;
    unsigned char *dk = (unsigned char *) (dh + n);
    e = cudaMemcpy(da, a, nb, cudaMemcpyHostToDevice);
    if (op < 0 || op > 5) e = cudaErrorInvalidValue;
    if (e == cudaSuccess) e = cudaMemcpy(db, op == 1 ? a : b, nb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        fx_eval_kernel<<<4 * 152, 256>>>(op, n, da, db, df, dh, dk);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(fast, df, nb, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(hw, dh, nb, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(ok, dk, (size_t) n, cudaMemcpyDeviceToHost);
    cudaFree(slab);
    return (int) e;
}

int hydro_gpu_pointwise_eval(int device, int op, long long n, const double *gamma, double tol,
                             const double *L, const double *R, const double *aux, double *out,
                             int *rc)
{
    if (n <= 0) return 0;
    if (op < 0 || op > 6) return (int) cudaErrorInvalidValue;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return (int) e;
    const int width = (op == 0) ? 4 : (op == 1) ? 1 : 3;
    const int naux = (op == 1) ? 2 : (op == 2 || op >= 4) ? 1 : 0;
    const size_t nb = (size_t) n * sizeof(double);
    char *slab = nullptr;
    e = cudaMalloc(&slab, (9 + naux + width) * nb + (size_t) n * sizeof(int));
    if (e != cudaSuccess) return (int) e;
    double *dg = (double *) slab, *dl = dg + n, *dr = dl + 4 * n, *da = dr + 4 * n;
    double *dout = da + naux * n;
    int *drc = (int *) (dout + width * n);
    e = cudaMemcpy(dg, gamma, nb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dl, L, 4 * nb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dr, R, 4 * nb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && naux) e = cudaMemcpy(da, aux, naux * nb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        if (op >= 5) pointwise_quad_kernel<<<152, 128>>>(op, n, dg, tol, dl, dr, da, dout, drc);
        else pointwise_kernel<<<152, 128>>>(op, n, dg, tol, dl, dr, da, dout, drc);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, width * nb, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(rc, drc, (size_t) n * sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(slab);
    return (int) e;
}

}  // extern "C"
